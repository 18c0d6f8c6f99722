"""Measures, with the reference's own receiver (compiled from its sources, oracle/_ref, the x86-64 build), how much
registration can matter on the distorted full receiver's hardest point: LIZARD-1024 (n = 1536) in the 128 ring,
painted by the reference's sender, seen in 1920 x 1080 frames through the configuration's views (rotation U(+-15
deg), tilt U(+-20 deg), the layout's side 1000 px x U(0.8, 1.1)), radial k1 = 0.03, blur 1.5 px in linear light, AWGN 3.
Per frame, the blocks the reference's finish verifies with (a) the reference's own whole registration (lizard_acquire),
(b) the camera's true map at every node of the mesh (the best any registration can do), (c) a finder's corners'
homography alone. TEST AND MEASUREMENT INFRASTRUCTURE ONLY.

Run from the repo root where the reference is present: python oracle/registration_bound.py  (writes
oracle/registration_bound.json)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import oracle  # noqa: E402
from lizard_gb300_testing import render  # noqa: E402
import make_e2e_golden as mg  # noqa: E402

FRAMES, K1, BLUR = 32, 0.03, 1.5


def main():
    oracle.build(ref=True)
    rows = []
    for k in range(FRAMES):
        seed = 9100 + k
        r = oracle.RefFmt(1536, 1024, 256)
        _, grey = r.encode(oracle.spec_blocks(r.blocks, seed=seed), 0)
        view = render.views(1536, 256, 1920, 1080, [seed], 1000.0)[0]
        luma = mg.render(grey, r.pxm, 256, 1920, 1080, view, K1, BLUR, 3.0, np.random.default_rng(seed))
        d = r.decode_frame(luma)
        true = render.registration(256, view, K1, 1920, 1080, true_mesh=True)
        corners = render.registration(256, view, K1, 1920, 1080)
        ft = r.finish_grid(r.sample_decode(luma, true[:9], true[9:])[0])
        fc = r.finish_grid(r.sample_decode(luma, corners[:9], corners[9:])[0])
        rows.append({"seed": seed, "reference_registration": int(d["ok"].sum()) if d["good"] >= 0 else 0,
                     "true_map": int(ft["ok"].sum()), "corners_homography": int(fc["ok"].sum())})
        print(rows[-1], flush=True)
    tot = {k: sum(r[k] for r in rows) for k in ("reference_registration", "true_map", "corners_homography")}
    blocks = 124 * FRAMES
    res = {"workload": "%d frames: LIZARD-1024 in the 128 ring (reference sender), 1920x1080, views as the distorted configuration's "
                       "(seeds 9100-%d), k1 %.2f, blur %.1f px in linear light, AWGN 3" % (FRAMES, 9100 + FRAMES - 1, K1, BLUR),
           "blocks": blocks, "verified": tot, "pass_rate": {k: round(v / blocks, 4) for k, v in tot.items()},
           "frames": rows}
    with open(os.path.join(HERE, "registration_bound.json"), "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: res[k] for k in ("blocks", "verified", "pass_rate")}))


if __name__ == "__main__":
    main()
