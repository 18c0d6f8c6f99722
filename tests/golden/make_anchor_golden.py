"""Makes tests/golden/anchor_ref.npz: the reference's own anchor search (its portable build, oracle/_ref/
libref_scalar.so, compiled from the reference's sources by `make -C oracle ref`) on seeded captures, for the GPU tests
on machines where the reference tree is absent.

Cases: LIZARD-64 pictures (n = 384) in the 64 ring (span 128) and the 128 ring (span 256), warped captures with the
map H put a fraction of a module off, with and without a lens model, one with anchors marked as found before. Each
frame keeps only the pixels about the anchors' windows (the rest set to 0), which is all the search reads, so the
fixture stays small; the outputs are the reference's on the stored frame.

    python tests/golden/make_anchor_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import lizard_gb300 as lz  # noqa: E402
import oracle  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402


def windows_mask(span, shape, H, lens):
    """Pixels within 3 of any anchor window's corners' hull (through H and the lens model): what the search reads."""
    h, w = shape
    a = span // 64
    hs = a / 16.0
    r = int(np.ceil(3 / hs))
    mask = np.zeros(shape, bool)
    Hm = np.asarray(H, np.float64).reshape(3, 3)
    for j in range(7):
        for i in range(7):
            m0x = int(np.floor(15 + span * (i + 0.5) / 7 - a / 2.0 + 0.5))
            m0y = int(np.floor(15 + span * (j + 0.5) / 7 - a / 2.0 + 0.5))
            xs = [m0x + (-r) * hs, m0x + (16 + r) * hs]
            ys = [m0y + (-r) * hs, m0y + (16 + r) * hs]
            pts = []
            for X in xs:
                for Y in ys:
                    q = Hm @ np.array([X, Y, 1.0])
                    u, v = q[0] / q[2], q[1] / q[2]
                    if lens is not None:
                        u, v = u + 8, v + 8   # the lens model moves points by a few pixels at most here: widen
                        pts.append((u - 16, v - 16))
                    pts.append((u, v))
            us, vs = [p[0] for p in pts], [p[1] for p in pts]
            x0, x1 = max(0, int(min(us)) - 3), min(w, int(max(us)) + 4)
            y0, y1 = max(0, int(min(vs)) - 3), min(h, int(max(vs)) + 4)
            mask[y0:y1, x0:x1] = True
    return mask


def case(span, W, Hh, seed, with_lens, skip):
    fmt = lz.Format(384, 64, span)
    rng = np.random.default_rng(seed)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed), parity=seed & 3)
    Hw = synth.warp(fmt, W, Hh, rng, rot_deg=8, scale=(0.95, 1.0))
    luma, reg = synth.capture(fmt, grey, W, Hh, H=Hw, sigma=2.0, rng=rng)
    H = reg[:9].astype(np.float32).copy()
    pxm = 384 / span
    H[2] += np.float32(rng.uniform(-0.8, 0.8) * pxm)
    H[5] += np.float32(rng.uniform(-0.8, 0.8) * pxm)
    lens = None
    if with_lens:
        lens = np.zeros(15, np.float64)
        lens[:4] = [2, W / 2, Hh / 2, np.hypot(W, Hh) / 2]
        lens[4:4 + 10] = rng.uniform(-0.4, 0.4, 10)
        lens[12:14] = rng.uniform(-0.05, 0.05, 2)
    luma = np.where(windows_mask(span, luma.shape, H, lens), luma, 0).astype(np.uint8)
    sk = np.zeros(49, np.uint8)
    if skip:
        sk[rng.choice(49, 10, replace=False)] = 1
    out = oracle.anchor_find(oracle.ref_scalar(), "refs_anchor_find", span, luma, H, lens, sk)
    return luma, H, lens, sk, out


def main():
    assert oracle.ref_scalar() is not None, "needs oracle/_ref/libref_scalar.so (make -C oracle ref)"
    cases = [(128, 520, 520, 11, False, False), (128, 520, 520, 12, True, True), (256, 470, 470, 13, False, False), (256, 470, 470, 14, True, False)]
    d = {}
    for c, (span, W, Hh, seed, with_lens, skip) in enumerate(cases):
        luma, H, lens, sk, out = case(span, W, Hh, seed, with_lens, skip)
        d["c%d_span" % c] = np.int32(span)
        d["c%d_luma" % c] = luma
        d["c%d_H" % c] = H
        d["c%d_lens" % c] = lens if lens is not None else np.zeros(0)
        d["c%d_skip" % c] = sk
        for k in ("ok", "peak", "dx", "dy", "u", "v"):
            d["c%d_%s" % (c, k)] = out[k]
        print("case", c, "span", span, "lens", with_lens, "skip", int(sk.sum()), "found", out["found"])
    d["cases"] = np.int32(len(cases))
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "anchor_ref.npz"), **d)


if __name__ == "__main__":
    main()
