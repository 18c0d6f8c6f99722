"""Generates tests/golden/rx_ref.npz: the reference receiver's own outputs (compiled from its sources by
oracle/Makefile) on small synthetic pictures, so the GPU receiver can be held to the reference on a GPU host where
the reference tree is absent.

Run from the repo root where the reference is present: python tests/golden/make_rx_golden.py
Cases: LIZARD-64 at n = 384 clean (the grid axis-aligned), and LIZARD-80 at n = 384 with the picture moved by
(0.3, -0.25) samples, which the reference's pilot fit finds and turns back. Pictures from lizard_gb300.synth, AWGN
sigma = 3 grey levels; the grid is stored as its 8-bit grey levels. For each: the reference's FP32 spectrum at the
used coefficients (lizard_debug), soft values, sub-channel estimates and rms, the pilots' shift, and per block its
iterations, estimate, pilot reading and CRC verdict.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
import lizard_gb300 as lz  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402


def main():
    oracle.build(ref=True)
    out = {}
    for tag, (n, subch, shift, seed) in {"a": (384, 64, None, 11), "b": (384, 80, (0.3, -0.25), 12)}.items():
        f = lz.Format(n, subch, 128)
        r = oracle.RefFmt(n, subch, 128)
        g, blocks = synth.grids(f, 1, seed=seed, sigma=3.0, shift=shift)
        grey = np.rint(g[0] * 255.0).astype(np.uint8)
        assert np.array_equal(grey.astype(np.float32) / np.float32(255.0), g[0])
        R = r.finish_grid(g[0])
        out[tag + "_fmt"] = np.array([n, subch, 128], np.int32)
        out[tag + "_grey"] = grey
        for k in ("coef", "llrf", "sub_est", "sub_rms", "align", "its", "est", "pilot", "ok"):
            out[tag + "_" + k] = R[k]
        out[tag + "_blocks"] = np.stack(blocks[0]) if isinstance(blocks[0], list) else blocks[0]
        print(tag, n, subch, "verified", int(R["ok"].sum()), "of", r.blocks, "align", R["align"])
    path = os.path.join(ROOT, "tests", "golden", "rx_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
