"""Generates tests/golden/fft_ref.npz: the reference's own FP32 transform (lizard_finish on a supplied grid, compiled
from its sources by oracle/Makefile, x86-64 build) on config-3-style pictures at every size the FFT demod batch takes:
n = 384, 768, 1152, 1536 at their top versions in the 64 ring (LIZARD-80, 320, 720, 1024), so the GPU's spectrum is held
to the reference's FP32 one (not only to the FP64 oracle) at each size, on a GPU host where the reference is absent.

Run from the repo root where the reference is present: python tests/golden/make_fft_golden.py
Per size: the picture grid's SHA-256 (the grid itself is made again where the test runs, by synth.grids: seeded
blocks painted, AWGN 3 grey levels, as 8-bit greys; the digest proves it is the same grid), the reference's detrended
FP32 spectrum at every eighth used coefficient (pos order), the reference's verified blocks and iterations.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
import lizard_gb300 as lz  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402

SIZES = [(384, 80), (768, 320), (1152, 720), (1536, 1024)]


def main():
    oracle.build(ref=True)
    out = {}
    for n, subch in SIZES:
        f = lz.Format(n, subch, 128)
        r = oracle.RefFmt(n, subch, 128)
        o = oracle.Fmt(n, subch, 128)
        g, _ = synth.grids(f, 1, seed=31 * n, sigma=3.0, shift=(0.15, -0.1))
        grey = np.rint(g[0] * 255.0).astype(np.uint8)
        assert np.array_equal(grey.astype(np.float32) / np.float32(255.0), g[0])
        R = r.finish_grid(g[0])
        ref = R["coef"][0::2].astype(np.float64) + 1j * R["coef"][1::2]
        fp64, _, _ = o.spectrum(g[0])
        idx = np.arange(0, ref.size, 8)
        t = "n%d" % n
        out[t + "_fmt"] = np.array([n, subch, 128], np.int32)
        out[t + "_sha256"] = np.frombuffer(hashlib.sha256(grey.tobytes()).digest(), np.uint8)
        out[t + "_ref"] = np.stack([ref.real[idx], ref.imag[idx]], 1).astype(np.float32)
        out[t + "_ok"] = R["ok"]
        out[t + "_its"] = R["its"]
        rms = np.sqrt(np.mean(np.abs(fp64) ** 2))
        e = np.abs(ref - fp64)
        print(n, subch, "reference FP32 vs FP64: max %.2e rms %.2e" % (e.max() / rms, np.sqrt(np.mean(e ** 2)) / rms),
              "verified", int(R["ok"].sum()), "of", r.blocks)
    path = os.path.join(ROOT, "tests", "golden", "fft_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
