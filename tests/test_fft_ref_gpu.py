"""The GPU's transform held to the reference's own FP32 one at every size of the FFT demod batch (n = 384, 768, 1152,
1536 at their top versions, tests/golden/make_fft_golden.py) and to the FP64 oracle on the same grids: within 1e-4 of
the spectrum's rms (max over the coefficients), the error stated per n; the reference's CRC-passing blocks verified."""
import hashlib
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fft_ref.npz")
SIZES = [384, 768, 1152, 1536]
TOL = 1e-4


def grid(n):
    z = np.load(GOLD)
    n_, subch, span = (int(v) for v in z["n%d_fmt" % n])
    f = lz.Format(n_, subch, span)
    g, _ = synth.grids(f, 1, seed=31 * n, sigma=3.0, shift=(0.15, -0.1))
    grey = np.rint(g[0] * 255.0).astype(np.uint8)
    assert hashlib.sha256(grey.tobytes()).digest() == z["n%d_sha256" % n].tobytes(), "the grid made here is not the fixture's"
    return z, f, g


def errors(c, ref):
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    e = np.abs(c - ref)
    return e.max() / rms, np.sqrt(np.mean(e ** 2)) / rms


@pytest.mark.parametrize("n", SIZES)
def test_grids_are_the_fixtures(n):
    grid(n)


@pytest.mark.gpu
@pytest.mark.parametrize("n", SIZES)
def test_gpu_spectrum_against_reference_fp32_and_fp64(n):
    z, f, g = grid(n)
    rx = lz.Receiver(f.n, f.subch, f.span, max_frames=1)
    out = rx.finish_grid(g)
    c = out["coef"][0][0::2] + 1j * out["coef"][0][1::2]
    r = z["n%d_ref" % n]
    ref = r[:, 0].astype(np.float64) + 1j * r[:, 1]
    fp64, _, _ = oracle.Fmt(f.n, f.subch, f.span).spectrum(g[0])
    idx = np.arange(0, c.size, 8)
    mr, rr = errors(c[idx], ref)
    m6, r6 = errors(c, fp64)
    mref, _ = errors(ref, fp64[idx])
    print("n=%d: GPU vs reference FP32 max %.2e rms %.2e; GPU vs FP64 max %.2e rms %.2e; reference vs FP64 max %.2e" % (n, mr, rr, m6, r6, mref))
    assert mr < TOL and m6 < TOL
    assert np.array_equal(out["ok"][0], z["n%d_ok" % n])
