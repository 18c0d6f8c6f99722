"""Row b on the GPU (anchor erase, detrend, 2D mixed-radix FFT) through the C ABI, then rows c-e: the spectrum held
to the FP64 oracle and to the reference's FP32 one within 1e-4 of the spectrum's rms, the error stated per picture
size; the soft values bit for bit from the GPU's own spectrum; the CRC-passing block set identical."""
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-4   # |T_gpu - T| / rms(T), max over the used coefficients


def spec_err(c32, ref):
    c = c32[0::2] + 1j * c32[1::2]
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    e = np.abs(c - ref)
    return e.max() / rms, np.sqrt(np.mean(e ** 2)) / rms


@pytest.mark.parametrize("tag", ["a", "b"])
def test_grid_spectrum_matches_reference_golden(tag):
    g = np.load(os.path.join(GOLD, "rx_ref.npz"))
    n, subch, span = (int(x) for x in g[tag + "_fmt"])
    rx = lz.Receiver(n, subch, span, max_frames=1)
    grid = g[tag + "_grey"].astype(np.float32) / np.float32(255.0)
    out = rx.finish_grid(grid[None])
    rc = g[tag + "_coef"]
    mx, rms = spec_err(out["coef"][0], rc[0::2] + 1j * rc[1::2])
    print("n=%d vs reference FP32: max %.2e rms %.2e" % (n, mx, rms))
    assert mx < TOL
    assert np.array_equal(out["ok"][0], g[tag + "_ok"])
    assert np.array_equal(out["blocks"][0][out["ok"][0].astype(bool)], g[tag + "_blocks"][g[tag + "_ok"].astype(bool)])


@pytest.mark.parametrize("n,subch,frames,shift", [(384, 64, 2, None), (512, 256, 1, (0.2, 0.1)), (768, 320, 2, None),
                                                  (1024, 1024, 1, None), (1152, 720, 1, (0.1, -0.3)), (1280, 880, 1, None),
                                                  (1536, 1024, 2, (0.3, -0.25))])
def test_grid_path_matches_oracle(n, subch, frames, shift):
    fmt = lz.Format(n, subch, 128)
    o = oracle.Fmt(n, subch, 128)
    grids, blocks = synth.grids(fmt, frames, seed=7 * n + frames, sigma=3.0, shift=shift)
    rx = lz.Receiver(n, subch, 128, max_frames=frames)
    out = rx.finish_grid(grids)
    for f in range(frames):
        spec, _, _ = o.spectrum(grids[f])
        mx, rms = spec_err(out["coef"][f], spec)
        print("n=%d frame %d vs FP64: max %.2e rms %.2e" % (n, f, mx, rms))
        assert mx < TOL
        # rows c-e from the GPU's own spectrum: the oracle's soft values and blocks bit for bit
        c = out["coef"][f]
        d, used = o.pilot_align(c)
        turn = d if (used and (d[0] != 0 or d[1] != 0)) else None
        llrf, est, rms_ = o.demap(c, turn)
        assert np.array_equal(out["llrf"][f], llrf)
        B = o.blocks_stage(llrf, est, rms_, c, turn)
        assert np.array_equal(out["its"][f], B["its"].astype(np.int32))
        assert np.array_equal(out["ok"][f], B["ok"])
        # against the FP64 path end to end: the same CRC-passing set, the sent blocks
        ref = o.receive(grids[f])
        assert np.array_equal(out["ok"][f], ref["ok"])
        okb = out["ok"][f].astype(bool)
        assert okb.all()
        assert np.array_equal(out["blocks"][f], blocks[f])
