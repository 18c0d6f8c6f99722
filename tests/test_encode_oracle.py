"""The sender's oracle (lizard_gb300.synth.encode_drive, a numpy restatement of lizard_encode and lizard_paint_grey)
and the library's border painter (lizg_layout_kind) held to the reference's own encoder, compiled here
(oracle/_ref/libref.so ref_encode, refh_layout_kind). Where the reference tree is absent, the committed crops of the
reference's pages (tests/golden/encode_ref.npz) hold the oracle instead."""
import ctypes
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "encode_ref.npz")
# (n, subch, span): the 64 ring at exact copy, the 128 ring resampled (1.5 samples a module onto 2 pixels), n = 768 in
# the 128 ring, LIZARD-1024 in the 128 ring (exact copy at 6 pixels a module)
FORMATS = ((384, 64, 128), (384, 64, 256), (768, 320, 256), (1536, 1024, 256))
DRIVE_TOL = 1e-6        # the transform's floats: a double's and a float's inverse
GREY_FRACTION = 1e-4    # grey levels one apart at a rounding tie, as a fraction of the page


def _ref():
    r = oracle.ref()
    if r is None:
        pytest.skip("the reference tree is not here")
    r.ref_fmt_new.restype = ctypes.c_void_p
    r.ref_fmt_new.argtypes = [ctypes.c_int] * 3
    r.ref_fmt_free.argtypes = [ctypes.c_void_p]
    r.ref_encode.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    r.refh_layout_kind.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return r


def ref_page(R, n, subch, span, blocks, pilots, fps=0):
    f = R.ref_fmt_new(n, subch, span)
    if fps:
        R.lizard_fmt_fps.argtypes = [ctypes.c_void_p, ctypes.c_int]
        R.lizard_fmt_fps(f, fps)
    pxm = synth.pxm_for(n, span)
    px = (span + 30) * pxm
    W = px + 4 * pxm
    drive, grey = np.zeros(px * px, np.float32), np.zeros(W * W, np.uint8)
    assert R.ref_encode(f, oracle._p(np.ascontiguousarray(blocks, np.uint8)), pilots, oracle._p(drive), oracle._p(grey)) == W
    R.ref_fmt_free(f)
    return drive.reshape(px, px), grey.reshape(W, W)


@pytest.mark.parametrize("n,subch,span", FORMATS)
def test_oracle_matches_reference(n, subch, span):
    R = _ref()
    fmt = lz.Format(n, subch, span)
    for seed, pilots in ((1, 0), (2, 3)):
        blocks = synth.random_blocks(fmt.blocks, seed)
        d_ref, g_ref = ref_page(R, n, subch, span, blocks, pilots)
        d, g = synth.encode_drive(fmt, blocks, parity=pilots)
        assert np.abs(d - d_ref).max() <= DRIVE_TOL
        diff = g.astype(int) - g_ref.astype(int)
        assert np.abs(diff).max() <= 1 and np.count_nonzero(diff) <= GREY_FRACTION * diff.size


def test_layout_kind_matches_reference():
    """The library's border painter (host C++) against the reference's layout, the format word painted, every ring."""
    R = _ref()
    for n, subch, span in ((384, 64, 128), (768, 320, 256), (1536, 1024, 512)):
        f = R.ref_fmt_new(n, subch, span)
        side = span + 30
        kind = np.zeros(side * side, np.uint8)
        R.refh_layout_kind(f, 42, oracle._p(kind))
        R.ref_fmt_free(f)
        mine = lz.layout_kind(span, subch // 16, 42)
        assert np.array_equal(mine, kind.reshape(side, side)), span


def test_layout_kind_matches_painter():
    """Without the reference: the library's painter against the test painter (itself held to the reference above)."""
    for span in (128, 256, 512):
        for version, fps in ((4, 0), (64, 255), (20, 60)):
            want = synth.border_kind(span, synth.fmt_word(version, fps, span))
            assert np.array_equal(lz.layout_kind(span, version, fps), want), (span, version, fps)
    # a version no format has: the word's cells light
    assert np.array_equal(lz.layout_kind(128, 2, 0), synth.border_kind(128, None))


def golden_crops(grey, pxm):
    """The reference page's parts a test can hold the oracle to: its top-left corner (the margin, a corner mark, the
    line, the track, the word, the guard, the picture's first rows) and a square about the middle anchor."""
    W = grey.shape[0]
    c = min(W, 40 * pxm)
    m = W // 2
    return grey[:c, :c].copy(), grey[m - 12 * pxm:m + 12 * pxm, m - 12 * pxm:m + 12 * pxm].copy()


def test_oracle_golden():
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        n, subch, span, seed, pilots = (int(v) for v in g["case"][c])
        fmt = lz.Format(n, subch, span)
        _, grey = synth.encode_drive(fmt, synth.random_blocks(fmt.blocks, seed), parity=pilots)
        for k, crop in enumerate(golden_crops(grey, synth.pxm_for(n, span))):
            diff = crop.astype(int) - g["crop_%d_%d" % (c, k)].astype(int)
            assert np.abs(diff).max() <= 1 and np.count_nonzero(diff) <= max(2, GREY_FRACTION * diff.size), (c, k)
