"""Camera-format ingest's oracle (oracle/oracle_ingest.c) held to the reference: its develop.cpp compiled here
(oracle/ref_develop.cpp) on random planes of every camera format, bin, crop and level set, the gamma table, and its
ob_luma (oracle/_ref/libref.so) for RGBA."""
import ctypes

import numpy as np
import pytest

import oracle

FORMATS = {0x20: "RAW16", 0x25: "RAW10", 0x26: "RAW12", 0x36: "P010"}


def row_bytes(fmt, w, ps):
    return {0x20: w * ps, 0x25: (w + 3) // 4 * 5, 0x26: (w + 1) // 2 * 3, 0x36: w * ps}[fmt]


def random_case(fmt, seed):
    """A plane of random samples at realistic levels, a crop inside it, the develop's arguments."""
    rng = np.random.default_rng(seed)
    bin_ = 1 if fmt == 0x36 else int(rng.integers(1, 3))
    ps = int(rng.choice([2, 4])) if fmt in (0x20, 0x36) else 0
    W, H = int(rng.integers(40, 300)), int(rng.integers(20, 120))
    rs = row_bytes(fmt, W, ps) + int(rng.integers(0, 24))
    plane = rng.integers(0, 256, H * rs, dtype=np.uint8)
    white = {0x20: 4095, 0x25: 1023, 0x26: 4095, 0x36: 1023}[fmt]
    levels = np.array(list(rng.uniform(0, white * 0.08, 4)) + [white] + list(rng.uniform(0.8, 2.4, 4)), np.float32)
    x0, y0 = 2 * int(rng.integers(0, 4)), 2 * int(rng.integers(0, 3))
    wmax, hmax = (W - x0) // bin_, (H - y0) // bin_
    ox, oy = int(rng.integers(0, 3)), int(rng.integers(0, 3))
    w, h = wmax - ox - int(rng.integers(0, 3)), hmax - oy - int(rng.integers(0, 3))
    return dict(fmt=fmt, plane=plane, row_stride=rs, pixel_stride=ps, x0=x0, y0=y0, bin_=bin_, levels=levels, ox=ox, oy=oy, w=w, h=h)


def run(lib, fn, c):
    return oracle.develop(lib, fn, c["fmt"], c["plane"], c["row_stride"], c["pixel_stride"], c["x0"], c["y0"], c["bin_"], c["levels"],
                          c["ox"], c["oy"], c["w"], c["h"])


@pytest.mark.skipif(oracle.ref_develop() is None, reason="the reference's develop is not here")
def test_gamma_table_matches_reference():
    a, b = np.zeros(4097, np.uint8), np.zeros(4097, np.uint8)
    oracle.port().orc_gamma_lut(oracle._p(a))
    oracle.ref_develop().refd_gamma_lut(oracle._p(b))
    assert np.array_equal(a, b)


@pytest.mark.skipif(oracle.ref_develop() is None, reason="the reference's develop is not here")
@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_develop_matches_reference(fmt):
    for seed in range(12):
        c = random_case(fmt, 100 * fmt + seed)
        assert np.array_equal(run(oracle.port(), "orc_develop", c), run(oracle.ref_develop(), "refd_develop", c)), (FORMATS[fmt], seed)


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not here")
def test_rgba_luma_matches_reference():
    L = oracle.ref()
    L.ob_luma.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(5)
    w, h = 333, 7
    px = rng.integers(0, 256, (h, 4 * w + 12), dtype=np.uint8)
    out = np.zeros((h, w), np.uint8)
    assert oracle.port().orc_ingest_pixels(oracle._p(px), w, h, 4 * w + 12, 3, oracle._p(out)) == 0
    for y in range(h):
        row = np.ascontiguousarray(px[y])
        ref = np.zeros(w, np.uint8)
        L.ob_luma(oracle._p(row), w, oracle._p(ref))
        assert np.array_equal(out[y], ref)
