"""Camera-format ingest on the GPU (lizg_ingest_pixels_dev, lizg_develop_dev), byte for byte the oracle's
restatement of the reference: every pixel format with padded rows, every camera format, bin and crop, batches of
frames; crops that would read past the plane refused."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from test_ingest_oracle import FORMATS, random_case, run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [1, 2, 3, 4])
def test_pixels_match_oracle(fmt):
    rng = np.random.default_rng(fmt)
    bpp = 1 if fmt == 1 else 4
    for w, h, pad in ((333, 41, 12), (64, 64, 0), (1, 1, 3), (1919, 17, 4)):
        stride = w * bpp + pad
        frames = rng.integers(0, 256, (3, h, stride), dtype=np.uint8)
        got = lz.ingest_pixels(frames, fmt, w=w)
        for f in range(3):
            want = np.zeros((h, w), np.uint8)
            assert oracle.port().orc_ingest_pixels(oracle._p(np.ascontiguousarray(frames[f])), w, h, stride, fmt, oracle._p(want)) == 0
            assert np.array_equal(got[f], want), (fmt, w, h)


@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_develop_matches_oracle(fmt):
    for seed in range(10):
        c = random_case(fmt, 1000 * fmt + seed)
        planes = np.stack([c["plane"], np.roll(c["plane"], 7)])
        got = lz.develop(c["fmt"], planes, c["row_stride"], c["pixel_stride"], c["x0"], c["y0"], c["bin_"], c["levels"], c["ox"], c["oy"], c["w"], c["h"])
        for f in range(2):
            c2 = dict(c, plane=planes[f])
            assert np.array_equal(got[f], run(oracle.port(), "orc_develop", c2)), (FORMATS[fmt], seed, f)


def test_develop_refuses_reads_past_the_plane():
    c = random_case(0x25, 7)
    with pytest.raises(lz.LizgError):
        lz.develop(c["fmt"], c["plane"], c["row_stride"], 0, c["x0"], c["y0"], c["bin_"], c["levels"], c["ox"], c["oy"], c["w"] + 64, c["h"])
    with pytest.raises(lz.LizgError):
        lz.develop(0x99, c["plane"], c["row_stride"], 0, 0, 0, 1, c["levels"], 0, 0, 4, 4)


@pytest.mark.parametrize("fmt", [0x25, 0x26])
def test_develop_group_aligned_crops(fmt):
    """Crops whose quads start on a RAW10 / RAW12 packing group (the grouped path) and ones that do not."""
    from test_ingest_oracle import row_bytes
    rng = np.random.default_rng(fmt)
    W, H = 260, 40
    rs = row_bytes(fmt, W, 0) + 8
    plane = rng.integers(0, 256, H * rs, dtype=np.uint8)
    lv = np.array([60, 61, 59, 62, 1023, 1.8, 1.0, 1.1, 1.5], np.float32)
    for bin_, x0, ox, w in ((1, 0, 0, 256), (1, 0, 4, 250), (1, 2, 1, 200), (2, 0, 0, 128), (2, 0, 2, 121), (2, 2, 1, 100)):
        h = (H // bin_) - 2
        got = lz.develop(fmt, plane, rs, 0, x0, 0, bin_, lv, ox, 1, w, h)
        want = oracle.develop(oracle.port(), "orc_develop", fmt, plane, rs, 0, x0, 0, bin_, lv, ox, 1, w, h)
        assert np.array_equal(got[0], want), (bin_, x0, ox, w)


@pytest.mark.parametrize("fmt,ps", [(0x25, 0), (0x26, 0), (0x20, 2), (0x20, 6)])
def test_develop_wide_tiles(fmt, ps):
    """Crops several tiles wide with a ragged last tile, rows whose 16-byte phase changes from row to row, output rows
    that are and are not a multiple of 16 bytes, three frames a call (each persistent CTA takes tiles in turn)."""
    from test_ingest_oracle import row_bytes
    rng = np.random.default_rng(fmt + ps)
    W, H = 5200, 36
    rs = row_bytes(fmt, W, ps) + 7
    plane = rng.integers(0, 256, H * rs, dtype=np.uint8)
    planes = np.stack([np.roll(plane, 13 * i) for i in range(3)])
    white = 1023 if fmt == 0x25 else 4095
    lv = np.array([60, 61, 59, 62, white, 1.8, 1.0, 1.1, 1.5], np.float32)
    for bin_, x0, ox, w in ((1, 0, 0, 2560), (1, 0, 8, 2501), (1, 1, 3, 2047), (2, 0, 0, 2560), (2, 0, 4, 2301), (2, 2, 1, 1999)):
        h = H // bin_ - 1
        got = lz.develop(fmt, planes, rs, ps, x0, 0, bin_, lv, ox, 1, w, h)
        for f in range(3):
            want = oracle.develop(oracle.port(), "orc_develop", fmt, planes[f], rs, ps, x0, 0, bin_, lv, ox, 1, w, h)
            assert np.array_equal(got[f], want), (bin_, x0, ox, w, f)
