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
