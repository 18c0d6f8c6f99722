"""The sender on the GPU (lizg_encoder_*, lizg_encode_dev) against the oracle (lizard_gb300.synth.encode_drive, held
to the reference's own encoder in test_encode_oracle.py) and the reference's page crops; and end to end: the GPU's
pages decoded by the GPU receiver give back every block, and their format word reads."""
import numpy as np
import pytest

import lizard_gb300 as lz
from lizard_gb300_testing import synth
from test_encode_oracle import DRIVE_TOL, FORMATS, GOLDEN, GREY_FRACTION, golden_crops

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,subch,span", FORMATS)
def test_encoder_matches_oracle(n, subch, span):
    fmt = lz.Format(n, subch, span)
    enc = lz.Encoder(n, subch, span, max_frames=2)
    blocks = np.stack([synth.random_blocks(fmt.blocks, 30 + k) for k in range(2)])
    for pilots in (0, 2):
        drive, grey = enc.encode(blocks, pilots=pilots)
        for k in range(2):
            d, g = synth.encode_drive(fmt, blocks[k], parity=pilots)
            assert np.abs(drive[k] - d).max() <= DRIVE_TOL, (k, pilots)
            diff = grey[k].astype(int) - g.astype(int)
            assert np.abs(diff).max() <= 1 and np.count_nonzero(diff) <= GREY_FRACTION * diff.size, (k, pilots)


def test_encoder_golden():
    """The reference sender's own pages, in the crops the fixture keeps."""
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        n, subch, span, seed, pilots = (int(v) for v in g["case"][c])
        fmt = lz.Format(n, subch, span)
        enc = lz.Encoder(n, subch, span, max_frames=1)
        _, grey = enc.encode(synth.random_blocks(fmt.blocks, seed)[None], pilots=pilots, drive=False)
        for k, crop in enumerate(golden_crops(grey[0], enc.pxm)):
            diff = crop.astype(int) - g["crop_%d_%d" % (c, k)].astype(int)
            assert np.abs(diff).max() <= 1 and np.count_nonzero(diff) <= max(2, GREY_FRACTION * diff.size), (c, k)


@pytest.mark.parametrize("n,subch,span", [(384, 64, 128), (768, 320, 256), (1536, 1024, 256)])
def test_pages_decode(n, subch, span):
    """The page seen straight on (module (x, y) at pixel 2 pxm + pxm (x, y)), with noise: the receiver gives back every
    block, and the format word reads as the version and rate painted."""
    fmt = lz.Format(n, subch, span)
    enc = lz.Encoder(n, subch, span, max_frames=2)
    enc.set_fps(60)
    blocks = np.stack([synth.random_blocks(fmt.blocks, 40 + k) for k in range(2)])
    _, grey = enc.encode(blocks, pilots=1, drive=False)
    rng = np.random.default_rng(5)
    pages = np.clip(np.rint(grey + rng.normal(0, 2.0, grey.shape)), 0, 255).astype(np.uint8)
    pxm = enc.pxm
    nn = synth.layout_nodes(span).size
    reg = np.zeros((2, 9 + 2 * nn * nn), np.float32)
    reg[:, :9] = [pxm, 0, 2 * pxm, 0, pxm, 2 * pxm, 0, 0, 1]
    rx = lz.Receiver(n, subch, span, max_frames=2)
    out = rx.finish_luma(pages, reg, grid=False)
    for k in range(2):
        assert out["ok"][k].all(), (k, int(out["ok"][k].sum()), fmt.blocks)
        assert np.array_equal(out["blocks"][k], blocks[k])
    _, word = lz.fmt_read(span, pages, reg)
    assert word.tolist() == [[1, 1, subch // 16, 60]] * 2


def test_encoder_arguments():
    with pytest.raises(lz.LizgError):
        lz.Encoder(384, 64, 100)
    enc = lz.Encoder(384, 64, 128, max_frames=1)
    with pytest.raises(lz.LizgError):
        enc.encode(np.zeros((2, enc.blocks, 476), np.uint8))
    with pytest.raises(lz.LizgError):
        enc.set_fps(256)
