"""The format word on the GPU (lizg_fmt_read_dev, lizg_fmt_decode_dev) against the oracle's restatement of the
reference (bit-exact soft values, the same words) and against the reference's own outputs in the committed fixture:
captures in the three rings that read cleanly, after erasures and not at all, batches of frames, frames with no
border contrast, soft values that are garbage."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth
from test_fmt_oracle import GOLDEN, capture_cases, random_q, read_oracle

pytestmark = pytest.mark.gpu


def test_fmt_read_matches_oracle():
    cases = capture_cases(7, 36)
    outcomes = set()
    for span in (128, 256, 512):
        mine = [c for c in cases if c[0] == span]
        lumas = np.stack([c[1] for c in mine])
        regs = np.stack([c[2] for c in mine])
        q, word = lz.fmt_read(span, lumas, regs)
        for f, (_, luma, reg) in enumerate(mine):
            qo, wo = read_oracle(span, luma, reg)
            assert np.array_equal(word[f], wo), (span, f, word[f], wo)
            if wo[0]:
                assert np.array_equal(q[f].view(np.uint32), qo.view(np.uint32)), (span, f)
            else:
                assert not q[f].any()
            outcomes.add((int(wo[0]), int(wo[1])))
    assert {(1, 1), (1, 0)} <= outcomes, outcomes


def test_fmt_golden_gpu():
    """The reference's own soft values and words, stored with the frames they were read from."""
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        span, iw, ih = (int(v) for v in g["geom"][c])
        q, word = lz.fmt_read(span, g["luma_%d" % c].reshape(1, ih, iw), g["reg_%d" % c][None])
        assert np.array_equal(word[0], g["word"][c]), c
        if word[0][0]:
            assert np.array_equal(q[0].view(np.uint32), g["q_%d" % c].view(np.uint32)), c
    for c in range(int(g["dcount"])):
        cells, nbytes = (int(v) for v in g["dgeom"][c])
        span = {32: 128, 64: 256, 128: 512}[cells]
        word = lz.fmt_decode(span, g["dq_%d" % c][None])[0]
        rc, ver, fps = (int(v) for v in g["dout"][c])
        assert (word[1], word[2], word[3]) == (int(rc == 0), ver, fps), c


def test_fmt_decode_matches_oracle():
    """Clean, noisy, faded (erasures) and garbage soft values, a batch a word length."""
    rng = np.random.default_rng(4)
    P = oracle.port()
    paths = set()
    for span in (128, 256, 512):
        cells, nbytes = synth.fmt_geometry(span)
        qs = np.stack([random_q(rng, cells, nbytes, ("noisy", "faded", "garbage", "clean")[t % 4]) for t in range(160)])
        word = lz.fmt_decode(span, qs)
        for f in range(qs.shape[0]):
            vf = np.zeros(2, np.int32)
            rc = P.orc_fmt_decode(oracle._p(qs[f]), cells, nbytes, oracle._p(vf))
            want = (1, int(rc == 0), int(vf[0]) if rc == 0 else 0, int(vf[1]) if rc == 0 else 0)
            assert tuple(int(v) for v in word[f]) == want, (span, f)
            paths.add(rc == 0)
    assert paths == {True, False}


def test_fmt_no_contrast_is_not_read():
    span = 256
    nn = synth.layout_nodes(span).size
    luma = np.full((2, 300, 400), 128, np.uint8)
    reg = np.zeros((2, 9 + 2 * nn * nn), np.float32)
    reg[:, 0] = reg[:, 4] = 1.2
    reg[:, 8] = 1.0
    q, word = lz.fmt_read(span, luma, reg)
    assert not word.any() and not q.any()
