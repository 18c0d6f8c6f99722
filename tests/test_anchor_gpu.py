"""The anchor search on the GPU (lizg_anchor_find_dev), held bit for bit to the reference's portable build through
its fixtures and to the oracle on seeded captures: every ring span, lens model or none, batches of frames with their
own maps, anchors marked found before left as they are."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from test_anchor_oracle import FIELDS, golden_cases, same, seeded_capture

pytestmark = pytest.mark.gpu


def test_gpu_matches_reference_golden():
    for span, luma, H, lens, skip, want in golden_cases():
        got = lz.anchor_find(span, luma, H, None if lens is None else lens[None], skip[None])
        want = dict(want)
        # an anchor found before keeps the caller's buffers (zeros here) but its ok flag is the caller's too
        for k in FIELDS:
            got[k] = got[k][0].copy()
        got["ok"] = np.where(skip.astype(bool), want["ok"], got["ok"])
        assert same(got, want), "span %d" % span


@pytest.mark.parametrize("span,n,subch,W,Hh", [(128, 384, 64, 640, 600), (256, 768, 320, 900, 880), (512, 1536, 1024, 1700, 1700)])
def test_gpu_batch_matches_oracle(span, n, subch, W, Hh):
    frames = []
    for seed in range(4):
        frames.append(seeded_capture(span, n, subch, W, Hh, 10 * span + seed, seed & 1))
    luma = np.stack([f[0] for f in frames])
    H = np.stack([f[1] for f in frames])
    lens = np.stack([f[2] if f[2] is not None else np.array([0, W / 2, Hh / 2, 1.0] + [0.0] * 11) for f in frames])
    got = lz.anchor_find(span, luma, H, lens)
    found = 0
    for k, (lu, h, ln) in enumerate(frames):
        ln2 = ln if ln is not None else np.array([0, W / 2, Hh / 2, 1.0] + [0.0] * 11)
        want = oracle.anchor_find(oracle.port(), "orc_anchor_find", span, lu, h, ln2)
        assert same({f: got[f][k] for f in FIELDS}, want), "frame %d" % k
        found += want["found"]
    assert found >= 4 * 40
    # no lens model at all
    got0 = lz.anchor_find(span, luma[:1], H[:1])
    want0 = oracle.anchor_find(oracle.port(), "orc_anchor_find", span, luma[0], H[0], None)
    assert same({f: got0[f][0] for f in FIELDS}, want0)


def test_skip_leaves_outputs():
    span, luma, H, lens, skip, want = next(iter(golden_cases()))
    skip = np.ones(49, np.uint8)
    skip[7] = 0
    got = lz.anchor_find(span, luma, H, None, skip[None])
    assert got["ok"][0].sum() == want["ok"][7] and np.count_nonzero(got["peak"][0]) == 1


def test_bad_arguments():
    with pytest.raises(lz.LizgError):
        lz.anchor_find(100, np.zeros((1, 64, 64), np.uint8), np.eye(3, dtype=np.float32).ravel()[None])
