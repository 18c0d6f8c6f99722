"""The border nodes on the GPU (lizg_border_nodes_dev) against the oracle (held to the reference in
test_mesh_oracle.py) bit for bit, a batch of frames a ring, with and without lens models; and against the reference's
outputs in the committed fixture."""
import numpy as np
import pytest

import lizard_gb300 as lz
from test_mesh_oracle import GOLDEN, mesh_cases, nodes_oracle

pytestmark = pytest.mark.gpu


def test_border_nodes_match_oracle():
    cases = mesh_cases(3, 18)
    for span in (128, 256, 512):
        for with_lens in (False, True):
            mine = [c for c in cases if c[0] == span and (c[3] is not None) == with_lens]
            if not mine:
                continue
            lumas = np.stack([c[1] for c in mine])
            Hs = np.stack([c[2] for c in mine])
            lens = np.stack([c[3] for c in mine]) if with_lens else None
            got = lz.border_nodes(span, lumas, Hs, lens)
            for f, (_, luma, Hm, ln) in enumerate(mine):
                want = nodes_oracle(span, luma, Hm, ln)
                assert np.array_equal(got[f].view(np.uint32), want.view(np.uint32)), (span, with_lens, f)


def test_border_nodes_golden_gpu():
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        span, iw, ih = (int(v) for v in g["geom"][c])
        lens = g["lens_%d" % c][None] if g["has_lens"][c] else None
        got = lz.border_nodes(span, g["luma_%d" % c].reshape(1, ih, iw), g["H_%d" % c][None], lens)
        assert np.array_equal(got[0].ravel().view(np.uint32), g["nodes_%d" % c].view(np.uint32)), c
