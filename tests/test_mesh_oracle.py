"""The border nodes' oracle (oracle/oracle_anchor.c orc_border_nodes: refine_node over the border lattice in the
reference's order) held to the reference's own portable build (oracle/_ref/libref_scalar.so refs_border_nodes,
compiled from its sources) bit for bit, on captures in the three rings with H off by up to a pixel, with and without
a lens model; where the reference tree is absent, to its outputs stored in tests/golden/mesh_ref.npz."""
import os

import numpy as np
import pytest

import oracle
from lizard_gb300_testing import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "mesh_ref.npz")


def mesh_cases(seed, count):
    """Seeded captures of a symbol's border (its word, track, line and corner marks): ring, pixels a module, blur,
    the map H put up to a pixel off, a lens model on every other."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        span, pxm = ((128, 3), (256, 2), (512, 1))[t % 3]
        W = H = 720
        luma, reg, _ = synth.word_capture(span, pxm, int(rng.integers(4, 65)), 30, W, H, rng, blur=float(rng.choice([0.0, 0.8, 1.5])), sigma=3.0)
        Hm = reg[:9].copy()
        Hm[2] += np.float32(rng.uniform(-1, 1))
        Hm[5] += np.float32(rng.uniform(-1, 1))
        lens = None
        if t % 2:
            lens = np.zeros(15, np.float64)
            lens[0], lens[1], lens[2], lens[3] = 1, W / 2, H / 2, np.hypot(W, H) / 2
            lens[4:] = rng.normal(0, 0.3, 11)
        out.append((span, luma, Hm, lens))
    return out


def nodes_oracle(span, luma, Hm, lens):
    nn = synth.layout_nodes(span).size
    out = np.zeros(4 * nn * nn, np.float32)
    assert oracle.port().orc_border_nodes(span, oracle._p(luma), luma.shape[1], luma.shape[0], oracle._p(Hm),
                                          None if lens is None else oracle._p(lens), oracle._p(out)) == nn
    return out.reshape(nn, nn, 4)


def test_border_nodes_match_reference():
    R = oracle.ref_scalar()
    if R is None:
        pytest.skip("the reference tree is not here")
    refined = 0
    for span, luma, Hm, lens in mesh_cases(3, 9):
        want = np.zeros_like(nodes_oracle(span, luma, Hm, lens)).ravel()
        R.refs_border_nodes(span, oracle._p(luma), luma.shape[1], luma.shape[0], oracle._p(Hm), None if lens is None else oracle._p(lens), oracle._p(want))
        got = nodes_oracle(span, luma, Hm, lens)
        assert np.array_equal(got.ravel().view(np.uint32), want.view(np.uint32)), span
        refined += int((got[..., 2] >= 0.35).sum())
    assert refined > 100


def test_border_nodes_golden():
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        span, iw, ih = (int(v) for v in g["geom"][c])
        lens = g["lens_%d" % c] if g["has_lens"][c] else None
        got = nodes_oracle(span, g["luma_%d" % c].reshape(ih, iw), g["H_%d" % c], lens)
        assert np.array_equal(got.ravel().view(np.uint32), g["nodes_%d" % c].view(np.uint32)), c
