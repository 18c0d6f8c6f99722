"""The anchor search's oracle (oracle/oracle_anchor.c), held bit for bit to the reference's own portable build: its
fixtures (tests/golden/anchor_ref.npz) and, where the reference tree is present, the reference compiled here on fresh
seeded captures (three ring spans, with and without a lens model, anchors found before)."""
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("ok", "peak", "dx", "dy", "u", "v")


def golden_cases():
    g = np.load(os.path.join(GOLD, "anchor_ref.npz"))
    for c in range(int(g["cases"])):
        lens = g["c%d_lens" % c]
        yield (int(g["c%d_span" % c]), g["c%d_luma" % c], g["c%d_H" % c], lens if lens.size else None, g["c%d_skip" % c],
               {k: g["c%d_%s" % (c, k)] for k in FIELDS})


def same(a, b):
    return all(np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)) for k in FIELDS)


def test_oracle_matches_reference_golden():
    n = 0
    for span, luma, H, lens, skip, want in golden_cases():
        got = oracle.anchor_find(oracle.port(), "orc_anchor_find", span, luma, H, lens, skip)
        assert same(got, want), "span %d" % span
        n += 1
    assert n == 4


def seeded_capture(span, n, subch, W, Hh, seed, with_lens):
    fmt = lz.Format(n, subch, span)
    rng = np.random.default_rng(seed)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed), parity=seed & 3)
    Hw = synth.warp(fmt, W, Hh, rng, rot_deg=12)
    luma, reg = synth.capture(fmt, grey, W, Hh, H=Hw, sigma=2.0, rng=rng)
    H = reg[:9].astype(np.float32).copy()
    pxm = n / span
    H[2] += np.float32(rng.uniform(-1, 1) * pxm)
    H[5] += np.float32(rng.uniform(-1, 1) * pxm)
    lens = None
    if with_lens:
        lens = np.zeros(15)
        lens[:4] = [1 + seed % 3, W / 2, Hh / 2, np.hypot(W, Hh) / 2]
        lens[4:12] = rng.uniform(-0.5, 0.5, 8)
        lens[12:12 + int(lens[0])] = rng.uniform(-0.05, 0.05, int(lens[0]))
    return luma, H, lens


@pytest.mark.skipif(oracle.ref_scalar() is None, reason="the reference's portable build is not here")
@pytest.mark.parametrize("span,n,subch,W,Hh,seed,with_lens", [(128, 384, 64, 640, 600, 1, False), (128, 384, 80, 640, 600, 2, True),
                                                               (256, 768, 320, 900, 880, 3, True), (512, 1536, 1024, 1700, 1700, 4, False)])
def test_oracle_matches_reference_build(span, n, subch, W, Hh, seed, with_lens):
    luma, H, lens = seeded_capture(span, n, subch, W, Hh, seed, with_lens)
    skip = np.zeros(49, np.uint8)
    skip[::5] = seed & 1
    a = oracle.anchor_find(oracle.port(), "orc_anchor_find", span, luma, H, lens, skip)
    b = oracle.anchor_find(oracle.ref_scalar(), "refs_anchor_find", span, luma, H, lens, skip)
    assert same(a, b)
    assert a["found"] == b["found"] and a["found"] >= 40


@pytest.mark.skipif(oracle.ref_scalar() is None, reason="the reference's portable build is not here")
@pytest.mark.parametrize("seed,k1", [(1, 0.0), (2, 0.03), (3, -0.04), (4, 0.05)])
def test_lens_fit_matches_reference(seed, k1):
    """The lens model from the anchors (anchor_model) on distorted captures, bit for bit."""
    fmt = lz.Format(1536, 1024, 256)
    rng = np.random.default_rng(seed)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed), parity=seed & 3)
    H = synth.distorted_view(fmt, 1920, 1080, rng, base_side=1000)
    luma, reg = synth.distorted_capture(fmt, grey, 1920, 1080, H, k1=k1, blur=1.0, sigma=3.0, rng=rng)
    a = oracle.anchor_find(oracle.port(), "orc_anchor_find", 256, luma, reg[:9])
    assert a["found"] >= 30
    f1, l1 = oracle.lens_fit(oracle.port(), "orc_lens_fit", 256, 1920, 1080, reg[:9], a["ok"], a["dx"], a["dy"])
    f2, l2 = oracle.lens_fit(oracle.ref_scalar(), "refs_anchor_model", 256, 1920, 1080, reg[:9], a["ok"], a["dx"], a["dy"])
    assert f1 == f2 == 1
    assert np.array_equal(l1.view(np.uint64), l2.view(np.uint64)), (l1, l2)


def registration_case(seed, k1, blur, moved):
    """A distorted capture of LIZARD-1024 in the 128 ring (1920 x 1080) and what a finder hands the registration: the
    corners in the image (quad; with moved = c + 1, corner c placed 15 modules off, past the 3 the rule allows),
    the homography through them and the pixels a module, as the reference's acquisition forms them."""
    fmt = lz.Format(1536, 1024, 256)
    rng = np.random.default_rng(seed)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed), parity=seed & 3)
    Hv = synth.distorted_view(fmt, 1920, 1080, rng, base_side=1000)
    luma, reg = synth.distorted_capture(fmt, grey, 1920, 1080, Hv, k1=k1, blur=blur, sigma=3.0, rng=rng)
    nodes = synth.layout_nodes(256)
    lo, hi = float(nodes[0]), float(nodes[-1])
    src = np.array([[lo, lo], [hi, lo], [hi, hi], [lo, hi]], np.float64)
    H0 = reg[:9].astype(np.float64).reshape(3, 3)
    q = H0 @ np.column_stack([src, np.ones(4)]).T
    quad = np.stack([q[0] / q[2], q[1] / q[2]], 1).astype(np.float32)
    sides = [np.hypot(*(quad[(k + 1) % 4] - quad[k])) / np.hypot(*(src[(k + 1) % 4] - src[k])) for k in range(4)]
    mpx = np.float32(sum(np.float32(s) / np.float32(4) for s in sides))
    if moved:
        quad[moved - 1] += np.float32(15 * mpx) * np.float32([0.6, 0.8])
    H = synth.homography_4(src, quad.astype(np.float64)).astype(np.float32).ravel()
    return luma, H, quad.ravel(), float(mpx)


@pytest.mark.skipif(oracle.ref_scalar() is None, reason="the reference's portable build is not here")
@pytest.mark.parametrize("seed,k1,blur,moved", [(1, 0.0, 1.0, 0), (2, 0.03, 1.5, 0), (3, -0.04, 0.8, 1), (4, 0.05, 1.0, 3)])
def test_anchor_register_matches_reference(seed, k1, blur, moved):
    """The code registered from the anchors (anchor_register: rounds through the anchors' own homography and robust
    model, each corner judged by their map and searched again where it disagrees, H made again, the model about H),
    the oracle against the reference's portable build, bit for bit."""
    luma, H, quad, mpx = registration_case(seed, k1, blur, moved)
    a = oracle.anchor_register(oracle.port(), "orc_anchor_register", 256, luma, H, quad, mpx)
    b = oracle.anchor_register(oracle.ref_scalar(), "refs_anchor_register", 256, luma, H, quad, mpx)
    assert a["held"] == b["held"] == 1
    for k in ("H", "quad", "lens") + FIELDS:
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k
    assert a["ok"].sum() >= 30
    if moved:   # the corner put 15 modules off comes back
        assert not np.array_equal(a["quad"], quad)
