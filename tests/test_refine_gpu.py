"""The registration's refinement from the anchors on the GPU (lizg_refine_dev): its lens model bit for bit the
oracle's restatement of the reference's anchor_model on the oracle's anchors, its node mesh the model's values at the
nodes, and on distorted captures (radial k1, blur in linear light) at least the plain homography's CRC-passing
blocks."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu
W, H = 1920, 1080


def distorted(seed, k1, blur, base=1000.0):
    fmt = lz.Format(1536, 1024, 256)
    rng = np.random.default_rng(seed)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed), parity=seed & 3)
    view = synth.distorted_view(fmt, W, H, rng, base_side=base)
    luma, reg = synth.distorted_capture(fmt, grey, W, H, view, k1=k1, blur=blur, sigma=3.0, rng=rng)
    return fmt, luma, reg


def mesh_expected(reg, lens, span):
    """The model's displacement at every node through H: float32 projection, double model, float32 result."""
    f32 = np.float32
    h = reg[:9].astype(np.float32)
    nodes = synth.layout_nodes(span).astype(np.float32)
    nn = nodes.size
    out = np.zeros(2 * nn * nn, np.float32)
    K = int(lens[0])
    for k in range(nn * nn):
        x, y = f32(nodes[k % nn]), f32(nodes[k // nn])
        w = h[6] * x + h[7] * y + f32(1)
        u = (h[0] * x + h[1] * y + h[2]) / w
        v = (h[3] * x + h[4] * y + h[5]) / w
        X, Y = (float(u) - lens[1]) / lens[3], (float(v) - lens[2]) / lens[3]
        rx = [X, Y, 0.0, 0.0, 1.0, 0.0, -X * X, -X * Y]
        ry = [0.0, 0.0, X, Y, 0.0, 1.0, -X * Y, -Y * Y]
        s = X * X + Y * Y
        sk = s
        for _ in range(3):
            rx.append(sk * X)
            ry.append(sk * Y)
            sk *= s
        fx = fy = 0.0
        for c in range(8 + K):
            fx += lens[4 + c] * rx[c]
            fy += lens[4 + c] * ry[c]
        out[2 * k], out[2 * k + 1] = f32(fx), f32(fy)
    return out


@pytest.mark.parametrize("seed,k1", [(1, 0.03), (2, -0.04), (3, 0.05)])
def test_one_round_matches_oracle(seed, k1):
    fmt, luma, reg = distorted(seed, k1, 1.0)
    reg2, found, lens = lz.Refiner(256, 1).refine(luma, reg, rounds=1)
    a = oracle.anchor_find(oracle.port(), "orc_anchor_find", 256, luma, reg[:9])
    fit, want = oracle.lens_fit(oracle.port(), "orc_lens_fit", 256, W, H, reg[:9], a["ok"], a["dx"], a["dy"])
    assert found[0] == a["found"] >= 30 and fit == 1
    assert np.array_equal(lens[0].view(np.uint64), want.view(np.uint64)), (lens[0], want)
    assert np.array_equal(reg2[0][:9], reg[:9])
    assert np.array_equal(reg2[0][9:], mesh_expected(reg, want, 256))


def test_refined_decodes_what_plain_cannot():
    """Radial distortion the four corners' homography cannot hold: the plain registration verifies next to nothing,
    the refined one most of what a clean capture at this scale verifies (about half of the 124 blocks)."""
    cases = [(10, 0.03, 0.0), (11, -0.04, 0.0), (12, 0.02, 0.5), (13, 0.04, 0.5)]
    frames = [distorted(s, k1, blur, base=1040.0) for s, k1, blur in cases]
    luma = np.stack([f[1] for f in frames])
    reg = np.stack([f[2] for f in frames])
    reg3, found3, _ = lz.Refiner(256, 4).refine(luma, reg, rounds=3)
    _, found1, _ = lz.Refiner(256, 4).refine(luma, reg, rounds=1)
    assert (found3 >= found1).all() and (found3 >= 40).all()
    rx = lz.Receiver(1536, 1024, 256, max_frames=4)
    plain = rx.finish_luma(luma, reg, keep=False, grid=False)
    refined = rx.finish_luma(luma, reg3, keep=False, grid=False)
    print("blocks verified: plain %d refined %d of %d" % (plain["ok"].sum(), refined["ok"].sum(), plain["ok"].size))
    assert refined["ok"].sum() >= plain["ok"].sum() + 4 * 25


def test_anchor_register_matches_oracle():
    """The reference's whole registration from the anchors on the GPU (lizg_anchor_register_dev: rounds through the
    anchors' own homography and robust model, the corners judged and searched again, H made again, the model about H)
    against the oracle's restatement (itself held to the reference's portable build on the same cases), four frames
    in one call: held, H, the corners, the model and every anchor bit for bit, the mesh the model at the nodes."""
    import test_anchor_oracle as tao
    cases = [tao.registration_case(seed, k1, blur, moved) for seed, k1, blur, moved in
             [(1, 0.0, 1.0, 0), (2, 0.03, 1.5, 0), (3, -0.04, 0.8, 1), (4, 0.05, 1.0, 3), (5, 0.02, 1.2, 2)]]
    nn = synth.layout_nodes(256).size
    luma = np.stack([c[0] for c in cases])
    reg = np.zeros((len(cases), 9 + 2 * nn * nn), np.float32)
    for f, c in enumerate(cases):
        reg[f, :9] = c[1]
    quad = np.stack([c[2] for c in cases])
    rf = lz.Refiner(256, len(cases))
    got = rf.register(luma, reg, quad=quad)
    for f, (lu, Hc, q, mpx) in enumerate(cases):
        want = oracle.anchor_register(oracle.port(), "orc_anchor_register", 256, lu, Hc, q, mpx)
        assert got["held"][f] == want["held"] == 1, f
        assert np.array_equal(got["reg"][f, :9].view(np.uint32), want["H"].view(np.uint32)), f
        assert np.array_equal(got["quad"][f].view(np.uint32), want["quad"].view(np.uint32)), f
        assert np.array_equal(got["lens"][f].view(np.uint64), want["lens"].view(np.uint64)), f
        for k in ("ok", "peak", "dx", "dy", "u", "v"):
            assert np.array_equal(np.asarray(got[k][f]).view(np.uint8), np.asarray(want[k]).view(np.uint8)), (f, k)
        assert np.array_equal(got["reg"][f, 9:], mesh_expected(got["reg"][f], got["lens"][f], 256)), f


def test_anchor_register_defaults():
    """lizg_anchor_register_dev with no corners given (the corner nodes through H) and the frame itself given as the
    border search's image: the oracle's results with the corners H gives; the same frames with rim omitted agree."""
    import test_anchor_oracle as tao
    luma, Hc, _, _ = tao.registration_case(6, 0.02, 1.0, 0)
    nn = synth.layout_nodes(256).size
    reg = np.zeros((1, 9 + 2 * nn * nn), np.float32)
    reg[0, :9] = Hc
    rf = lz.Refiner(256, 1)
    a = rf.register(luma[None], reg)
    b = rf.register(luma[None], reg, rim=luma[None])
    assert a["quad"] is None
    for k in ("reg", "held", "lens", "ok", "u", "v"):
        assert np.array_equal(a[k], b[k]), k
    # the corners the device took: the corner nodes through H, as float projections
    nodes = synth.layout_nodes(256).astype(np.float32)
    lo, hi = nodes[0], nodes[-1]
    h = Hc.astype(np.float32)
    quad = []
    for x, y in ((lo, lo), (hi, lo), (hi, hi), (lo, hi)):
        w = h[6] * x + h[7] * y + np.float32(1)
        quad += [(h[0] * x + h[1] * y + h[2]) / w, (h[3] * x + h[4] * y + h[5]) / w]
    quad = np.array(quad, np.float32)
    sides = [np.float32(np.hypot(*(quad[2 * ((k + 1) % 4):2 * ((k + 1) % 4) + 2] - quad[2 * k:2 * k + 2]))) for k in range(4)]
    assert a["held"][0] == 1 and a["ok"][0].sum() >= 30
    want = oracle.anchor_register(oracle.port(), "orc_anchor_register", 256, luma, Hc, quad,
                                  float(sum(np.float32(s) / np.float32(hi - lo) / np.float32(4) for s in sides)))
    assert want["held"] == 1
    assert np.array_equal(a["ok"][0], want["ok"])
