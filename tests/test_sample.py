"""Row a, the picture sampler in its two reads: the oracle's exact walk and its restatement of the decode's integer
read held to the reference's own (where built here) and, on the GPU, the sampler kernel and the transform's fused
sampling held to the oracle bit for bit, then rows a-e end to end from captured luma frames."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

CASES = [(384, 64, 1280, 720, False), (384, 64, 1280, 720, True), (768, 320, 1920, 1080, True), (1536, 1024, 3840, 2160, True)]


def frame(n, subch, W, H, warped, seed=1, mesh=0.0):
    f = lz.Format(n, subch, 128)
    rng = np.random.default_rng(seed)
    blocks = synth.random_blocks(f.blocks, seed)
    grey = synth.picture(f, blocks)
    Hm = synth.warp(f, W, H, rng) if warped else None
    luma, reg = synth.capture(f, grey, W, H, H=Hm, sigma=2.0, rng=rng)
    if mesh:
        reg[9:] = rng.uniform(-mesh, mesh, reg[9:].size).astype(np.float32)
    return f, luma, reg, blocks


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")
@pytest.mark.parametrize("n,subch,W,H,warped", CASES[:3])
def test_oracle_walk_matches_reference(n, subch, W, H, warped):
    f, luma, reg, _ = frame(n, subch, W, H, warped, mesh=0.6)
    o, r = oracle.Fmt(n, subch, 128), oracle.RefFmt(n, subch, 128)
    go = o.sample(luma, reg)
    assert np.array_equal(go, r.sample_grid(luma, reg[:9], reg[9:], fast=False))
    # the reference decoder's own integer read, within its test's 1/200 of grey of the walk
    assert np.abs(r.sample_grid(luma, reg[:9], reg[9:], fast=True) - go).max() < 1 / 200


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")
@pytest.mark.parametrize("n,subch,W,H,warped", CASES)
def test_oracle_decode_read_matches_reference(n, subch, W, H, warped):
    """The decode's own read (strips of 64 columns, the integer read) and the shading fit's samples, bit for bit."""
    f, luma, reg, _ = frame(n, subch, W, H, warped, mesh=0.6)
    o, r = oracle.Fmt(n, subch, 128), oracle.RefFmt(n, subch, 128)
    go, so = o.sample_decode(luma, reg)
    gr, sr, lin = r.sample_decode(luma, reg[:9], reg[9:])
    assert lin
    assert np.array_equal(go.view(np.uint32), gr.view(np.uint32))
    assert np.array_equal(so.view(np.uint32), sr.view(np.uint32))
    # the same map as the exact walk, within the reference's own bar of 1/200 of a grey level
    assert np.abs(go - o.sample(luma, reg)).max() < 1 / 200


@pytest.mark.parametrize("n,subch,W,H,warped", CASES)
def test_captures_decode_in_the_oracle(n, subch, W, H, warped):
    f, luma, reg, blocks = frame(n, subch, W, H, warped)
    o = oracle.Fmt(n, subch, 128)
    res = o.receive(o.sample(luma, reg))
    assert res["ok"].all() and np.array_equal(res["blocks"], blocks)


@pytest.mark.gpu
@pytest.mark.parametrize("read", ["decode", "exact"])
@pytest.mark.parametrize("n,subch,W,H,warped", CASES)
def test_gpu_luma_path_matches_oracle(n, subch, W, H, warped, read):
    import torch
    f, luma, reg, blocks = frame(n, subch, W, H, warped, mesh=0.3 if warped else 0.0)
    o = oracle.Fmt(n, subch, 128)
    go = o.sample(luma, reg) if read == "exact" else o.sample_decode(luma, reg)[0]
    rx = lz.Receiver(n, subch, 128, max_frames=2, read=read)
    out = rx.finish_luma(np.stack([luma, luma]), np.stack([reg, reg]))
    for k in range(2):
        assert np.array_equal(out["grid"][k], go)
    res = o.receive(go.copy())
    c = out["coef"][0]
    d, used = o.pilot_align(c)
    turn = d if (used and (d[0] != 0 or d[1] != 0)) else None
    llrf, est, rms = o.demap(c, turn)
    assert np.array_equal(out["llrf"][0], llrf)
    assert np.array_equal(out["ok"][0], res["ok"]) and out["ok"][0].all()
    assert np.array_equal(out["blocks"][0], blocks)
    assert rx.launches == 1 + 4 + 3 + f.tiers
    # the sampler fused into the transform's passes (no grid asked for) gives the same spectrum, soft values, blocks
    fused = rx.finish_luma(np.stack([luma, luma]), np.stack([reg, reg]), grid=False)
    for k in ("coef", "llrf", "its", "ok", "blocks", "align"):
        assert np.array_equal(fused[k], out[k]), k
    assert rx.launches == 5 + 3 + f.tiers


@pytest.mark.gpu
@pytest.mark.parametrize("n,subch,W,H,warped", [CASES[0], CASES[3]])
def test_gpu_autotune_keeps_every_block(n, subch, W, H, warped):
    """The receiver's per-tier LDPC choice (lizg_rx_autotune) times every kernel variant of each tier's code on the
    batch; the variants decode bit for bit alike, so the blocks, verdicts and iterations stay the same, directly and
    from a captured graph."""
    import torch
    f, luma, reg, blocks = frame(n, subch, W, H, warped, mesh=0.3)
    frames = 3
    rx = lz.Receiver(n, subch, 128, max_frames=frames)
    before = rx.finish_luma(np.stack([luma] * frames), np.stack([reg] * frames), grid=False)
    d_l = torch.from_numpy(np.stack([luma] * frames)).cuda()
    d_r = torch.from_numpy(np.stack([reg] * frames)).cuda()
    choice = rx.autotune_dev(d_l.data_ptr(), W, H, W, W * H, d_r.data_ptr(), frames)
    for t in range(4):
        if t < f.tiers:
            assert 0 <= choice[t] < lz.lib().lizg_ldpc_variants(f.tier[t][0]) and rx.variant(t) == choice[t]
        else:
            assert choice[t] == -1
    after = rx.finish_luma(np.stack([luma] * frames), np.stack([reg] * frames), grid=False)
    for k in ("blocks", "ok", "its", "llrf", "coef"):
        assert np.array_equal(after[k], before[k]), k
    assert after["ok"].all() and np.array_equal(after["blocks"][0], blocks)
