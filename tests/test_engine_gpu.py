"""The multi-stream engine (lizg_engine_*): batches of several formats decoded together, each on its own stream from
its own CUDA graph, or stage-wise across formats (every stage one launch over every format's items), give exactly what each format's receiver gives alone (blocks, CRC flags, iterations, soft values); replays of
the captured graphs give it again; the tuner keeps one of the two; bad runs are refused."""
import numpy as np
import pytest
import torch

import lizard_gb300 as lz
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu

FORMATS = [(384, 64, 128, 1280, 720), (768, 320, 128, 1100, 1000), (1152, 720, 256, 1400, 1400)]


def captures(n, subch, span, W, H, frames, seed, sigma=2.0):
    fmt = lz.Format(n, subch, span)
    rng = np.random.default_rng(seed)
    lumas, regs = [], []
    for k in range(frames):
        grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, seed + k), parity=k & 3)
        Hw = synth.warp(fmt, W, H, rng, rot_deg=10, scale=(0.95, 1.0))
        luma, reg = synth.capture(fmt, grey, W, H, H=Hw, sigma=sigma, rng=rng)
        lumas.append(luma)
        regs.append(reg)
    return np.stack(lumas), np.stack(regs)


def test_engine_matches_each_receiver():
    eng = lz.Engine()
    st = torch.cuda.current_stream().cuda_stream
    batches, keep, want = [], [], []
    for i, (n, subch, span, W, H) in enumerate(FORMATS):
        frames = 3 - (i % 2)
        assert eng.add_format(n, subch, span, frames) == i
        luma, reg = captures(n, subch, span, W, H, frames, 100 * i)
        want.append(lz.Receiver(n, subch, span, max_frames=frames).finish_luma(luma, reg, keep=False, grid=False))
        d_l, d_r = torch.from_numpy(luma).cuda(), torch.from_numpy(reg).cuda()
        o, s = lz.rx_outputs(eng.formats[i], frames)
        keep.append((d_l, d_r, o))
        batches.append((i, d_l.data_ptr(), W, H, W, W * H, d_r.data_ptr(), frames, s))
    for rep in range(3):   # the first run captures the graphs, the others replay them
        for _, _, o in keep:
            for t in o.values():
                t.zero_()
        eng.run_dev(batches, st)
        torch.cuda.synchronize()
        for i, (_, _, o) in enumerate(keep):
            for k in ("blocks", "ok", "its"):
                assert np.array_equal(o[k].cpu().numpy(), want[i][k]), (rep, i, k)
            assert want[i]["ok"].all()
    assert eng.launches == sum(5 + 3 + f.tiers for f in eng.formats)
    eng.close()


# two picture sizes of one ring, a size with two rings, noise enough at 768 for stalled and capped blocks
MIXED = [(384, 64, 128, 1280, 720, 3, 2.0), (768, 320, 128, 1100, 1000, 2, 45.0), (1152, 720, 256, 1400, 1400, 2, 2.0),
         (1536, 1024, 256, 1800, 1800, 1, 2.0), (1536, 1024, 512, 2400, 2400, 1, 2.0)]


def test_stage_wise_engine_matches_each_receiver():
    eng = lz.Engine()
    st = torch.cuda.current_stream().cuda_stream
    batches, keep, want = [], [], []
    for i, (n, subch, span, W, H, frames, sigma) in enumerate(MIXED):
        assert eng.add_format(n, subch, span, frames) == i
        luma, reg = captures(n, subch, span, W, H, frames, 300 + 100 * i, sigma)
        want.append(lz.Receiver(n, subch, span, max_frames=frames).finish_luma(luma, reg, keep=True, grid=False))
        d_l, d_r = torch.from_numpy(luma).cuda(), torch.from_numpy(reg).cuda()
        o, s = lz.rx_outputs(eng.formats[i], frames, keep=True)
        keep.append((d_l, d_r, o))
        batches.append((i, d_l.data_ptr(), W, H, W, W * H, d_r.data_ptr(), frames, s))
    assert (want[1]["its"] < 0).any() and (want[1]["ok"] == 0).any() and (want[1]["ok"] == 1).any()
    assert eng.set_mixed(1) == 0

    def check(tag):
        for i, (_, _, o) in enumerate(keep):
            for k in ("blocks", "ok", "its", "llrf", "est", "pilot", "align", "sub_rms"):
                a = o[k].cpu().numpy()
                assert np.array_equal(a, want[i][k], equal_nan=a.dtype.kind == "f"), (tag, i, k)   # a tier without pilots: NaN

    for rep in range(3):   # the first run captures the stage-wise graph, the others replay it
        for _, _, o in keep:
            for t in o.values():
                t.zero_()
        eng.run_dev(batches, st)
        torch.cuda.synchronize()
        check(rep)
    assert eng.launches == 8   # every stage one launch over the five formats
    # new contents in the same buffers: the replay reads them
    luma, reg = captures(*MIXED[0][:5], MIXED[0][5], 999)
    keep[0][0].copy_(torch.from_numpy(luma))
    keep[0][1].copy_(torch.from_numpy(reg))
    want[0] = lz.Receiver(*MIXED[0][:3], max_frames=MIXED[0][5]).finish_luma(luma, reg, keep=True, grid=False)
    eng.run_dev(batches, st)
    torch.cuda.synchronize()
    check("new frames")
    # the tuner runs both ways and keeps one; the outputs stay the same
    mode, ms = eng.autotune(batches, st)
    torch.cuda.synchronize()
    assert mode in (0, 1) and ms[0] > 0 and ms[1] > 0 and eng.set_mixed(mode) == mode
    check("tuned")
    eng.close()


def test_stage_wise_engine_chunks_many_formats():
    """More formats than one grid takes (8) and more tiers than one decode launch takes (32): the column and row
    passes and the decode split into several grids, the outputs still each receiver's own."""
    eng = lz.Engine()
    st = torch.cuda.current_stream().cuda_stream
    specs = [(384, 64, 128, 1280, 720)] * 6 + [(768, 320, 128, 1100, 1000)] * 4
    batches, keep, want = [], [], []
    for i, (n, subch, span, W, H) in enumerate(specs):
        assert eng.add_format(n, subch, span, 1) == i
        luma, reg = captures(n, subch, span, W, H, 1, 900 + i, 2.0 if i % 3 else 30.0)
        want.append(lz.Receiver(n, subch, span, max_frames=1).finish_luma(luma, reg, keep=True, grid=False))
        d_l, d_r = torch.from_numpy(luma).cuda(), torch.from_numpy(reg).cuda()
        o, s = lz.rx_outputs(eng.formats[i], 1, keep=True)
        keep.append((d_l, d_r, o))
        batches.append((i, d_l.data_ptr(), W, H, W, W * H, d_r.data_ptr(), 1, s))
    tiers = sum(f.tiers for f in eng.formats)
    assert len(specs) > 8 and tiers > 32
    eng.set_mixed(1)
    for rep in range(2):
        eng.run_dev(batches, st)
        torch.cuda.synchronize()
        for i, (_, _, o) in enumerate(keep):
            for k in ("blocks", "ok", "its", "llrf", "est"):
                a = o[k].cpu().numpy()
                assert np.array_equal(a, want[i][k], equal_nan=a.dtype.kind == "f"), (rep, i, k)
    assert eng.launches == 7 * 2 + (tiers + 31) // 32   # each stage over 8 formats a launch
    eng.close()


def test_engine_refuses_bad_runs():
    eng = lz.Engine()
    eng.add_format(384, 64, 128, 1)
    o, s = lz.rx_outputs(eng.formats[0], 1)
    d = torch.zeros((720, 1280), dtype=torch.uint8, device="cuda")
    r = torch.zeros(9 + 2 * 40 * 40, dtype=torch.float32, device="cuda")
    b = (0, d.data_ptr(), 1280, 720, 1280, 1280 * 720, r.data_ptr(), 1, s)
    with pytest.raises(lz.LizgError):
        eng.run_dev([b, b], 0)          # a format twice
    with pytest.raises(lz.LizgError):
        eng.run_dev([(3,) + b[1:]], 0)  # no such format
    with pytest.raises(lz.LizgError):
        eng.add_format(500, 64, 128, 1)  # no such picture size
    eng.close()
