"""The batching front (lizg_receiver_*, the reference's liz_receiver_* for registered frames) and the host-memory
finish (lizg_rx_finish_luma_host, the reference's lizard_finish from host buffers), driven through the C ABI: every
frame pushed is released before push returns and exactly once, the frames are decoded in batches on the front's own
thread, and each frame's CRC verdicts, iterations and verified bytes equal lizg_rx_finish_luma_dev's on the same
frame; with fewer slots than frames in flight the frames that find none are dropped and counted, and still released."""
import json

import numpy as np
import pytest

import lizard_gb300 as lz
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu


def frames(count, seed=31):
    f = lz.Format(384, 64, 128)
    rng = np.random.default_rng(seed)
    lumas, regs = [], []
    for k in range(count):
        grey = synth.picture(f, synth.random_blocks(f.blocks, seed + k), parity=k & 3)
        luma, reg = synth.capture(f, grey, 1280, 720, H=synth.warp(f, 1280, 720, rng) if k % 2 else None, sigma=2.0 + 4.0 * (k % 3 == 2), rng=rng)
        lumas.append(luma)
        regs.append(reg)
    return np.stack(lumas), np.stack(regs)


def test_front_matches_the_batched_finish():
    luma, reg = frames(12)
    want = lz.Receiver(384, 64, 128, max_frames=12).finish_luma(luma, reg, grid=False)
    got, released = {}, []

    def on_frame(tag, ts, verified, ok, its):
        got[tag] = (ts, verified, ok, its)

    fr = lz.FrontReceiver(384, 64, 128, 1280, 720, batch_cap=5, slots=64, on_frame=on_frame, on_release=released.append)
    order = [k % 12 for k in range(40)]
    for i, k in enumerate(order):
        fr.push(luma[k], ts_ns=1000000 * i, tag=i, reg=reg[k])
        assert released[-1] == i, "release(tag) comes before push returns"
    assert fr.flush() == 40
    assert sorted(released) == list(range(40))
    for i, k in enumerate(order):
        ts, verified, ok, its = got[i]
        assert ts == 1000000 * i
        assert np.array_equal(ok, want["ok"][k]) and np.array_equal(its, want["its"][k])
        assert verified == want["blocks"][k][want["ok"][k] > 0].tobytes()
    st = fr.stats()
    assert st["framesIn"] == 40 and st["decoded"] == 40 and st["dropped"] == 0 and st["batches"] >= 8 and st["B"] <= 5
    s = fr.series()
    assert s[0] == 4 and s.size == 1 + 8 * 40
    rows = s[1:].reshape(40, 8)
    assert np.array_equal(rows[:, 1], [int(want["ok"][k].sum()) for k in order])
    assert (rows[:, 3] == 1).all()
    fr.close()


def test_front_drops_and_counts_when_every_slot_waits():
    luma, reg = frames(4, seed=40)
    released, seen = [], []
    fr = lz.FrontReceiver(384, 64, 128, 1280, 720, batch_cap=1, slots=2, on_frame=lambda tag, *a: seen.append(tag), on_release=released.append)
    for i in range(60):
        fr.push(luma[i % 4], ts_ns=i, tag=i, reg=reg[i % 4])
    fr.flush()
    st = fr.stats()
    assert sorted(released) == list(range(60))
    assert st["framesIn"] == 60 and st["decoded"] + st["dropped"] == 60 and st["decoded"] == len(seen)
    fr.close()


def test_host_finish_matches_device_finish():
    luma, reg = frames(6, seed=50)
    rx = lz.Receiver(384, 64, 128, max_frames=6)
    want = rx.finish_luma(luma, reg, grid=False)
    blocks, ok, its, v = rx.finish_luma_host(luma, reg)
    assert np.array_equal(ok, want["ok"]) and np.array_equal(its, want["its"]) and v == int(want["ok"].sum())
    assert np.array_equal(blocks[ok > 0], want["blocks"][ok > 0])
    # a smaller call after a larger one reuses the handle's buffers
    b1, ok1, its1, _ = rx.finish_luma_host(luma[2:3], reg[2:3])
    assert np.array_equal(ok1[0], want["ok"][2]) and np.array_equal(its1[0], want["its"][2])
