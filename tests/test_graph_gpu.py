"""The captured per-frame pipeline (lizg_rx_finish_luma_graph): replays give the direct call's results, and a replay
after the input buffers' contents change decodes the new frames (the graph reads the buffers, not copies)."""
import ctypes

import numpy as np
import pytest

import lizard_gb300 as lz
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu


def test_graph_replays_match_direct_calls():
    torch = pytest.importorskip("torch")
    rx = lz.Receiver(384, 64, 128, max_frames=2)
    f = rx.fmt
    frames = []
    for seed in (3, 4, 5, 6):
        rng = np.random.default_rng(seed)
        blocks = synth.random_blocks(f.blocks, seed)
        luma, reg = synth.capture(f, synth.picture(f, blocks, parity=seed & 3), 1280, 720, H=synth.warp(f, 1280, 720, rng), sigma=2.0, rng=rng)
        frames.append((luma, reg, blocks))
    L = lz.lib()
    d_l = torch.zeros((2, 720, 1280), dtype=torch.uint8, device="cuda")
    d_r = torch.zeros((2, frames[0][1].size), dtype=torch.float32, device="cuda")
    o, s = rx._outputs(2, torch, keep=True)
    st = torch.cuda.current_stream().cuda_stream
    for call, pair in enumerate([(0, 1), (2, 3), (1, 0)]):
        d_l.copy_(torch.from_numpy(np.stack([frames[i][0] for i in pair])))
        d_r.copy_(torch.from_numpy(np.stack([frames[i][1] for i in pair])))
        rc = L.lizg_rx_finish_luma_graph(rx._h, ctypes.c_void_p(d_l.data_ptr()), 1280, 720, 1280, 720 * 1280, ctypes.c_void_p(d_r.data_ptr()), 2,
                                         ctypes.byref(s), None, None, ctypes.c_void_p(st))
        assert rc == 0, L.lizg_last_error()
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy().copy() for k, v in o.items()}
        want = rx.finish_luma(np.stack([frames[i][0] for i in pair]), np.stack([frames[i][1] for i in pair]), grid=False)
        for k in ("blocks", "ok", "its", "llrf", "align"):
            assert np.array_equal(got[k], want[k]), (call, k)
        for j, i in enumerate(pair):
            assert got["ok"][j].all() and np.array_equal(got["blocks"][j], frames[i][2])
