"""The allocation-free batch decode (lizg_ldpc_decode_noalloc), for callers that cannot allocate device memory (a
plug-in inside a host application that owns the device allocator). Called through the C ABI on two calls in a row,
with different batches, each held bit for bit to the plan API's decode of the same batch; sizes past its fixed
scratch are refused. This file is collected last on purpose: a run that stops at the first failure has run every
other test before it. It passes alone in a fresh process as well as after the rest."""
import ctypes

import numpy as np
import pytest

import lizard_gb300 as lz
from lizard_gb300 import synth

pytestmark = pytest.mark.gpu


def noalloc(lib):
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    fn = lib.lizg_ldpc_decode_noalloc
    fn.argtypes = [P, P, I, I, I, F, P, P, P, P]
    return fn


def test_noalloc_matches_plan_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = lz.lib()
    fn = noalloc(lib)
    maximum = 8192
    for call, (count, seed) in enumerate([(3000, 21), (maximum, 22)]):
        b = synth.ldpc_batch(count, seed=seed)
        plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
        want_bits, want_its, want_ok = plan.run(b["llr"])
        d_llr = torch.from_numpy(b["llr"]).cuda()
        d_rate = torch.from_numpy(b["rates"]).cuda()
        d_bits = torch.full((plan.llr_bytes // 8,), 0xAA, dtype=torch.uint8, device="cuda")
        d_its = torch.full((count,), 99, dtype=torch.int32, device="cuda")
        d_ok = torch.full((count,), 7, dtype=torch.uint8, device="cuda")
        s = torch.cuda.current_stream()
        rc = fn(d_llr.data_ptr(), d_rate.data_ptr(), count, 20, 9, 0.95, d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), s.cuda_stream)
        assert rc == 0, lib.lizg_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(d_its.cpu().numpy(), want_its), "call %d: iterations differ" % call
        assert np.array_equal(d_bits.cpu().numpy(), want_bits), "call %d: hard bits differ" % call
        assert np.array_equal(d_ok.cpu().numpy(), want_ok), "call %d: CRC verdicts differ" % call


def test_noalloc_refuses_sizes_past_its_scratch():
    torch = pytest.importorskip("torch")
    lib = lz.lib()
    fn = noalloc(lib)
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    assert fn(d.data_ptr(), d.data_ptr(), 8193, 20, 9, 0.95, d.data_ptr(), d.data_ptr(), d.data_ptr(), None) == -1
    assert b"8192" in lib.lizg_last_error()
    assert fn(d.data_ptr(), d.data_ptr(), 0, 20, 9, 0.95, d.data_ptr(), d.data_ptr(), d.data_ptr(), None) == -1
