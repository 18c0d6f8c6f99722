"""The allocation-free batch decode (lizg_ldpc_decode_noalloc), for callers that cannot allocate device memory (a
plug-in inside a host application that owns the device allocator). Called through the C ABI on two calls in a row,
with different batches, each held bit for bit to the plan API's decode of the same batch and to the oracle's
decoder; a batch mixing in rates that have no code (those codewords get its = -4, ok = 0 and no share of the LLR
layout) decodes the rest as the plan decodes them alone; sizes past its fixed scratch are refused. This file is
collected last on purpose: a run that stops at the first failure has run every other test before it. It passes
alone in a fresh process as well as after the rest."""
import ctypes

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

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
        ob, oi, oo = oracle.ldpc_batch(oracle.port(), b["llr"], b["offsets"], b["rates"], 20, 9, 0.95, threads=8)
        assert np.array_equal(d_its.cpu().numpy(), oi) and np.array_equal(d_bits.cpu().numpy(), ob) and np.array_equal(d_ok.cpu().numpy(), oo), \
            "call %d: differs from the oracle" % call


def test_noalloc_rates_without_a_code():
    """Codewords whose rate index has no code (5, 0, 9) among valid ones: its = -4, ok = 0, no share of the LLR or bit
    layout; the others decoded as the plan decodes the valid codewords alone (whose offsets close up the gaps)."""
    torch = pytest.importorskip("torch")
    lib = lz.lib()
    fn = noalloc(lib)
    b = synth.ldpc_batch(1500, seed=23)
    rng = np.random.default_rng(5)
    count = 1600
    bad = np.sort(rng.choice(count, count - 1500, replace=False))
    valid = np.setdiff1d(np.arange(count), bad)
    rates = np.empty(count, np.int32)
    rates[valid] = b["rates"]
    rates[bad] = rng.choice([5, 0, 9], bad.size).astype(np.int32)
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    want_bits, want_its, want_ok = plan.run(b["llr"])
    d_llr = torch.from_numpy(b["llr"]).cuda()
    d_rate = torch.from_numpy(rates).cuda()
    d_bits = torch.full((plan.llr_bytes // 8,), 0xAA, dtype=torch.uint8, device="cuda")
    d_its = torch.full((count,), 99, dtype=torch.int32, device="cuda")
    d_ok = torch.full((count,), 7, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    assert fn(d_llr.data_ptr(), d_rate.data_ptr(), count, 20, 9, 0.95, d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), s.cuda_stream) == 0
    torch.cuda.synchronize()
    its, ok = d_its.cpu().numpy(), d_ok.cpu().numpy()
    assert (its[bad] == -4).all() and (ok[bad] == 0).all()
    assert np.array_equal(its[valid], want_its) and np.array_equal(ok[valid], want_ok)
    assert np.array_equal(d_bits.cpu().numpy(), want_bits)


def test_noalloc_refuses_sizes_past_its_scratch():
    torch = pytest.importorskip("torch")
    lib = lz.lib()
    fn = noalloc(lib)
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    assert fn(d.data_ptr(), d.data_ptr(), 8193, 20, 9, 0.95, d.data_ptr(), d.data_ptr(), d.data_ptr(), None) == -1
    assert b"8192" in lib.lizg_last_error()
    assert fn(d.data_ptr(), d.data_ptr(), 0, 20, 9, 0.95, d.data_ptr(), d.data_ptr(), d.data_ptr(), None) == -1
