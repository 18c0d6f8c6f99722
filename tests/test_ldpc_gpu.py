"""LDPC + CRC-32C on the GPU, through the C ABI, held bit for bit to the reference (its golden decodes) and to the
oracle (seeded batches across the Eb/N0 sweep, edge cases), and at the benchmark's full size by properties."""
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    return np.load(os.path.join(GOLD, "ldpc_ref.npz"))


@pytest.mark.parametrize("tag,mi,si,ratio", [("stall", 20, 9, 0.95), ("plain", 30, 0, 0.0)])
def test_batch_matches_reference_golden(tag, mi, si, ratio):
    g = golden()
    plan = lz.LdpcPlan(g["rates"], mi, si, ratio)
    bits, its, ok = plan.run(g["llr"])
    assert np.array_equal(its, g["its_" + tag])
    assert np.array_equal(bits, g["bits_" + tag])


def test_single_codeword_entry_matches_reference_golden():
    g = golden()
    at = 0
    for i, rate in enumerate(g["rates"][:12]):
        n = lz.CODE_N[int(rate)]
        its, out = lz.ldpc_decode_stall(int(rate), g["llr"][at:at + n], 20, 9, 0.95)
        assert its == g["its_stall"][i]
        assert np.array_equal(np.packbits(out), g["bits_stall"][at // 8:(at + n) // 8])
        at += n


def check_against_oracle(b, mi=20, si=9, ratio=0.95):
    plan = lz.LdpcPlan(b["rates"], mi, si, ratio)
    bits, its, ok = plan.run(b["llr"])
    ob, oi, oo = oracle.ldpc_batch(oracle.port(), b["llr"], b["offsets"], b["rates"], mi, si, ratio, threads=os.cpu_count() or 4)
    bad = np.nonzero(oi != its)[0]
    assert bad.size == 0, "iterations differ at %s: gpu %s oracle %s" % (bad[:8], its[bad[:8]], oi[bad[:8]])
    assert np.array_equal(bits, ob)
    assert np.array_equal(ok, oo)
    return bits, its, ok


@pytest.mark.parametrize("seed", [1, 2])
def test_seeded_sweep_matches_oracle(seed):
    b = synth.ldpc_batch(3000, seed=seed)
    bits, its, ok = check_against_oracle(b)
    # the sweep spans failing and clean codewords
    assert (its == -1).any() or (its == -3).any()
    assert (its > 0).any() and ok[its > 0].all()


@pytest.mark.parametrize("mi,si,ratio", [(1, 0, 0.0), (2, 2, 0.95), (30, 0, 0.0), (9, 9, 0.5), (255, 9, 0.95)])
def test_decoder_settings_match_oracle(mi, si, ratio):
    b = synth.ldpc_batch(400, seed=7)
    check_against_oracle(b, mi, si, ratio)


@pytest.mark.parametrize("count", [1, 2, 5, 9, 10, 31])
def test_small_and_ragged_batches(count):
    b = synth.ldpc_batch(count, seed=count, rates=synth.mixed_rates(count, seed=count))
    check_against_oracle(b)


def test_extreme_llrs_match_oracle():
    rng = np.random.default_rng(9)
    rates, parts = [], []
    for r in lz.RATES:
        n = lz.CODE_N[r]
        for pat in (np.full(n, -128), np.full(n, 127), np.zeros(n), np.tile([127, -128], n // 2),
                    rng.integers(-128, 128, n), rng.integers(-2, 3, n)):
            rates.append(r)
            parts.append(np.asarray(pat, np.int8))
    rates = np.array(rates, np.int32)
    llr = np.concatenate(parts)
    off = np.concatenate([[0], np.cumsum([lz.CODE_N[int(r)] for r in rates])[:-1]]).astype(np.int64)
    for mi, si in [(20, 9), (30, 0)]:
        check_against_oracle({"rates": rates, "llr": llr, "offsets": off}, mi, si, 0.95)


def test_device_entry_on_a_side_stream_matches_host_entry():
    torch = pytest.importorskip("torch")
    b = synth.ldpc_batch(1000, seed=3)
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    hb, hi, ho = plan.run(b["llr"])
    s = torch.cuda.Stream()
    d_llr = torch.from_numpy(b["llr"]).cuda()
    d_bits = torch.empty(plan.llr_bytes // 8, dtype=torch.uint8, device="cuda")
    d_its = torch.empty(plan.count, dtype=torch.int32, device="cuda")
    d_ok = torch.empty(plan.count, dtype=torch.uint8, device="cuda")
    s.wait_stream(torch.cuda.current_stream())
    for _ in range(2):   # the second run reuses the plan's counters
        plan.run_dev(d_llr.data_ptr(), d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), s.cuda_stream)
    s.synchronize()
    assert np.array_equal(d_bits.cpu().numpy(), hb)
    assert np.array_equal(d_its.cpu().numpy(), hi)
    assert np.array_equal(d_ok.cpu().numpy(), ho)
    assert plan.launches == 4


@pytest.mark.parametrize("chunks", [1, 2, 7, 16])
def test_chunked_host_entry_matches_device_entry(chunks):
    """The host-memory entry pipelines the batch over chunks of consecutive codewords: the outputs are those of the
    one-pass device entry, from pageable and from pinned host memory."""
    torch = pytest.importorskip("torch")
    b = synth.ldpc_batch(1000, seed=4)
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    d_llr = torch.from_numpy(b["llr"]).cuda()
    d_bits = torch.empty(plan.llr_bytes // 8, dtype=torch.uint8, device="cuda")
    d_its = torch.empty(plan.count, dtype=torch.int32, device="cuda")
    d_ok = torch.empty(plan.count, dtype=torch.uint8, device="cuda")
    plan.run_dev(d_llr.data_ptr(), d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    want = d_bits.cpu().numpy(), d_its.cpu().numpy(), d_ok.cpu().numpy()
    assert plan.set_chunks(chunks) == chunks
    got = plan.run(b["llr"])
    assert plan.launches >= chunks and plan.transfer == 0
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    pinned = [torch.empty(n, dtype=t).pin_memory() for n, t in
              ((plan.llr_bytes, torch.int8), (plan.llr_bytes // 8, torch.uint8), (plan.count, torch.int32), (plan.count, torch.uint8))]
    pinned[0].copy_(torch.from_numpy(b["llr"]))
    for in_place in (0, 1):
        for t in pinned[1:]:
            t.fill_(0x5A)
        plan.set_transfer(in_place)
        got = plan.run(*(t.numpy() for t in pinned))
        assert plan.transfer == in_place
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
    # page-locked but 8 bytes off a 16-byte boundary: the decoder cannot read it in place, so the batch is staged
    big = torch.empty(plan.llr_bytes + 32, dtype=torch.int8).pin_memory()
    off = (-big.data_ptr()) % 16 + 8
    llr8 = big.numpy()[off:off + plan.llr_bytes]
    llr8[:] = b["llr"]
    plan.set_transfer(1)
    got = plan.run(llr8, *(t.numpy() for t in pinned[1:]))
    assert plan.transfer == 0
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("rates", [[6, 2], [2, 6, 2], [6, 6, 6, 2]])
def test_every_chunk_holds_a_codeword(rates):
    """Chunks split at codeword boundaries by bytes: with a large last codeword no offset reaches the last targets,
    yet each chunk keeps a codeword and the outputs are those of one pass."""
    b = synth.ldpc_batch(len(rates), seed=8, rates=np.array(rates, np.int32))
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    want = plan.run(b["llr"])
    for k in range(2, len(rates) + 1):
        assert plan.set_chunks(k) == k
        got = plan.run(b["llr"])
        assert plan.launches >= k
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_registered_host_buffers_are_read_in_place():
    """Buffers the caller already owns, page-locked with cudaHostRegister, take the in-place route too."""
    torch = pytest.importorskip("torch")
    b = synth.ldpc_batch(500, seed=6)
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    want = plan.run(b["llr"])
    assert plan.transfer == 0
    page = 1 << 16   # the largest page size a host may use: each buffer gets pages of its own

    def own_pages(n, dtype):
        nbytes = n * np.dtype(dtype).itemsize
        raw = np.zeros(nbytes + 2 * page, np.uint8)
        at = (-raw.ctypes.data) % page
        return raw[at:at + nbytes].view(dtype)

    bufs = [own_pages(plan.llr_bytes, np.int8), own_pages(plan.llr_bytes // 8, np.uint8), own_pages(plan.count, np.int32),
            own_pages(plan.count, np.uint8)]
    bufs[0][:] = b["llr"]
    rt = torch.cuda.cudart()
    done = []
    try:
        for a in bufs:
            assert int(rt.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) == 0
            done.append(a)
        got = plan.run(*bufs)
        assert plan.transfer == 1
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
    finally:
        for a in done:
            rt.cudaHostUnregister(a.ctypes.data)


def test_full_size_batch_properties():
    """The benchmark's batch (65,536 codewords): every decoded block is its sent codeword and passes its CRC, the
    CRC flags agree with a host CRC of the output, clean-channel codewords all decode, and a sample matches the oracle."""
    b = synth.ldpc_batch(65536, seed=0)
    plan = lz.LdpcPlan(b["rates"], 20, 9, 0.95)
    bits, its, ok = plan.run(b["llr"])
    truth = np.packbits(b["codewords"])
    for i in np.nonzero(its > 0)[0][::97]:
        o, n = int(b["offsets"][i]) // 8, lz.CODE_N[int(b["rates"][i])] // 8
        assert np.array_equal(bits[o:o + n], truth[o:o + n])
    for i in range(0, 65536, 331):
        o = int(b["offsets"][i]) // 8
        blk = bits[o:o + 480]
        assert ok[i] == (lz.crc32c(blk[:476].tobytes()) == int.from_bytes(blk[476:480].tobytes(), "big"))
    hi = b["ebn0"] >= 4.0
    assert (its[hi & (b["rates"] != 6)] > 0).mean() > 0.99
    sub = {k: v for k, v in synth.ldpc_batch(512, seed=0).items()}
    check_against_oracle(sub)


@pytest.mark.parametrize("rate", [6, 4, 3, 2])
def test_every_variant_decodes_alike(rate):
    """Each kernel variant (warps a codeword, layer form) gives the oracle's decodes bit for bit."""
    b = synth.ldpc_batch(600, seed=40 + rate, rates=np.full(600, rate, np.int32))
    ob, oi, oo = oracle.ldpc_batch(oracle.port(), b["llr"], b["offsets"], b["rates"], 20, 9, 0.95, threads=os.cpu_count() or 4)
    try:
        for v in range(lz.ldpc_variants(rate)):
            lz.ldpc_set_variant(rate, v)
            assert lz.ldpc_variant(rate)[0] == v
            bits, its, ok = lz.LdpcPlan(b["rates"], 20, 9, 0.95).run(b["llr"])
            assert np.array_equal(its, oi), "variant %d" % v
            assert np.array_equal(bits, ob) and np.array_equal(ok, oo), "variant %d" % v
    finally:
        lz.ldpc_set_variant(rate, 0)


def test_autotune_keeps_a_variant_and_decodes_alike():
    try:
        ch = lz.ldpc_autotune(256, (1.5, 3.0))
        assert [lz.ldpc_variant(r)[0] for r in (6, 4, 3, 2)] == ch
        for c, r in zip(ch, (6, 4, 3, 2)):
            assert 0 <= c < lz.ldpc_variants(r)
        check_against_oracle(synth.ldpc_batch(1500, seed=77))
    finally:
        for r in (6, 4, 3, 2):
            lz.ldpc_set_variant(r, 0)
