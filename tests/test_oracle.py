"""The oracle pinned: against the reference's recorded hashes and check values, the SPEC 7.4 vectors, the golden
decodes the reference made (tests/golden/ldpc_ref.npz), and, where it was built here, the reference itself."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
SPEC = json.load(open(os.path.join(GOLD, "spec_7_4.json")))
SHAPE = {6: (4608, 3968, 4480), 4: (5120, 3840, 5120), 3: (5760, 3840, 5760), 2: (7680, 3840, 7680)}


def spec_block(b):
    blk = bytes([b, 0, 0, 0]) + bytes(j & 255 for j in range(472))
    return blk


def hexbits(bits):
    return np.packbits(np.asarray(bits, np.uint8)).tobytes().hex()


@pytest.mark.parametrize("rate", [6, 4, 3, 2])
def test_h_hash(rate):
    assert "%08x" % oracle.h_hash(rate) == SPEC["h_hash"][str(rate)]


def test_crc_check_value():
    assert "%08X" % oracle.crc32c(b"123456789") == SPEC["crc_check_value"]["crc32c"]


def test_crc_random_against_bit_loop():
    rng = np.random.default_rng(5)
    for n in [0, 1, 7, 8, 9, 15, 16, 476, 600]:
        b = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        c = 0xFFFFFFFF
        for x in b:
            c ^= x
            for _ in range(8):
                c = (c >> 1) ^ (0x82F63B78 if c & 1 else 0)
        assert oracle.crc32c(b) == c ^ 0xFFFFFFFF


@pytest.mark.parametrize("blk", SPEC["blocks"], ids=lambda b: "block%d" % b["b"])
def test_spec_7_4_codeword(blk):
    rate = blk["rate"]
    n, k, nt = SHAPE[rate]
    data = spec_block(blk["b"])
    crc = oracle.crc32c(data)
    assert "%08X" % crc == blk["crc"]
    info = np.unpackbits(np.frombuffer(data + crc.to_bytes(4, "big"), np.uint8))
    d = np.zeros(k, np.uint8)
    d[:3840] = info
    cw = oracle.ldpc_encode(rate, d)
    assert hexbits(cw[3800:3840]) == blk["bits_3800_3839"]
    assert not cw[3840:k].any()
    if rate == 6:
        assert hexbits(cw[k:k + 128]) == blk["parity_0_127"]
    # SPEC 7.4's parity prefixes for the 3/4, 2/3 and 1/2 blocks predate the codes the reference now ships (its own
    # encoder, oracle/_ref, does not give them either; the 7/8 ones it does). Those codes are pinned by their H
    # hashes above and by the encoder test against the reference below.
    # The per-codeword SHA-256 lines of SPEC 7.4 are not reproduced by the reference's own encoder either (checked
    # against oracle/_ref: the CRCs, bits 3800-3839 and parity prefixes agree, the digests do not), so they pin
    # nothing; the frame-level slot digest, which the reference's own vectors test checks, is pinned instead.


def _golden():
    return np.load(os.path.join(GOLD, "ldpc_ref.npz"))


@pytest.mark.parametrize("tag,mi,si,ratio", [("stall", 20, 9, 0.95), ("plain", 30, 0, 0.0)])
def test_oracle_matches_reference_golden(tag, mi, si, ratio):
    g = _golden()
    at = bat = 0
    for i, rate in enumerate(g["rates"]):
        n = SHAPE[int(rate)][0]
        its, out = oracle.ldpc_decode(int(rate), g["llr"][at:at + n], mi, si, ratio)
        assert its == g["its_" + tag][i], "codeword %d rate %d" % (i, rate)
        assert np.array_equal(np.packbits(out), g["bits_" + tag][bat:bat + n // 8]), "codeword %d" % i
        at += n
        bat += n // 8


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")
def test_oracle_batch_matches_reference_batch():
    """The port and the reference on a fresh seeded mixed-rate batch across the Eb/N0 sweep, every bit and return."""
    from lizard_gb300_testing import synth
    b = synth.ldpc_batch(600, seed=11)
    for mi, si, ratio in [(20, 9, 0.95), (30, 9, 0.95), (12, 0, 0.0)]:
        pb, pi, po = oracle.ldpc_batch(oracle.port(), b["llr"], b["offsets"], b["rates"], mi, si, ratio, threads=8)
        rb, ri, ro = oracle.ldpc_batch(oracle.ref(), b["llr"], b["offsets"], b["rates"], mi, si, ratio, threads=8)
        assert np.array_equal(pi, ri)
        assert np.array_equal(pb, rb)
        assert np.array_equal(po, ro)


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")
@pytest.mark.parametrize("rate", [6, 4, 3, 2])
def test_encoder_matches_reference(rate):
    n, k, nt = SHAPE[rate]
    rng = np.random.default_rng(rate)
    for _ in range(20):
        d = rng.integers(0, 2, k).astype(np.uint8)
        cw = np.zeros(n, np.uint8)
        oracle.ref().ref_ldpc_encode(rate, oracle._p(d), oracle._p(cw))
        assert np.array_equal(cw, oracle.ldpc_encode(rate, d))
