"""Synthetic inputs shaped like the reference's own test channels (no dataset exists for this path).

LDPC batch: 476-byte blocks (4-byte id, 472 seeded random payload bytes) with their CRC-32C appended MSB first
(liblizard/src/lizard_phy.c:1120-1131), the 7/8 code's 128 extra data bits zero, encoded by the format's codes;
BPSK over AWGN at a given Eb/N0 with R = 3840 / nt; LLR = 2 y / sigma^2 in float; int8 = round-half-even(8 LLR)
clipped to +-80 (the receiver's soft stage, liblizard/test/ldpc_awgn.c:67-78, liblizard/test/ldpc_ref.h:41-42);
the 7/8 code's never-sent bits fed as known zeros, +127 (liblizard/src/lizard_phy.c:1823).
"""
import numpy as np

from . import BLOCK_BYTES, CODE_K, CODE_N, CODE_NT, INFO_BITS, crc32c, ldpc_encode_many

# Rate mix of the batch by count (the format's profile: 39% 7/8, 26% 3/4, 15% 2/3, 20% 1/2) and the Eb/N0 sweep.
MIX = ((6, 0.39), (4, 0.26), (3, 0.15), (2, 0.20))
EBN0_SWEEP_DB = (1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0)


def mixed_rates(count, seed=0):
    """count rate indices in the profile's proportions (floor of each share, the 1/2 tier takes the rest), shuffled."""
    n = [int(count * f) for _, f in MIX[:-1]]
    n.append(count - sum(n))
    rates = np.concatenate([np.full(k, r, np.int32) for (r, _), k in zip(MIX, n)])
    np.random.default_rng(seed).shuffle(rates)
    return rates


def blocks(count, seed=0):
    """count 480-byte rows: block id (uint32 LE), 472 random bytes, CRC-32C of the 476 big-endian."""
    rng = np.random.default_rng(seed + 1)
    b = np.zeros((count, BLOCK_BYTES + 4), np.uint8)
    b[:, :4] = np.arange(count, dtype="<u4").view(np.uint8).reshape(count, 4)
    b[:, 4:BLOCK_BYTES] = rng.integers(0, 256, (count, BLOCK_BYTES - 4), dtype=np.uint8)
    for i in range(count):
        c = crc32c(b[i, :BLOCK_BYTES].tobytes())
        b[i, BLOCK_BYTES:] = (c >> 24) & 255, (c >> 16) & 255, (c >> 8) & 255, c & 255
    return b


def ldpc_batch(count, seed=0, ebn0_db=EBN0_SWEEP_DB, rates=None):
    """The LDPC batch. Codeword i runs at ebn0_db[i % len(ebn0_db)]. Returns a dict: rates, offsets, llr (flat int8,
    codewords back to back), codewords (flat uint8 bits), blocks (count x 480) and ebn0 (per codeword)."""
    rates = mixed_rates(count, seed) if rates is None else np.asarray(rates, np.int32)
    count = rates.size
    n = np.array([CODE_N[int(r)] for r in rates], np.int64)
    off = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    blk = blocks(count, seed)
    bits = np.unpackbits(blk, axis=1)          # 3840 information bits, MSB first
    ebn0 = np.asarray(ebn0_db, np.float64)[np.arange(count) % len(ebn0_db)]
    llr = np.empty(int(n.sum()), np.int8)
    cws = np.empty(int(n.sum()), np.uint8)
    rng = np.random.default_rng(seed + 2)
    for r in np.unique(rates):
        r = int(r)
        idx = np.nonzero(rates == r)[0]
        k, nn, nt = CODE_K[r], CODE_N[r], CODE_NT[r]
        data = np.zeros((idx.size, k), np.uint8)
        data[:, :INFO_BITS] = bits[idx]
        cw = ldpc_encode_many(r, data)
        R = INFO_BITS / nt
        sigma = np.sqrt(1.0 / (2.0 * R * 10.0 ** (ebn0[idx] / 10.0)))[:, None]
        y = (1.0 - 2.0 * cw) + sigma * rng.standard_normal(cw.shape, dtype=np.float32)
        fl = (2.0 * y / (sigma * sigma)).astype(np.float32)
        q = np.clip(np.rint(8.0 * fl.astype(np.float64)), -80, 80).astype(np.int8)
        if nt < nn:   # the 7/8 code's never-sent data column: known zeros
            q[:, k - (nn - nt):k] = 127
        for j, i in enumerate(idx):
            llr[off[i]:off[i] + nn] = q[j]
            cws[off[i]:off[i] + nn] = cw[j]
    return {"rates": rates, "offsets": off, "llr": llr, "codewords": cws, "blocks": blk, "ebn0": ebn0}
