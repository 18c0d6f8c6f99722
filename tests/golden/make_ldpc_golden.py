"""Generates tests/golden/ldpc_ref.npz: LDPC decodes by the reference itself (its C decoder compiled from its
sources by oracle/Makefile), so the GPU decoder can be held to the reference's own outputs on a GPU host where the
reference tree is absent.

Run from the repo root where the reference is present: python tests/golden/make_ldpc_golden.py
Cases, for each of the four codes: codewords through BPSK/AWGN at Eb/N0 from 0.5 to 4.5 dB (the receiver's int8
quantiser, +-80), a clean codeword, all-zero LLRs, and uniform random int8 over the whole range (-128 included).
Each is decoded twice: max 20 iterations with the stall rule (9, 0.95) and max 30 without it.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

RATES = (6, 4, 3, 2)
SHAPE = {6: (4608, 3968, 4480), 4: (5120, 3840, 5120), 3: (5760, 3840, 5760), 2: (7680, 3840, 7680)}


def main():
    oracle.build(ref=True)
    R = oracle.ref()
    if R is None:
        raise SystemExit("the reference could not be built here")
    rng = np.random.default_rng(20261203)
    rates, llrs = [], []
    for rate in RATES:
        n, k, nt = SHAPE[rate]
        for ebn0 in (0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0, 4.5):
            data = rng.integers(0, 2, k).astype(np.uint8)
            data[3840:] = 0
            cw = oracle.ldpc_encode(rate, data)
            sigma = np.sqrt(1.0 / (2.0 * (3840.0 / nt) * 10 ** (ebn0 / 10)))
            y = (1.0 - 2.0 * cw) + sigma * rng.standard_normal(n)
            q = np.clip(np.rint(8.0 * (2 * y / sigma ** 2).astype(np.float32).astype(np.float64)), -80, 80).astype(np.int8)
            if nt < n:
                q[k - (n - nt):k] = 127
            rates.append(rate); llrs.append(q)
        data = rng.integers(0, 2, k).astype(np.uint8)
        data[3840:] = 0
        cw = oracle.ldpc_encode(rate, data)
        rates.append(rate); llrs.append(np.where(cw == 1, -80, 80).astype(np.int8))
        rates.append(rate); llrs.append(np.zeros(n, np.int8))
        rates.append(rate); llrs.append(rng.integers(-128, 128, n).astype(np.int8))
    rates = np.array(rates, np.int32)
    out = {"rates": rates, "llr": np.concatenate(llrs)}
    for tag, (mi, si, ratio) in {"stall": (20, 9, 0.95), "plain": (30, 0, 0.0)}.items():
        its, bits = [], []
        for rate, q in zip(rates, llrs):
            n = SHAPE[int(rate)][0]
            o = np.zeros(n, np.uint8)
            it = np.zeros(1, np.int32)
            R.ref_ldpc_decode_many(int(rate), oracle._p(q), 1, oracle._p(o), oracle._p(it), mi, si, ratio)
            its.append(int(it[0])); bits.append(np.packbits(o))
        out["its_" + tag] = np.array(its, np.int32)
        out["bits_" + tag] = np.concatenate(bits)
    path = os.path.join(ROOT, "tests", "golden", "ldpc_ref.npz")
    np.savez_compressed(path, **out)
    print(path, {k: v.shape for k, v in out.items()}, "stall its:", out["its_stall"].tolist())


if __name__ == "__main__":
    main()
