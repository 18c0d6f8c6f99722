"""The C ABI without a GPU: the library loads, exports every function include/*.h declares, its host-side
functions agree with the oracle, and device entry points fail loudly (an error code and message, no fallback)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from conftest import ROOT, gpu_available


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"//.*", "", open(h).read())
        for m in re.finditer(r"\b(liz[g]?_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 10
    lib = ctypes.CDLL(lz.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_no_error():
    assert b"sm_103a" in lz.lib().lizg_version()


@pytest.mark.parametrize("rate", [6, 4, 3, 2])
def test_host_encoder_matches_oracle(rate):
    rng = np.random.default_rng(rate + 10)
    k = lz.CODE_K[rate]
    for _ in range(5):
        d = rng.integers(0, 2, k).astype(np.uint8)
        assert np.array_equal(lz.ldpc_encode(rate, d), oracle.ldpc_encode(rate, d))
    many = rng.integers(0, 2, (4, k)).astype(np.uint8)
    cw = lz.ldpc_encode_many(rate, many)
    for i in range(4):
        assert np.array_equal(cw[i], oracle.ldpc_encode(rate, many[i]))


def test_host_crc_matches_oracle():
    rng = np.random.default_rng(3)
    assert lz.crc32c(b"123456789") == 0xE3069283
    for n in [0, 1, 5, 476, 1000]:
        b = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        assert lz.crc32c(b) == oracle.crc32c(b)


def test_bad_arguments_are_errors():
    assert lz.lib().lizg_ldpc_n(5) == 0
    assert lz.lib().lizg_ldpc_plan_set_chunks(None, 2) == -1
    assert lz.lib().lizg_ldpc_plan_set_transfer(None, 1) == -1 and lz.lib().lizg_ldpc_plan_transfer(None) == -1
    with pytest.raises(lz.LizgError):
        lz.ldpc_encode(5, np.zeros(3840, np.uint8))
    with pytest.raises(lz.LizgError):
        lz.LdpcPlan(np.array([6, 7], np.int32))
    with pytest.raises(lz.LizgError):
        lz.LdpcPlan(np.array([6], np.int32), max_iter=0)
    with pytest.raises(lz.LizgError):
        lz.ldpc_variants(5)
    with pytest.raises(lz.LizgError):
        lz.ldpc_set_variant(6, 99)
    with pytest.raises(lz.LizgError):
        lz.ldpc_autotune(0)
    with pytest.raises(lz.LizgError):
        lz.fmt_geometry(200)
    P = ctypes.c_void_p(8)
    assert lz.lib().lizg_fmt_read_dev(300, P, 64, 64, 4096, P, 4000, 1, None, P, None) == -1
    assert lz.lib().lizg_fmt_read_dev(256, P, 64, 64, 4096, P, 20, 1, None, P, None) == -1   # reg_stride short
    assert lz.lib().lizg_fmt_read_dev(256, P, 1, 64, 4096, P, 4000, 1, None, P, None) == -1    # frame under 2 x 2
    assert lz.lib().lizg_fmt_decode_dev(128, None, 1, P, None) == -1


def test_fmt_geometry_matches_oracle():
    """The format word's cells and bytes a ring, as the reference's fmt.c computes them (through the oracle)."""
    import oracle
    for span in (128, 256, 512):
        side = span + 30
        assert lz.fmt_geometry(span) == (oracle.port().orc_fmt_side_cells(side, 15), oracle.port().orc_fmt_bytes(side, 15))


def test_decoder_variants_listed():
    assert [lz.ldpc_variants(r) for r in (6, 4, 3, 2)] == [6, 6, 5, 5]


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly():
    with pytest.raises(lz.LizgError) as e:
        lz.LdpcPlan(np.array([6, 4], np.int32))
    assert "cuda" in str(e.value).lower() or "device" in str(e.value).lower()
    with pytest.raises(lz.LizgError):
        lz.Engine()


def test_synth_batch_shapes():
    from lizard_gb300_testing import synth
    b = synth.ldpc_batch(40, seed=1)
    n = sum(lz.CODE_N[int(r)] for r in b["rates"])
    assert b["llr"].size == n and b["offsets"][0] == 0
    counts = {r: int((b["rates"] == r).sum()) for r in lz.RATES}
    assert counts == {6: 15, 4: 10, 3: 6, 2: 9}
    # the codewords satisfy their code: re-encoding the data part gives the same parity
    for i in range(3):
        r, o = int(b["rates"][i]), int(b["offsets"][i])
        cw = b["codewords"][o:o + lz.CODE_N[r]]
        assert np.array_equal(oracle.ldpc_encode(r, cw[:lz.CODE_K[r]]), cw)
