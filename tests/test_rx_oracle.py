"""The receiver's tables and oracle, on the CPU: the library's format tables against the oracle's (which the
reference pins where it is built), the synthetic pictures decodable, and the oracle held to the reference's own
receiver outputs (tests/golden/rx_ref.npz) and, where the reference is built here, to the reference on fresh
pictures."""
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FORMATS = [(384, 64), (384, 80), (512, 256), (768, 320), (1024, 1024), (1152, 720), (1280, 880), (1536, 1024)]


@pytest.mark.parametrize("n,subch", FORMATS)
def test_format_tables_match_oracle(n, subch):
    f, o = lz.Format(n, subch, 128), oracle.Fmt(n, subch, 128)
    assert (f.blocks, f.used, f.vblocks, f.tiers) == (o.blocks, o.used, o.vblocks, o.tiers)
    assert f.tier == o.tier
    for a, b in [(f.uv, o.uv), (f.white, o.white), (f.block_tier, o.block_tier), (f.block_slot, o.block_slot), (f.erase, o.erase)]:
        assert np.array_equal(a, b)
    assert np.array_equal(f.hole_inv, o.hole_inv)
    for t in range(f.tiers):
        assert np.array_equal(f.perm[t], o.perm(t))


@pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")
@pytest.mark.parametrize("n,subch,span", [(384, 64, 128), (768, 320, 256), (1536, 1024, 512), (1152, 720, 128)])
def test_oracle_tables_match_reference(n, subch, span):
    o, r = oracle.Fmt(n, subch, span), oracle.RefFmt(n, subch, span)
    t = r.tables()
    assert np.array_equal(o.pos, t["pos"]) and np.array_equal(o.white, t["white"])
    assert np.array_equal(o.block_tier, t["block_tier"]) and np.array_equal(o.block_slot, t["block_slot"])
    assert np.array_equal(o.erase, t["erase"]) and np.array_equal(o.hole_inv, t["hole_inv"])
    for k in range(o.tiers):
        assert np.array_equal(o.perm(k), r.perm(k))


def test_spec_7_4_whitening_and_slots():
    """SPEC 7.3/7.4: the whitening prefix, the permutation strides, and LIZARD-64's slot bits of the spec's blocks."""
    import json
    spec = json.load(open(os.path.join(GOLD, "spec_7_4.json")))
    f = lz.Format(384, 64, 128)
    assert np.packbits(f.white[:128]).tobytes().hex() == spec["whitening_first_128"]
    assert np.packbits(f.white[36576:36576 + 128]).tobytes().hex() == spec["padding_white_0_127"]
    for b in spec["blocks"]:
        s0 = b["first_slot"]
        assert int(f.block_slot[b["b"]]) == s0
        assert np.packbits(f.white[s0:s0 + 128]).tobytes().hex() == b["white_0_127"]
    p34 = f.perm[1]
    assert list(p34[:6]) == spec["perm_7_3"]["4"]["perm_0_5"]
    blocks = oracle.spec_blocks(7)
    sl = synth.slots(f, blocks, parity=0)
    for b in spec["blocks"]:
        if b["rate"] != 6:     # the spec's 3/4, 2/3, 1/2 rows predate the codes shipped (see test_oracle.py)
            continue
        s0 = b["first_slot"]
        assert np.packbits(sl[s0:s0 + 128]).tobytes().hex() == b["slots_0_127"]
        for c in range(4):
            t = synth.slots(f, blocks, parity=c)[s0 + 4480:s0 + 4496]
            assert np.packbits(t).tobytes().hex() == b["tail"][c]


@pytest.mark.parametrize("n,subch,shift", [(384, 64, None), (768, 320, (0.3, -0.25)), (1536, 1024, None)])
def test_synthetic_pictures_decode_in_the_oracle(n, subch, shift):
    f, o = lz.Format(n, subch, 128), oracle.Fmt(n, subch, 128)
    g, blocks = synth.grids(f, 1, seed=n, sigma=3.0, shift=shift)
    res = o.receive(g[0])
    assert res["ok"].all()
    assert np.array_equal(res["blocks"], blocks[0])
    if shift:
        assert abs(res["align"][0] + shift[0]) < 0.05 and abs(res["align"][1] + shift[1]) < 0.05


def _gold():
    return np.load(os.path.join(GOLD, "rx_ref.npz"))


@pytest.mark.parametrize("tag", ["a", "b"])
def test_oracle_matches_reference_golden(tag):
    g = _gold()
    n, subch, span = (int(x) for x in g[tag + "_fmt"])
    o = oracle.Fmt(n, subch, span)
    coef = g[tag + "_coef"]
    d, used = o.pilot_align(coef)
    turn = d if (used and (d[0] != 0 or d[1] != 0)) else None
    assert np.array_equal(d if turn is not None else np.zeros(2, np.float32), g[tag + "_align"])
    llrf, est, rms = o.demap(coef, turn)
    assert np.array_equal(llrf, g[tag + "_llrf"])
    assert np.array_equal(rms, g[tag + "_sub_rms"])
    np.testing.assert_allclose(est, g[tag + "_sub_est"], rtol=1e-13)
    B = o.blocks_stage(llrf, est, rms, coef, turn)
    assert np.array_equal(B["its"], g[tag + "_its"]) and np.array_equal(B["ok"], g[tag + "_ok"])
    assert np.array_equal(B["pilot"], g[tag + "_pilot"], equal_nan=True)
    # the FP64 spectrum of the same grid against the reference's FP32 one
    spec, _, _ = o.spectrum(g[tag + "_grey"].astype(np.float32) / np.float32(255.0))
    rc = coef[0::2] + 1j * coef[1::2]
    rms_s = np.sqrt(np.mean(np.abs(spec) ** 2))
    assert np.abs(rc - spec).max() / rms_s < 1e-4
