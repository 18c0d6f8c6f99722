"""Rows c-e on the GPU (pilot fit, soft demap, block stage, LDPC, CRC) through the C ABI: held bit for bit to the
reference's own outputs (tests/golden/rx_ref.npz) and to the oracle on synthetic frames of every picture size."""
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def check(out, want, frame=0):
    assert np.array_equal(out["align"][frame][:2], want["align"])
    assert np.array_equal(out["llrf"][frame], want["llrf"])
    assert np.array_equal(out["sub_rms"][frame], want["sub_rms"])
    np.testing.assert_allclose(out["sub_est"][frame], want["sub_est"], rtol=1e-13)
    assert np.array_equal(out["its"][frame], want["its"].astype(np.int32))
    assert np.array_equal(out["ok"][frame], want["ok"])
    np.testing.assert_allclose(out["est"][frame], want["est"], rtol=1e-6)
    assert np.array_equal(out["pilot"][frame], want["pilot"], equal_nan=True)


@pytest.mark.parametrize("tag", ["a", "b"])
def test_finish_coef_matches_reference_golden(tag):
    g = np.load(os.path.join(GOLD, "rx_ref.npz"))
    n, subch, span = (int(x) for x in g[tag + "_fmt"])
    rx = lz.Receiver(n, subch, span, max_frames=1)
    out = rx.finish_coef(g[tag + "_coef"][None])
    check(out, {k: g[tag + "_" + k] for k in ("align", "llrf", "sub_rms", "sub_est", "its", "ok", "est", "pilot")})
    ok = out["ok"][0].astype(bool)
    assert ok.all()
    assert np.array_equal(out["blocks"][0], g[tag + "_blocks"])


def oracle_frames(fmt, frames, seed, shift=None, sigma=3.0):
    o = oracle.Fmt(fmt.n, fmt.subch, fmt.span)
    grids, blocks = synth.grids(fmt, frames, seed=seed, sigma=sigma, shift=shift)
    res = [o.receive(grids[f]) for f in range(frames)]
    return grids, blocks, res


@pytest.mark.parametrize("n,subch,frames,shift,sigma", [(384, 64, 3, None, 3.0), (512, 256, 2, (0.2, 0.1), 3.0),
                                                        (768, 320, 2, None, 12.0), (1024, 1024, 1, (-0.15, 0.3), 3.0),
                                                        (1152, 720, 1, None, 3.0), (1280, 880, 1, None, 3.0),
                                                        (1536, 1024, 2, (0.3, -0.25), 3.0)])
def test_finish_coef_matches_oracle(n, subch, frames, shift, sigma):
    fmt = lz.Format(n, subch, 128)
    _, blocks, res = oracle_frames(fmt, frames, seed=n + frames, shift=shift, sigma=sigma)
    rx = lz.Receiver(n, subch, 128, max_frames=frames)
    out = rx.finish_coef(np.stack([r["coef"] for r in res]))
    for f in range(frames):
        check(out, {"align": res[f]["align"], "llrf": res[f]["llrf"], "sub_rms": res[f]["sub_rms"], "sub_est": res[f]["sub_est"],
                    "its": res[f]["its"], "ok": res[f]["ok"], "est": res[f]["est"], "pilot": res[f]["pilot"]}, f)
        ok = out["ok"][f].astype(bool)
        assert np.array_equal(out["blocks"][f][ok], blocks[f][ok])
    assert rx.launches == 3 + fmt.tiers


@pytest.mark.parametrize("n,subch,frames,sigma", [(384, 64, 3, 3.0), (768, 320, 4, 60.0), (1536, 1024, 2, 3.0)])
def test_mixed_decode_matches_per_tier(n, subch, frames, sigma):
    """The decode stage in one persistent launch across the tiers (lizg_rx_set_ldpc_mixed) against a launch a tier:
    the same blocks, verdicts and iterations (declined, stalled and capped blocks included at the noisy size)."""
    fmt = lz.Format(n, subch, 128)
    grids, _ = synth.grids(fmt, frames, seed=n + 7, sigma=sigma)
    rx = lz.Receiver(n, subch, 128, max_frames=frames)
    assert rx.set_ldpc_mixed(0) == 0
    a = rx.finish_grid(grids)
    assert rx.launches == 4 + 3 + fmt.tiers
    assert rx.set_ldpc_mixed(1) == 0
    b = rx.finish_grid(grids)
    assert rx.launches == 4 + 3 + 1
    for k in ("blocks", "ok", "its", "llrf", "est"):
        assert np.array_equal(a[k], b[k]), k
    if sigma > 10:
        assert (a["its"] < 0).any() and (a["ok"] == 1).any()


def test_receiver_refuses_bad_calls():
    """Every receiver entry point checks its arguments before it queues anything: a zero or oversized batch, a frame
    under 2 x 2 or a pitch or frame stride too short for it, a NULL frame, registration or output, an unknown read,
    decode stage or tier; each is refused with LIZG_E_ARG and the handle stays usable."""
    import ctypes
    import torch
    n, subch, span, W, H = 384, 64, 128, 1280, 720
    fmt = lz.Format(n, subch, span)
    grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, 5))
    luma, reg = synth.capture(fmt, grey, W, H, sigma=2.0, rng=np.random.default_rng(5))
    rx = lz.Receiver(n, subch, span, max_frames=2)
    o, s = lz.rx_outputs(rx.fmt, 2)
    d = torch.zeros((2, H, W), dtype=torch.uint8, device="cuda")
    r = torch.zeros((2, reg.size), dtype=torch.float32, device="cuda")
    L, P = lz.lib(), ctypes.c_void_p

    def call(luma=d.data_ptr(), w=W, h=H, pitch=W, stride=W * H, reg=r.data_ptr(), frames=1, out=s):
        return L.lizg_rx_finish_luma_dev(rx._h, P(luma), w, h, pitch, stride, P(reg), frames, ctypes.byref(out) if out else None,
                                         None, None, None)

    for kw in ({"frames": 0}, {"frames": 3}, {"w": 1}, {"pitch": W - 1}, {"stride": W * H - 1}, {"luma": 0}, {"reg": 0}, {"out": None}):
        assert call(**kw) == -1, kw
    assert call(out=lz.RxOut(None, s.ok, s.its, None, None, None, None, None, None)) == -1
    assert L.lizg_rx_set_read(rx._h, 7) == -1 and L.lizg_rx_set_ldpc_mixed(rx._h, 3) == -1 and L.lizg_rx_variant(rx._h, 9) == -1
    assert L.lizg_rx_finish_coef_dev(rx._h, None, 1, ctypes.byref(s), None) == -1
    # still usable: the clean frame decodes every block
    out = rx.finish_luma(luma[None], reg[None], grid=False)
    assert out["ok"].all()
