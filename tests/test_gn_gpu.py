"""The registration refined from the pilots (lizg_gn_*): its tangent pictures against central finite differences of
the receiver's own spectrum at the pilots, one Gauss-Newton step against an FP64 host implementation of the same step
(numpy sampling and tangents, the oracle's FP64 front), and the refinement bringing a homography a pixel off back:
the corners' error falls and the frames decode no worse than the plain registration; a frame with no signal keeps it."""
import numpy as np
import pytest

import lizard_gb300 as lz
import oracle
from lizard_gb300_testing import synth

pytestmark = pytest.mark.gpu


def pilots(fmt):
    """Pilot coefficients (pos order), symbols for a count bit of 0, block parity, radius band (8 quantile bands)."""
    pk, par = [], []
    for b in range(fmt.blocks):
        rate, _, slots = fmt.tier[fmt.block_tier[b]]
        first = fmt.block_slot[b] // 2
        for s in range(lz.CODE_NT[rate] // 2, slots // 2):
            pk.append(first + s)
            par.append(b & 1)
    pk = np.array(pk)
    a = np.float32(0.70710678)
    shat = np.where(fmt.white[2 * pk] == 1, -a, a) + 1j * np.where(fmt.white[2 * pk + 1] == 1, -a, a)
    uv = fmt.uv.reshape(-1, 2)[pk].astype(np.float64)
    rho = np.hypot(uv[:, 0], uv[:, 1])
    srt = np.sort(rho)
    th = [srt[int(q * (len(rho) - 1) / 8)] for q in range(1, 8)]
    band = np.array([sum(r > t for t in th) for r in rho])
    return pk, shat, np.array(par), band


def corners_of(Hm, side):
    c = np.array([[0, 0], [side, 0], [side, side], [0, side]], np.float64)
    q = np.asarray(Hm, np.float64).reshape(3, 3) @ np.column_stack([c, np.ones(4)]).T
    return np.stack([q[0] / q[2], q[1] / q[2]], 1)


def perturbed(reg, span, rng, px=1.2):
    side = span + 30
    c = np.array([[0, 0], [side, 0], [side, side], [0, side]], np.float64)
    cq = corners_of(reg[:9], side) + rng.uniform(-px, px, (4, 2))
    out = reg.copy()
    out[:9] = synth.homography_4(c, cq).astype(np.float32)
    return out


def capture64(seed):
    fmt = lz.Format(384, 64, 128)
    rng = np.random.default_rng(seed)
    blocks = synth.random_blocks(fmt.blocks, seed)
    luma, reg = synth.capture(fmt, synth.picture(fmt, blocks), 1280, 720, H=synth.warp(fmt, 1280, 720, rng, scale=(0.95, 1.05)), sigma=2.0, rng=rng)
    return fmt, luma, reg, blocks, rng


def test_tangents_match_finite_differences():
    fmt, luma, reg, _, rng = capture64(5)
    reg = perturbed(reg, 128, rng, 0.5)
    gn = lz.PilotRefiner(384, 64, 128, chunk=2)
    rx = lz.Receiver(384, 64, 128, max_frames=9)
    pk = pilots(fmt)[0]
    pics = gn.pictures(luma[None], reg[None])[0]
    J = rx.spectrum_grid(pics[1:])[:, pk]               # 8 x pilots
    for j in range(8):
        # a step that moves the map by about 0.02 pixels at the picture's far corner
        mx = 15 + 384 / (384 / 128)
        scale = {0: mx, 1: mx, 2: 1.0, 3: mx, 4: mx, 5: 1.0, 6: mx * 1000, 7: mx * 1000}[j]
        eps = 0.02 / scale
        rp, rm = reg.copy(), reg.copy()
        rp[j] += np.float32(eps)
        rm[j] -= np.float32(eps)
        e = float(np.float32(reg[j] + np.float32(eps)) - np.float32(reg[j] - np.float32(eps))) / 2
        gp = gn.pictures(luma[None], rp[None])[0][0]
        gm = gn.pictures(luma[None], rm[None])[0][0]
        cp, cm = rx.spectrum_grid(np.stack([gp, gm]))[:, pk]
        fd = (cp - cm) / (2 * e)
        rel = np.linalg.norm(fd - J[j]) / np.linalg.norm(J[j])
        assert rel < 0.1, (j, rel)


def fp64_step(fmt, luma, reg):
    """The same step in double on the host: bilinear samples and tangents of the plain map (the mesh is zero here),
    the oracle's FP64 front, the gains, the mismatch, the column-scaled normal equations."""
    n, span = fmt.n, fmt.span
    O = oracle.Fmt(n, fmt.subch, span)
    pk, shat, par, band = pilots(fmt)
    h_, w_ = luma.shape
    L = luma.astype(np.float64) / 255.0
    mx = np.float32(15) + np.float32(0.5) / fmt.scale + np.arange(n, dtype=np.float32) * (np.float32(1) / fmt.scale)
    MX, MY = np.meshgrid(mx.astype(np.float64), mx.astype(np.float64))
    h = reg[:9].astype(np.float64)
    wd = h[6] * MX + h[7] * MY + 1
    U = (h[0] * MX + h[1] * MY + h[2]) / wd
    V = (h[3] * MX + h[4] * MY + h[5]) / wd
    xs, ys = np.clip(U - 0.5, 0, w_ - 1.001), np.clip(V - 0.5, 0, h_ - 1.001)
    xi, yi = np.floor(xs).astype(int), np.floor(ys).astype(int)
    fx, fy = xs - xi, ys - yi
    A, B, C, D = L[yi, xi], L[yi, xi + 1], L[yi + 1, xi], L[yi + 1, xi + 1]
    g = (A + (B - A) * fx) * (1 - fy) + (C + (D - C) * fx) * fy
    Iu, Iv = (B - A) * (1 - fy) + (D - C) * fy, (C - A) * (1 - fx) + (D - B) * fx
    z = 0 * wd
    du = [MX / wd, MY / wd, 1 / wd, z, z, z, -U * MX / wd, -U * MY / wd]
    dv = [z, z, z, MX / wd, MY / wd, 1 / wd, -V * MX / wd, -V * MY / wd]
    Cp = O.spectrum(g.astype(np.float32))[0][pk]
    Js = np.stack([O.spectrum((Iu * du[j] + Iv * dv[j]).astype(np.float32))[0][pk] for j in range(8)], 1)
    r = np.zeros_like(Cp)
    for c in (0, 1):
        for b in range(8):
            m = (par == c) & (band == b)
            if m.any():
                gk = np.sum(np.real(np.conj(shat[m]) * Cp[m])) / np.sum(np.abs(shat[m]) ** 2)
                r[m] = Cp[m] - gk * shat[m]
    Jr, rr = np.concatenate([Js.real, Js.imag]), np.concatenate([r.real, r.imag])
    N, gv = Jr.T @ Jr, Jr.T @ rr
    s = np.sqrt(np.diag(N))
    return -np.linalg.solve(N / np.outer(s, s) + 1e-9 * np.eye(8), gv / s) / s


def test_step_matches_fp64_host():
    fmt, luma, reg, _, rng = capture64(6)
    reg = perturbed(reg, 128, rng, 1.0)
    want = fp64_step(fmt, luma, reg)
    gn = lz.PilotRefiner(384, 64, 128, chunk=1)
    out, _, improved = gn.refine(luma[None], reg[None], steps=1)
    assert improved[0] == 1
    # the two steps' homographies put the layout's corners within 0.05 pixels of each other
    h_fp64 = reg[:9].astype(np.float64).copy()
    h_fp64[:8] += want
    moved = np.abs(corners_of(h_fp64, 158) - corners_of(reg[:9], 158)).max()
    diff = np.abs(corners_of(out[0, :9], 158) - corners_of(h_fp64, 158)).max()
    assert moved > 0.1 and diff < 0.05, (moved, diff)


def decoded(rx, luma, reg):
    return rx.finish_luma(luma, reg, grid=False)["ok"].sum(1)


def test_refinement_recovers_homography_64():
    gn = lz.PilotRefiner(384, 64, 128, chunk=4)
    rx = lz.Receiver(384, 64, 128, max_frames=4)
    caps = [capture64(20 + k) for k in range(4)]
    luma = np.stack([c[1] for c in caps])
    true = np.stack([c[2] for c in caps])
    rng = np.random.default_rng(9)
    plain = np.stack([perturbed(t, 128, rng, 1.2) for t in true])
    ref, loss, improved = gn.refine(luma, plain, steps=3)
    side = 158
    err = lambda R: [np.abs(corners_of(R[k, :9], side) - corners_of(true[k, :9], side)).max() for k in range(4)]
    assert np.mean(err(ref)) < 0.5 * np.mean(err(plain)), (err(plain), err(ref))
    assert np.all(decoded(rx, luma, ref) >= decoded(rx, luma, plain))


def test_refinement_recovers_homography_1024():
    """Config-4-style captures: LIZARD-1024 in the 128 ring on 1920 x 1080, tilted and rotated, mild blur."""
    fmt = lz.Format(1536, 1024, 256)
    lumas, trues = [], []
    for k in range(2):
        rng = np.random.default_rng(300 + k)
        grey = synth.picture(fmt, synth.random_blocks(fmt.blocks, 300 + k))
        view = synth.distorted_view(fmt, 1920, 1080, rng, base_side=1000.0)
        luma, reg = synth.distorted_capture(fmt, grey, 1920, 1080, view, k1=0.0, blur=0.5, sigma=3.0, rng=rng)
        lumas.append(luma)
        trues.append(reg)
    luma, true = np.stack(lumas), np.stack(trues)
    rng = np.random.default_rng(10)
    plain = np.stack([perturbed(t, 256, rng, 1.2) for t in true])
    gn = lz.PilotRefiner(1536, 1024, 256, chunk=2)
    ref, loss, improved = gn.refine(luma, plain, steps=3)
    rx = lz.Receiver(1536, 1024, 256, max_frames=2)
    d_plain, d_ref = decoded(rx, luma, plain), decoded(rx, luma, ref)
    assert improved.all() and np.all(d_ref >= d_plain) and d_ref.sum() > d_plain.sum(), (d_plain, d_ref)


def test_no_signal_keeps_the_plain_registration():
    _, luma, reg, _, _ = capture64(7)
    gn = lz.PilotRefiner(384, 64, 128, chunk=1)
    grey = np.full_like(luma, 128)
    out, _, improved = gn.refine(grey[None], reg[None], steps=3)
    assert improved[0] == 0 and np.array_equal(out[0], reg)
