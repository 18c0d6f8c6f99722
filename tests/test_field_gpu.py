"""The registration refined by its adjoint (lizg_field_*): the three terms' gradients (pilots, timing track, anchors'
centres) against central finite differences of the GPU's own terms, the pilots' adjoint against an FP64 host
implementation of the same adjoint (numpy: the warp, the bilinear read and its gradient, the erase held constant, the
detrend, the pilots' DFT, the gains, the residuals' inverse transform and the tangents, every step in double), and the
refinement taking a perturbed registration back towards the true one and the blocks back."""
import numpy as np
import pytest

import lizard_gb300 as lz
from lizard_gb300_testing import render, synth

pytestmark = pytest.mark.gpu

N, SUBCH, SPAN, W, HH = 384, 64, 128, 1280, 720
FP = lz.FIELD_PARAMS


def capture(seed=5, k1=0.02, blur=0.8):
    import torch
    fmt = lz.Format(N, SUBCH, SPAN)
    blocks = synth.random_blocks(fmt.blocks, seed)[None]
    pg, pxm = render.pages(lz, N, SUBCH, SPAN, blocks, 1)
    rng = np.random.default_rng(seed)
    Hw = np.asarray(synth.warp(fmt, W, HH, rng, rot_deg=12, scale=(1.2, 1.3)), np.float64).reshape(3, 3)
    luma = render.capture(pg[0], pxm, W, HH, Hw, k1, blur, 2.0, seed).cpu().numpy()
    return fmt, luma, Hw, blocks[0]


def knots(span):
    """The field's knots along an axis and every node's Hermite weights on them, in double (field.cu's host set-up)."""
    pos = synth.layout_nodes(span).astype(np.float64)
    aside = span // 64
    anc = np.array([np.floor(15 + span * (i + 0.5) / 7 - aside / 2.0 + 0.5) + aside / 2.0 for i in range(7)])
    X0, SX = pos[0], pos[-1] - pos[0]
    t = np.concatenate([[0.0], (anc - X0) / SX, [1.0]])
    wk = np.zeros((pos.size, 9))
    for i, p in enumerate(pos):
        x = (p - X0) / SX
        k = 0
        while k < 9 - 2 and x >= t[k + 1]:
            k += 1
        hc = t[k + 1] - t[k]
        s = (x - t[k]) / hc
        s2, s3 = s * s, s * s * s
        w = [0.0, 2 * s3 - 3 * s2 + 1, -2 * s3 + 3 * s2, 0.0]
        A, B = (s3 - 2 * s2 + s) * hc, (s3 - s2) * hc
        if k > 0:
            d = t[k + 1] - t[k - 1]; w[0] -= A / d; w[2] += A / d
        else:
            w[1] -= A / hc; w[2] += A / hc
        if k + 2 < 9:
            d = t[k + 2] - t[k]; w[1] -= B / d; w[3] += B / d
        else:
            w[1] -= B / hc; w[2] += B / hc
        for q in range(4):
            if 0 <= k - 1 + q < 9:
                wk[i, k - 1 + q] += w[q]
    return pos, anc, wk


def pilots(fmt):
    """Every block tail's coefficient: index, (u, v), symbol for a count bit of 0, group (parity x 8 + radius band)."""
    ks, par = [], []
    for b in range(fmt.blocks):
        rate, _, slots = fmt.tier[fmt.block_tier[b]]
        first = fmt.block_slot[b] // 2
        for s in range(lz.CODE_NT[rate] // 2, slots // 2):
            ks.append(first + s)
            par.append(b & 1)
    ks = np.array(ks)
    u, v = fmt.uv[2 * ks].astype(np.int64), fmt.uv[2 * ks + 1].astype(np.int64)
    a = np.float32(0.70710678)
    shat = np.where(fmt.white[2 * ks], -a, a).astype(np.float64) + 1j * np.where(fmt.white[2 * ks + 1], -a, a).astype(np.float64)
    rho = np.hypot(u, v)
    srt = np.sort(rho)
    band = np.zeros(ks.size, np.int64)
    for q in range(1, 8):
        band[rho > srt[int(q * (ks.size - 1) / 8)]] = q
    return ks, u, v, shat, np.array(par) * 8 + band


def fp64_pilot_adjoint(fmt, luma, reg, theta):
    """The pilots' loss and its gradient in the 106 parameters, every step in double."""
    n = fmt.n
    pos, anc, wk = knots(fmt.span)
    nn = pos.size
    scale = n / fmt.span
    g0, step = 15 + 0.5 / scale, 1.0 / scale
    Hh = np.append(np.asarray(theta[:8], np.float64), 1.0)
    F = np.zeros((9, 9, 2))
    F[1:8, 1:8] = np.asarray(theta[8:], np.float64).reshape(7, 7, 2)
    mesh = np.asarray(reg[9:], np.float64).reshape(nn, nn, 2) + np.einsum("jb,ia,bac->jic", wk, wk, F)
    m = g0 + np.arange(n) * step

    def cells(mm):
        k = np.zeros(mm.size, np.int64)
        for q in range(1, nn - 1):
            k[mm >= pos[q]] = q
        return k, (mm - pos[k]) / (pos[k + 1] - pos[k])
    i, uu = cells(m)
    j, vv = cells(m)
    MX, MY = np.meshgrid(m, m)
    UU, VV = np.meshgrid(uu, vv)
    II, JJ = np.meshgrid(i, j)
    D = (mesh[JJ, II] * (1 - UU)[..., None] + mesh[JJ, II + 1] * UU[..., None]) * (1 - VV)[..., None] + \
        (mesh[JJ + 1, II] * (1 - UU)[..., None] + mesh[JJ + 1, II + 1] * UU[..., None]) * VV[..., None]
    wd = Hh[6] * MX + Hh[7] * MY + 1
    U = (Hh[0] * MX + Hh[1] * MY + Hh[2]) / wd
    V = (Hh[3] * MX + Hh[4] * MY + Hh[5]) / wd
    sx0, sy0 = U + D[..., 0] - 0.5, V + D[..., 1] - 0.5
    sx, sy = np.clip(sx0, 0, W - 1.001), np.clip(sy0, 0, HH - 1.001)
    xi, yi = np.floor(sx).astype(np.int64), np.floor(sy).astype(np.int64)
    fx, fy = sx - xi, sy - yi
    L = luma.astype(np.float64) / 255.0
    A, B, C, Dd = L[yi, xi], L[yi, xi + 1], L[yi + 1, xi], L[yi + 1, xi + 1]
    z = (A + (B - A) * fx) * (1 - fy) + (C + (Dd - C) * fx) * fy
    Iu = np.where(sx == sx0, (B - A) * (1 - fy) + (Dd - C) * fy, 0.0)
    Iv = np.where(sy == sy0, (C - A) * (1 - fx) + (Dd - B) * fx, 0.0)
    # the anchors' erase: the shading surface, fitted over every eighth sample outside the squares
    elo, ehi = fmt.erase[:7], fmt.erase[7:]
    insq = np.zeros(n, bool)
    for a in range(7):
        insq[elo[a]:ehi[a] + 1] = True
    er = insq[:, None] & insq[None, :]
    det = fmt.detrend.astype(np.float64)
    cx, qx = det[0:n], det[n:2 * n]
    X1, X2 = det[2 * n:3 * n] + 1j * det[3 * n:4 * n], det[4 * n:5 * n] + 1j * det[5 * n:6 * n]
    sx2, sq2 = float(fmt.detrend[6 * n]), float(fmt.detrend[6 * n + 1])
    rhs = np.zeros(6)
    for ky in range(n // 8):
        for kx in range(n // 8):
            x, y = 8 * kx, 8 * ky
            if er[y, x]:
                continue
            rhs += np.array([1, cx[x], qx[x], cx[y], qx[y], cx[x] * cx[y]]) * z[y, x]
    beta = fmt.hole_inv.reshape(6, 6) @ rhs
    ze = z.copy()
    Y, X = np.nonzero(er)
    ze[Y, X] = beta[0] + beta[1] * cx[X] + beta[2] * qx[X] + beta[3] * cx[Y] + beta[4] * qx[Y] + beta[5] * cx[X] * cx[Y]
    px = (ze * cx[None, :]).sum() / (n * sx2)
    py = (ze * cx[:, None]).sum() / (n * sx2)
    pxy = (ze * cx[None, :] * cx[:, None]).sum() / (sx2 * sx2)
    pxx = (ze * qx[None, :]).sum() / (n * sq2)
    pyy = (ze * qx[:, None]).sum() / (n * sq2)
    ks, pu, pv, shat, grp = pilots(fmt)
    um = (pu + n) % n
    xs = np.arange(n)
    Ex = np.exp(-2j * np.pi * np.outer(pu, xs) / n)
    Ey = np.exp(-2j * np.pi * np.outer(pv, xs) / n)
    Cp = np.einsum("py,yp->p", Ey, ze @ Ex.T)
    Cp = Cp - pxy * X1[um] * X1[pv] - (pv == 0) * n * (px * X1[um] + pxx * X2[um]) - (pu == 0) * n * (py * X1[pv] + pyy * X2[pv])
    r = np.zeros(ks.size, np.complex128)
    for gidx in np.unique(grp):
        s = grp == gidx
        den = (np.abs(shat[s]) ** 2).sum()
        gain = (np.real(np.conj(shat[s]) * Cp[s])).sum() / den if den > 0 else 0.0
        r[s] = Cp[s] - gain * shat[s]
    loss = float((np.abs(r) ** 2).sum())
    G = 2 * np.real((r[None, :] * np.conj(Ey).T) @ np.conj(Ex))
    K1 = 2 * np.real(np.conj(r) * X1[um] * X1[pv]).sum() / sx2 ** 2
    K2 = 2 * np.real((np.conj(r) * X1[um])[pv == 0]).sum() / sx2
    K3 = 2 * np.real((np.conj(r) * X2[um])[pv == 0]).sum() / sq2
    K4 = 2 * np.real((np.conj(r) * X1[pv])[pu == 0]).sum() / sx2
    K5 = 2 * np.real((np.conj(r) * X2[pv])[pu == 0]).sum() / sq2
    G = G - K1 * cx[None, :] * cx[:, None] - K2 * cx[None, :] - K3 * qx[None, :] - K4 * cx[:, None] - K5 * qx[:, None]
    G[er] = 0
    iw = 1 / wd
    du = [MX * iw, MY * iw, iw, 0, 0, 0, -U * MX * iw, -U * MY * iw]
    dv = [0, 0, 0, MX * iw, MY * iw, iw, -V * MX * iw, -V * MY * iw]
    grad = np.zeros(FP)
    for q in range(8):
        grad[q] = (G * (Iu * du[q] + Iv * dv[q])).sum()
    Wx = wk[i] * (1 - uu)[:, None] + wk[i + 1] * uu[:, None]   # x -> knot weights
    Wy = wk[j] * (1 - vv)[:, None] + wk[j + 1] * vv[:, None]
    for c, Ic in enumerate((Iu, Iv)):
        Fg = Wy.T @ (G * Ic) @ Wx   # [b, a]
        grad[8 + c::2] = Fg[1:8, 1:8].ravel()
    return loss, grad


def anchors_at(luma, reg):
    out = lz.anchor_find(SPAN, luma[None], reg[None, :9])
    return {k: out[k] for k in ("ok", "u", "v")}


def theta0(reg, rng, field=0.3):
    th = np.zeros(FP, np.float32)
    th[:8] = reg[:8]
    th[8:] = rng.uniform(-field, field, FP - 8).astype(np.float32)
    return th


def test_pilots_adjoint_matches_fp64():
    fmt, luma, Hw, _ = capture()
    reg = render.registration(SPAN, Hw, 0.02, W, HH)
    th = theta0(reg, np.random.default_rng(1))
    fr = lz.FieldRefiner(N, SUBCH, SPAN, chunk=2)
    t = fr.terms(luma[None], reg[None], th[None])[0]
    loss, grad = fp64_pilot_adjoint(fmt, luma, reg, th)
    assert abs(t[0, 0] - loss) < 1e-3 * loss
    g = t[0, 1:]
    err = np.linalg.norm(g - grad) / np.linalg.norm(grad)
    errh = np.linalg.norm(g[:8] - grad[:8]) / np.linalg.norm(grad[:8])
    print("pilots' adjoint against FP64: loss %.6g / %.6g, gradient relative error %.3g (H alone %.3g)" % (t[0, 0], loss, err, errh))
    assert err < 1e-2 and errh < 1e-2


def steps_for(reg, span, px=0.01):
    """A finite-difference step a parameter: about px pixels of image motion at the layout's corners for H, px for a
    knot."""
    side = span + 30
    Hm = np.append(reg[:8], 1.0).reshape(3, 3).astype(np.float64)
    eps = np.full(FP, px)
    for q in range(8):
        worst = 0.0
        for X, Y in ((0, 0), (side, 0), (side, side), (0, side)):
            for d in (1e-6, -1e-6):
                Hp = Hm.copy().ravel()
                Hp[q] += d
                Hp = Hp.reshape(3, 3)
                a, b = Hm @ [X, Y, 1], Hp @ [X, Y, 1]
                worst = max(worst, np.hypot(*(a[:2] / a[2] - b[:2] / b[2])) / 1e-6)
        eps[q] = px / worst
    return eps


@pytest.mark.parametrize("term", [0, 1, 2], ids=["pilots", "track", "anchors"])
def test_terms_gradients_match_central_differences(term):
    """Central differences of 0.01 px of image motion, on a capture blurred to 1.5 px for the pilots and the track (the
    bilinear read's kinks at pixel edges, which a difference straddles now and then, stay small against the gradient)
    and 0.8 px for the anchors (their search finds them)."""
    fmt, luma, Hw, _ = capture(blur=1.5 if term < 2 else 0.8)
    reg = render.registration(SPAN, Hw, 0.02, W, HH)
    anc = anchors_at(luma, reg)
    assert term < 2 or anc["ok"].sum() >= 20
    th = theta0(reg, np.random.default_rng(2))
    fr = lz.FieldRefiner(N, SUBCH, SPAN, chunk=16)
    eps = steps_for(reg, SPAN)
    rng = np.random.default_rng(3)
    params = list(range(8)) + sorted(rng.choice(np.arange(8, FP), 8, replace=False).tolist())
    # every probe in one batch: theta, then theta +- eps e_q
    thetas = [th]
    for q in params:
        for sgn in (1, -1):
            t = th.astype(np.float64).copy()
            t[q] += sgn * eps[q]
            thetas.append(t.astype(np.float32))
    out = []
    for a in range(0, len(thetas), 16):
        chunk = np.stack(thetas[a:a + 16])
        k = chunk.shape[0]
        out.append(fr.terms(np.broadcast_to(luma, (k,) + luma.shape), np.broadcast_to(reg, (k, reg.size)), chunk,
                            anchors={key: np.broadcast_to(v, (k, 49)) for key, v in anc.items()}))
    T = np.concatenate(out)
    g = T[0, term, 1:]
    fd = np.array([(T[1 + 2 * i, term, 0] - T[2 + 2 * i, term, 0]) / (np.float64(thetas[1 + 2 * i][q]) - np.float64(thetas[2 + 2 * i][q]))
                   for i, q in enumerate(params)])
    ga = g[params]
    for lo, hi, name in ((0, 8, "H"), (8, len(params), "field")):
        rel = np.linalg.norm(fd[lo:hi] - ga[lo:hi]) / np.linalg.norm(ga[lo:hi])
        print("term %d %s: |fd - adjoint| / |adjoint| = %.3g over %d parameters" % (term, name, rel, hi - lo))
        assert rel < (0.05 if term < 2 else 0.01)


def test_refinement_recovers_a_perturbed_registration():
    fmt, luma, Hw, blocks = capture(seed=8, k1=0.03, blur=0.6)
    true = render.registration(SPAN, Hw, 0.03, W, HH, true_mesh=True)
    plain = render.registration(SPAN, Hw, 0.03, W, HH)
    bad = plain.copy()
    bad[2] += 0.8
    bad[5] -= 0.6
    rx = lz.Receiver(N, SUBCH, SPAN, max_frames=3)
    fr = lz.FieldRefiner(N, SUBCH, SPAN, chunk=2)
    anc = anchors_at(luma, bad)
    ref, loss, imp = fr.refine(luma[None], bad[None], steps=6, anchors={k: v for k, v in anc.items()})
    out = rx.finish_luma(np.stack([luma, luma, luma]), np.stack([true, bad, ref[0]]), grid=False)
    ok_true, ok_bad, ok_ref = (int(out["ok"][k].sum()) for k in range(3))
    print("blocks verified: true map %d, perturbed %d, refined %d of %d" % (ok_true, ok_bad, ok_ref, fmt.blocks))
    assert imp[0] == 1 and ok_ref >= ok_true - 1 and ok_ref > ok_bad
