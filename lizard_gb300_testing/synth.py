"""Synthetic inputs shaped like the reference's own test channels (no dataset exists for this path).

LDPC batch: 476-byte blocks (4-byte id, 472 seeded random payload bytes) with their CRC-32C appended MSB first
(liblizard/src/lizard_phy.c:1120-1131), the 7/8 code's 128 extra data bits zero, encoded by the format's codes;
BPSK over AWGN at a given Eb/N0 with R = 3840 / nt; LLR = 2 y / sigma^2 in float; int8 = round-half-even(8 LLR)
clipped to +-80 (the receiver's soft stage, liblizard/test/ldpc_awgn.c:67-78, liblizard/test/ldpc_ref.h:41-42);
the 7/8 code's never-sent bits fed as known zeros, +127 (liblizard/src/lizard_phy.c:1823).
"""
import numpy as np

from lizard_gb300 import BLOCK_BYTES, CODE_K, CODE_N, CODE_NT, INFO_BITS, SUB, crc32c, ldpc_encode_many

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


# ---------------------------------------------------------------- pictures and captures

def _block_bits(block_rows):
    """count x 476 bytes -> count x 3840 bits: the bytes MSB first, then the CRC-32C MSB first."""
    count = block_rows.shape[0]
    crc = np.array([crc32c(block_rows[i].tobytes()) for i in range(count)], np.uint32)
    cb = np.stack([(crc >> 24) & 255, (crc >> 16) & 255, (crc >> 8) & 255, crc & 255], axis=1).astype(np.uint8)
    return np.unpackbits(np.concatenate([block_rows, cb], axis=1), axis=1)


def slots(fmt, block_rows, parity=0):
    """The frame's subch x 640 slot bits (liblizard/src/lizard_phy.c:1096-1150): each block's codeword through the bit
    map and the whitening, its tail the pilot bit (bit 0 of the count on an even block, bit 1 on an odd one), the
    padding the whitening alone."""
    out = fmt.white.copy()
    bits = _block_bits(np.asarray(block_rows, np.uint8))
    for t in range(fmt.tiers):
        rate = fmt.tier[t][0]
        idx = np.nonzero(fmt.block_tier == t)[0]
        data = np.zeros((idx.size, CODE_K[rate]), np.uint8)
        data[:, :INFO_BITS] = bits[idx]
        cw = ldpc_encode_many(rate, data)
        nt, nb = CODE_NT[rate], fmt.tier[t][2]
        for j, b in enumerate(idx):
            s0 = int(fmt.block_slot[b])
            seg = np.empty(nb, np.uint8)
            seg[:nt] = cw[j][fmt.perm[t]]
            seg[nt:] = (parity >> (b & 1)) & 1
            out[s0:s0 + nb] = seg ^ fmt.white[s0:s0 + nb]
    return out


def picture(fmt, block_rows, parity=0, anchors=True):
    """The n x n picture as grey levels (uint8): Gray QPSK of unit magnitude on the used coefficients, the Hermitian
    inverse transform, clipped at 2 sqrt(640 subch) and mapped to 0..1 (liblizard/src/lizard_phy.c:1134-1187), the
    anchors' squares painted over it (liblizard/src/lizard_phy.c:1218-1234), rounded to 8 bits (:700-716). Computed
    in double; a sender's own rounding differs in the last bits, not in what a receiver reads."""
    n = fmt.n
    sb = slots(fmt, block_rows, parity)
    a = np.float32(0.70710678)
    sym = np.where(sb[0::2], -a, a).astype(np.float64) + 1j * np.where(sb[1::2], -a, a).astype(np.float64)
    S = np.zeros((n, n), np.complex128)
    u, v = fmt.uv[0::2].astype(np.int64), fmt.uv[1::2].astype(np.int64)
    S[v, (u + n) % n] = sym
    z = 2.0 * np.real(np.fft.ifft2(S)) * (n * n)      # z[y, x]
    lim = np.float32(2.0 * 2.0 * np.sqrt(np.float32(0.5 * fmt.subch * SUB)))
    sc = np.float32(0.5) / lim
    d = (np.float32(0.5) + np.clip(z.astype(np.float32), -lim, lim) * sc).astype(np.float32)
    if anchors:
        span = fmt.span
        aside = span // 64
        pxm = n / span
        for j in range(7):
            for i in range(7):
                m0x = int(np.floor(15 + span * (i + 0.5) / 7 - aside / 2.0 + 0.5)) - 15
                m0y = int(np.floor(15 + span * (j + 0.5) / 7 - aside / 2.0 + 0.5)) - 15
                side = aside * pxm
                half = 0.5 * side
                ys = np.arange(int(m0y * pxm), int(m0y * pxm + side))
                xs = np.arange(int(m0x * pxm), int(m0x * pxm + side))
                yy, xx = np.meshgrid(ys - m0y * pxm + 0.5 - half, xs - m0x * pxm + 0.5 - half, indexing="ij")
                dd = np.maximum(np.abs(xx), np.abs(yy)) / half
                d[np.ix_(ys, xs)] = np.where((dd < 0.25) | (dd >= 0.6), 1.0, 0.0)
    return np.clip((d.astype(np.float64) * 255.0 + 0.5).astype(np.int64), 0, 255).astype(np.uint8)


def noisy(grey, sigma, rng):
    """AWGN of sigma grey levels, rounded and clipped to 8 bits."""
    return np.clip(np.rint(grey.astype(np.float64) + sigma * rng.standard_normal(grey.shape)), 0, 255).astype(np.uint8)


def random_blocks(count, seed):
    b = np.zeros((count, BLOCK_BYTES), np.uint8)
    b[:, :4] = np.arange(count, dtype="<u4").view(np.uint8).reshape(count, 4)
    b[:, 4:] = np.random.default_rng(seed).integers(0, 256, (count, BLOCK_BYTES - 4), dtype=np.uint8)
    return b


def grids(fmt, frames, seed=0, sigma=3.0, shift=None):
    """Config-3-style picture grids: frames x n x n float32 (grey / 255), each a seeded random frame of blocks painted,
    AWGN of sigma grey levels added. shift=(dx, dy) samples moves every picture by a sub-sample amount (a phase ramp on
    its spectrum) before quantisation, which the pilots' fit then has to find. Also returns the blocks."""
    rng = np.random.default_rng(seed)
    out = np.empty((frames, fmt.n, fmt.n), np.float32)
    blocks = []
    for f in range(frames):
        b = random_blocks(fmt.blocks, seed * 1000 + f)
        g = picture(fmt, b, parity=f & 3).astype(np.float64)
        if shift is not None:
            n = fmt.n
            k = np.fft.fftfreq(n) * n
            ramp = np.exp(-2j * np.pi * (k[None, :] * shift[0] + k[:, None] * shift[1]) / n)
            g = np.real(np.fft.ifft2(np.fft.fft2(g) * ramp))
        out[f] = noisy(g, sigma, rng).astype(np.float32) / np.float32(255.0)
        blocks.append(b)
    return out, blocks


def layout_nodes(span):
    """The registration mesh's node centres (module coordinates) of a ring of span modules."""
    from lizard_gb300 import lib, _ptr
    import ctypes
    nx = np.zeros(40, np.float32)
    nn = np.zeros(2, np.int32)
    lib().lizg_layout_nodes.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    k = lib().lizg_layout_nodes(span, _ptr(nx), None, _ptr(nn))
    return nx[:k].copy()


def capture(fmt, grey, width=1280, height=720, H=None, sigma=2.0, rng=None, mid=128):
    """A captured luma frame holding the picture: the n x n grey picture at exact-copy scale (one pixel a sample;
    pxm = n / span pixels a module) inside its layout (light border, not read by the receiver), mapped into a
    width x height frame of mid-grey by the homography H (module coordinates to image pixels; None: axis-aligned and
    centred), bilinear in the picture's pixels, AWGN of sigma grey levels. Returns (luma uint8, registration floats:
    H then a zero node mesh)."""
    n, span = fmt.n, fmt.span
    pxm = n / span
    side = span + 30
    px = int(round(side * pxm))
    drive = np.full((px, px), 255.0)
    o = int(round(15 * pxm))
    drive[o:o + n, o:o + n] = grey
    if H is None:
        ox, oy = (width - px) // 2, (height - px) // 2
        H = np.array([pxm, 0, ox, 0, pxm, oy, 0, 0, 1], np.float64)
    Hm = np.asarray(H, np.float64).reshape(3, 3)
    Hi = np.linalg.inv(Hm)
    V, U = np.mgrid[0:height, 0:width].astype(np.float64)
    q = Hi @ np.stack([U.ravel() + 0.5, V.ravel() + 0.5, np.ones(U.size)])
    mx, my = q[0] / q[2], q[1] / q[2]
    # drive pixel coordinates, centres at half-integers
    sx, sy = mx * pxm - 0.5, my * pxm - 0.5
    inside = (sx >= 0) & (sy >= 0) & (sx <= px - 1.001) & (sy <= px - 1.001)
    x0 = np.clip(np.floor(sx).astype(np.int64), 0, px - 2)
    y0 = np.clip(np.floor(sy).astype(np.int64), 0, px - 2)
    fx, fy = np.clip(sx - x0, 0, 1), np.clip(sy - y0, 0, 1)
    val = (drive[y0, x0] * (1 - fx) + drive[y0, x0 + 1] * fx) * (1 - fy) + (drive[y0 + 1, x0] * (1 - fx) + drive[y0 + 1, x0 + 1] * fx) * fy
    img = np.where(inside, val, float(mid)).reshape(height, width)
    rng = np.random.default_rng(0) if rng is None else rng
    luma = np.clip(np.rint(img + sigma * rng.standard_normal(img.shape)), 0, 255).astype(np.uint8)
    nn = layout_nodes(span).size
    reg = np.concatenate([np.asarray(H, np.float32).ravel() / np.float32(np.asarray(H).ravel()[8]), np.zeros(2 * nn * nn, np.float32)])
    return luma, reg


def warp(fmt, width, height, rng, rot_deg=15.0, tilt=0.0002, scale=(0.9, 1.05)):
    """A random homography (module -> image): rotation, a little perspective and scale about the frame centre, the
    picture at exact-copy pixels a module times the scale."""
    pxm = fmt.n / fmt.span
    side = fmt.span + 30
    th = np.deg2rad(rng.uniform(-rot_deg, rot_deg))
    s = pxm * rng.uniform(*scale)
    c, si = np.cos(th), np.sin(th)
    # centre the layout's middle on the frame centre
    A = np.array([[s * c, -s * si, 0], [s * si, s * c, 0], [0, 0, 1]])
    T0 = np.array([[1, 0, -side / 2], [0, 1, -side / 2], [0, 0, 1]])
    P = np.array([[1, 0, 0], [0, 1, 0], [rng.uniform(-tilt, tilt), rng.uniform(-tilt, tilt), 1]])
    T1 = np.array([[1, 0, width / 2], [0, 1, height / 2], [0, 0, 1]])
    H = T1 @ P @ A @ T0
    return (H / H[2, 2]).ravel()


def distorted_view(fmt, width, height, rng, base_side=700.0, rot_deg=15.0, tilt_deg=20.0, scale=(0.8, 1.1), focal=None, tries=50):
    """A camera's view of the layout: rotation U(+-rot_deg) in the image plane, a tilt U(+-tilt_deg) of the symbol's
    plane about a random in-plane axis (a pinhole camera of focal length `focal` pixels, default the frame's width),
    the layout's side base_side x U(scale) pixels at the frame centre. Redrawn until the layout's four corners stay
    inside the frame. Returns H (module -> ideal image pixels, 3 x 3)."""
    side = fmt.span + 30
    f = float(width) if focal is None else focal
    for _ in range(tries):
        rot = np.deg2rad(rng.uniform(-rot_deg, rot_deg))
        tilt = np.deg2rad(rng.uniform(-tilt_deg, tilt_deg))
        phi = rng.uniform(0, np.pi)
        s = base_side * rng.uniform(*scale) / side
        ax = np.array([np.cos(phi), np.sin(phi), 0.0])
        Kx = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        Rt = np.eye(3) + np.sin(tilt) * Kx + (1 - np.cos(tilt)) * (Kx @ Kx)   # Rodrigues: the tilt about ax
        Rz = np.array([[np.cos(rot), -np.sin(rot), 0], [np.sin(rot), np.cos(rot), 0], [0, 0, 1]])
        R = Rz @ Rt
        Kc = np.array([[f, 0, width / 2.0], [0, f, height / 2.0], [0, 0, 1]])
        M = Kc @ np.column_stack([R[:, 0], R[:, 1], np.array([0, 0, f])])
        A = np.array([[s, 0, -s * side / 2.0], [0, s, -s * side / 2.0], [0, 0, 1]])
        H = M @ A
        H = H / H[2, 2]
        corners = np.array([[0, 0, 1], [side, 0, 1], [side, side, 1], [0, side, 1]], np.float64).T
        q = H @ corners
        u, v = q[0] / q[2], q[1] / q[2]
        if (u > 2).all() and (u < width - 3).all() and (v > 2).all() and (v < height - 3).all():
            return H
    raise RuntimeError("no view keeps the layout inside the frame")


def radial(u, v, width, height, k1):
    """Radial distortion about the frame centre: p -> c + (p - c)(1 + k1 r^2), r = |p - c| / the half-diagonal."""
    cx, cy, R = width / 2.0, height / 2.0, np.hypot(width, height) / 2.0
    dx, dy = u - cx, v - cy
    g = 1 + k1 * (dx * dx + dy * dy) / (R * R)
    return cx + dx * g, cy + dy * g


def _unradial(ud, vd, width, height, k1, rounds=8):
    """The inverse of radial() by fixed-point rounds (|k1| small)."""
    cx, cy, R = width / 2.0, height / 2.0, np.hypot(width, height) / 2.0
    u, v = ud.copy(), vd.copy()
    for _ in range(rounds):
        dx, dy = u - cx, v - cy
        g = 1 + k1 * (dx * dx + dy * dy) / (R * R)
        u, v = cx + (ud - cx) / g, cy + (vd - cy) / g
    return u, v


def homography_4(src, dst):
    """The homography (h33 = 1) taking four points src to dst (each 4 x 2), by the 8 x 8 linear system."""
    A, b = [], []
    for (x, y), (u, v) in zip(src, dst):
        A.append([x, y, 1, 0, 0, 0, -u * x, -u * y]); b.append(u)
        A.append([0, 0, 0, x, y, 1, -v * x, -v * y]); b.append(v)
    h = np.linalg.solve(np.array(A, np.float64), np.array(b, np.float64))
    return np.append(h, 1.0)


def distorted_capture(fmt, grey, width, height, H, k1=0.0, blur=0.0, sigma=3.0, rng=None, mid=128, gamma=2.2):
    """A capture through a real lens: the n x n grey picture inside its light layout, seen through the view H (module
    -> ideal image), radial distortion k1 about the frame centre, a Gaussian blur of `blur` pixels in linear light
    (grey -> (g / 255)^gamma -> blur -> ^(1 / gamma)), AWGN of sigma grey levels, 8 bits. Returns (luma, the plain
    registration: the homography through the layout's four corners as the camera sees them, then a zero node mesh)."""
    from scipy.ndimage import gaussian_filter
    n, span = fmt.n, fmt.span
    pxm = n / span
    side = span + 30
    px = int(round(side * pxm))
    drive = np.full((px, px), 255.0)
    o = int(round(15 * pxm))
    drive[o:o + n, o:o + n] = grey
    Hm = np.asarray(H, np.float64).reshape(3, 3)
    Hi = np.linalg.inv(Hm)
    V, U = np.mgrid[0:height, 0:width].astype(np.float64)
    ui, vi = _unradial(U.ravel() + 0.5, V.ravel() + 0.5, width, height, k1)
    q = Hi @ np.stack([ui, vi, np.ones(ui.size)])
    mx, my = q[0] / q[2], q[1] / q[2]
    sx, sy = mx * pxm - 0.5, my * pxm - 0.5
    inside = (sx >= 0) & (sy >= 0) & (sx <= px - 1.001) & (sy <= px - 1.001)
    x0 = np.clip(np.floor(sx).astype(np.int64), 0, px - 2)
    y0 = np.clip(np.floor(sy).astype(np.int64), 0, px - 2)
    fx, fy = np.clip(sx - x0, 0, 1), np.clip(sy - y0, 0, 1)
    val = (drive[y0, x0] * (1 - fx) + drive[y0, x0 + 1] * fx) * (1 - fy) + (drive[y0 + 1, x0] * (1 - fx) + drive[y0 + 1, x0 + 1] * fx) * fy
    img = np.where(inside, val, float(mid)).reshape(height, width)
    if blur > 0:
        lin = (img / 255.0) ** gamma
        img = 255.0 * np.clip(gaussian_filter(lin, blur, mode="nearest"), 0, 1) ** (1.0 / gamma)
    rng = np.random.default_rng(0) if rng is None else rng
    luma = np.clip(np.rint(img + sigma * rng.standard_normal(img.shape)), 0, 255).astype(np.uint8)
    corners = np.array([[0, 0], [side, 0], [side, side], [0, side]], np.float64)
    qc = Hm @ np.column_stack([corners, np.ones(4)]).T
    cu, cv = radial(qc[0] / qc[2], qc[1] / qc[2], width, height, k1)
    Hp = homography_4(corners, np.column_stack([cu, cv]))
    nn = layout_nodes(span).size
    reg = np.concatenate([Hp.astype(np.float32), np.zeros(2 * nn * nn, np.float32)])
    return luma, reg


# ---------------------------------------------------------------- the border and its format word

CELL_DATA, CELL_LIGHT, CELL_DARK, CELL_WORD = 0, 1, 2, 8


def _gf():
    exp, log = np.zeros(512, np.int64), np.zeros(256, np.int64)
    x = 1
    for i in range(255):
        exp[i], log[x] = x, i
        x <<= 1
        if x & 256:
            x ^= 0x11D
    exp[255:] = exp[:257]
    return exp, log


_EXP, _LOG = _gf()


def _gmul(a, b):
    return int(_EXP[_LOG[a] + _LOG[b]]) if a and b else 0


def rs_encode(data, nroots):
    """Reed-Solomon parity over GF(256) (polynomial 0x11d, roots alpha^0 .. alpha^(nroots - 1)), systematic, as
    liblizard/src/rs.c:19-35 computes it: the data bytes then nroots parity bytes."""
    g = [1] + [0] * nroots
    for i in range(nroots):
        for j in range(i + 1, 0, -1):
            g[j] ^= _gmul(g[j - 1], int(_EXP[i]))
    par = [0] * nroots
    for d in data:
        fb = d ^ par[0]
        par = par[1:] + [0]
        if fb:
            par = [p ^ _gmul(fb, g[j + 1]) for j, p in enumerate(par)]
    return bytes(list(data) + par)


def fmt_geometry(span):
    """Word cells a side and the codeword's bytes for a ring of span modules (border side span + 30;
    liblizard/src/fmt.c:6-20, layout.c:66)."""
    side = span + 30
    thin = (side - 30) // 2 if side > 30 else 0
    cells = thin // 8 * 4
    cells = cells if cells >= 32 else 0
    return cells, min(64, 4 * (cells // 8))


def fmt_word(version, fps, span):
    """The format word a sender paints (liblizard/src/fmt.c:32-41): magic 0x4c, version, fps, RS parity."""
    _, nbytes = fmt_geometry(span)
    return rs_encode([0x4C, version, fps], nbytes - 3)


def track_bit(side, j):
    """Whether track cell j of a side is dark (liblizard/src/layout.c:57-61)."""
    v = ((side * 4099 + (j >> 1)) * 2654435761 + 40503) & 0xFFFFFFFF
    v ^= v >> 15
    v = (v * 2246822519) & 0xFFFFFFFF
    v ^= v >> 13
    return (v ^ j) & 1


def border_kind(span, cw=None):
    """The layout's cell kinds, side x side modules (CELL_DATA / LIGHT / DARK, | CELL_WORD on word cells): the corner
    marks, the line, the timing track and the word's cells (liblizard/src/layout.c:69-141, thin_init, thin_corner,
    ob_layout_set_fmt). cw: the word's codeword (None: the word cells light)."""
    side = span + 30
    S, reserve, margin = 12, 15, 15
    y, x = np.mgrid[0:side, 0:side]
    dx, dy = np.minimum(x, side - 1 - x), np.minimum(y, side - 1 - y)
    d = np.minimum(dx, dy)
    kind = np.where(d >= margin - 3, CELL_DATA, CELL_LIGHT).astype(np.uint8)
    kind[(d >= 1) & (d <= 2) & (d < margin - 3)] = CELL_DARK
    horiz = dy <= dx
    along = np.where(horiz, x, y)
    sidev = np.where(horiz, np.where(y < side // 2, 0, 2), np.where(x < side // 2, 3, 1))
    band = (d >= 5) & (d < 7) & (along >= reserve) & (along < side - reserve)
    cell = (along - reserve) // 2
    run = cell // 4
    for yy, xx in zip(*np.nonzero(band & (run % 2 == 0))):
        if track_bit(int(sidev[yy, xx]), int(run[yy, xx] // 2 * 4 + cell[yy, xx] % 4)):
            kind[yy, xx] = CELL_DARK
    # the corner marks: a solid square, its outer and inner rings light, the gap band light
    cx, cy = dx, dy
    corner = (cx < S) & (cy < S)
    inner = (cx >= 1) & (cx <= S - 2) & (cy >= 1) & (cy <= S - 2)
    cd = np.minimum(cx, cy)
    kind[corner] = np.where(inner & ~((cd >= 3) & (cd < 5)), CELL_DARK, CELL_LIGHT)[corner]
    cells, nbytes = fmt_geometry(span)
    for s in range(4):
        for i in range(cells):
            k = 4 * (i >> 3) + s
            bit = (cw[k] >> (7 - (i & 7))) & 1 if cw is not None and k < nbytes else 0
            v = (CELL_DARK if bit else CELL_LIGHT) | CELL_WORD
            off = ((i // 4) * 8 + i % 4 + 4) * 2
            for j in range(2):
                for e in range(2):
                    t, dd = reserve + off + j, 5 + e
                    xx = t if s in (0, 2) else (dd if s == 3 else side - 1 - dd)
                    yy = dd if s == 0 else (side - 1 - dd if s == 2 else t)
                    kind[yy, xx] = v
    return kind


def border_drive(span, pxm, cw, picture=None):
    """The symbol's drive in grey levels at pxm pixels a module: the border's dark cells 0, its light cells 255
    (liblizard/src/lizard_phy.c:1155-1163), the picture (n x n at exact-copy scale) inside when given, else white."""
    kind = border_kind(span, cw)
    side = span + 30
    drive = np.where((kind & 3) == CELL_DARK, 0.0, 255.0).repeat(pxm, 0).repeat(pxm, 1)
    if picture is not None:
        n = picture.shape[0]
        o = 15 * pxm
        drive[o:o + n, o:o + n] = picture
    return drive


def render_drive(drive, pxm, width, height, H, k1=0.0, blur=0.0, sigma=3.0, rng=None, mid=128, gamma=2.2, glare=None):
    """A capture of a drive (pxm pixels a module) through the view H (module -> ideal image), radial k1 about the frame
    centre, blur in linear light, AWGN; glare: (u0, v0, radius, strength) a bright disc added in linear light over
    part of the frame. Returns luma."""
    from scipy.ndimage import gaussian_filter
    px = drive.shape[0]
    Hi = np.linalg.inv(np.asarray(H, np.float64).reshape(3, 3))
    V, U = np.mgrid[0:height, 0:width].astype(np.float64)
    ui, vi = _unradial(U.ravel() + 0.5, V.ravel() + 0.5, width, height, k1)
    q = Hi @ np.stack([ui, vi, np.ones(ui.size)])
    sx, sy = q[0] / q[2] * pxm - 0.5, q[1] / q[2] * pxm - 0.5
    inside = (sx >= 0) & (sy >= 0) & (sx <= px - 1.001) & (sy <= px - 1.001)
    x0 = np.clip(np.floor(sx).astype(np.int64), 0, px - 2)
    y0 = np.clip(np.floor(sy).astype(np.int64), 0, px - 2)
    fx, fy = np.clip(sx - x0, 0, 1), np.clip(sy - y0, 0, 1)
    val = (drive[y0, x0] * (1 - fx) + drive[y0, x0 + 1] * fx) * (1 - fy) + (drive[y0 + 1, x0] * (1 - fx) + drive[y0 + 1, x0 + 1] * fx) * fy
    img = np.where(inside, val, float(mid)).reshape(height, width)
    lin = (img / 255.0) ** gamma
    if blur > 0:
        lin = gaussian_filter(lin, blur, mode="nearest")
    if glare is not None:
        gu, gv, gr, gs = glare
        lin = lin + gs * np.exp(-((U - gu) ** 2 + (V - gv) ** 2) / (2.0 * gr * gr))
    img = 255.0 * np.clip(lin, 0, 1) ** (1.0 / gamma)
    rng = np.random.default_rng(0) if rng is None else rng
    return np.clip(np.rint(img + sigma * rng.standard_normal(img.shape)), 0, 255).astype(np.uint8)


def word_capture(span, pxm, version, fps, width, height, rng, rot_deg=12.0, tilt=0.0003, scale=(0.85, 1.05), blur=0.0,
                 sigma=3.0, glare=None, mesh=0.0):
    """A capture of a symbol's border carrying the format word (version, fps) of a ring of span modules, at pxm pixels
    a module, under a random view; returns (luma, registration: H then the node mesh's (dx, dy), each node displaced
    by up to `mesh` pixels, a registration that far off; the codeword)."""
    side = span + 30
    cw = fmt_word(version, fps, span)
    drive = border_drive(span, pxm, cw)
    th = np.deg2rad(rng.uniform(-rot_deg, rot_deg))
    s = rng.uniform(*scale) * min(width, height) * 0.9 / side
    c, sn = np.cos(th) * s, np.sin(th) * s
    A = np.array([[c, -sn], [sn, c]])
    ctr = A @ np.array([side / 2.0, side / 2.0])
    H = np.array([[c, -sn, width / 2.0 - ctr[0]], [sn, c, height / 2.0 - ctr[1]],
                  [rng.uniform(-tilt, tilt), rng.uniform(-tilt, tilt), 1.0]])
    luma = render_drive(drive, pxm, width, height, H, blur=blur, sigma=sigma, rng=rng, glare=glare)
    nn = layout_nodes(span).size
    reg = np.concatenate([(H / H[2, 2]).astype(np.float32).ravel(), np.zeros(2 * nn * nn, np.float32)])
    if mesh > 0:
        reg[9:] = rng.uniform(-mesh, mesh, 2 * nn * nn).astype(np.float32)
    return luma, reg, cw


# ---------------------------------------------------------------- the sender's drive

def pxm_for(n, span):
    """Whole pixels a module the ring is painted at (liblizard/src/lizard_phy.c:1497-1501)."""
    return int(np.ceil(np.float32(n) / np.float32(span) - np.float32(1e-4)))


def _lanczos3(x):
    x = abs(x)
    if x >= 3:
        return 0.0
    px = np.pi * x
    return 3 * np.sin(px) * np.sin(px / 3) / (px * px)


def resample_taps(n, span, pxm, cp=3):
    """The Lanczos-3 resampler's taps from the picture's n samples to the ring's pixels (liblizard/src/lizard_phy.c:
    962-1025 resample_init): for each of q = (span + 2 cp) pxm pixels its first tap i0 and six float weights."""
    q = (span + 2 * cp) * pxm
    sc = n / span
    i0 = np.zeros(q, np.int64)
    w = np.zeros((q, 6), np.float32)
    for x in range(q):
        u = (x + 0.5) * sc / pxm - cp * sc - 0.5
        r = np.floor(u + 0.5)
        if abs(u - r) < 1e-6:
            i0[x] = int(r) - 2
            w[x, 2] = 1.0
            continue
        a = int(np.floor(u)) - 2
        tw = np.array([_lanczos3(u - (a + t)) for t in range(6)])
        i0[x] = a
        w[x] = (tw / tw.sum()).astype(np.float32)
    return i0, w


def picture_float(fmt, block_rows, parity=0):
    """The picture before painting, n x n floats in 0..1 (liblizard/src/lizard_phy.c:1134-1199): the QPSK spectrum's
    Hermitian inverse in double, clipped and mapped as the sender does in float."""
    n = fmt.n
    sb = slots(fmt, block_rows, parity)
    a = np.float32(0.70710678)
    sym = np.where(sb[0::2], -a, a).astype(np.float64) + 1j * np.where(sb[1::2], -a, a).astype(np.float64)
    S = np.zeros((n, n), np.complex128)
    u, v = fmt.uv[0::2].astype(np.int64), fmt.uv[1::2].astype(np.int64)
    S[v, (u + n) % n] = sym
    z = 2.0 * np.real(np.fft.ifft2(S)) * (n * n)
    lim = np.float32(2.0 * 2.0 * np.sqrt(np.float32(0.5 * fmt.subch * SUB)))
    sc = np.float32(0.5) / lim
    return (np.float32(0.5) + np.clip(z.astype(np.float32), -lim, lim) * sc).astype(np.float32)


def encode_drive(fmt, block_rows, parity=0, fps=0):
    """The sender's drive and its grey page (liblizard/src/lizard_phy.c:1087-1236 lizard_encode, :700-716
    lizard_paint_grey): the border's cells 0 or 1 at pxm pixels a module (its format word for version subch / 16 at
    fps), the picture resampled onto the ring's pixels over the picture and its 3-module guard (the picture periodic),
    each pass six weights in order, clamped to 0..1; the anchors' squares over it; then round(drive 255) inside a
    2-module white margin. Returns (drive px x px float32, grey W x W uint8)."""
    n, span = fmt.n, fmt.span
    pxm = pxm_for(n, span)
    side = span + 30
    px = side * pxm
    cp = 3
    pic = picture_float(fmt, block_rows, parity)
    kind = border_kind(span, fmt_word(fmt.subch // 16, fps, span) if fmt.subch % 16 == 0 else None)
    drive = np.where((kind & 3) == CELL_DARK, 0.0, 1.0).astype(np.float32).repeat(pxm, 0).repeat(pxm, 1)
    i0, w = resample_taps(n, span, pxm, cp)
    q, o = i0.size, (15 - cp) * pxm
    rows = (i0[:, None] + np.arange(6)[None, :]) % n            # q x 6 picture rows
    tmp = np.zeros((q, n), np.float32)
    for t in range(6):
        tmp = (tmp + w[:, t:t + 1] * pic[rows[:, t]]).astype(np.float32) if t else (w[:, 0:1] * pic[rows[:, 0]]).astype(np.float32)
    cols = (i0[:, None] + np.arange(6)[None, :]) % n            # q x 6 picture columns
    out = np.zeros((q, q), np.float32)
    for t in range(6):
        term = (tmp[:, cols[:, t]] * w[None, :, t]).astype(np.float32)
        out = (out + term).astype(np.float32) if t else term
    drive[o:o + q, o:o + q] = np.clip(out, 0, 1)
    a = span // 64
    sidep = a * pxm
    half = np.float32(0.5 * sidep)
    ii = np.arange(sidep, dtype=np.float32) + np.float32(0.5) - half
    dd = np.maximum(np.abs(ii)[None, :], np.abs(ii)[:, None]) / half
    pat = np.where((dd < 0.25) | (dd >= 0.6), 1.0, 0.0).astype(np.float32)
    for j in range(7):
        for i in range(7):
            x0 = int(np.floor(15 + span * (i + 0.5) / 7 - a / 2.0 + 0.5)) * pxm
            y0 = int(np.floor(15 + span * (j + 0.5) / 7 - a / 2.0 + 0.5)) * pxm
            drive[y0:y0 + sidep, x0:x0 + sidep] = pat
    m = 2 * pxm
    W = px + 2 * m
    grey = np.full((W, W), 255, np.uint8)
    t = drive.astype(np.float32) * np.float32(255.0) + np.float32(0.5)
    grey[m:m + px, m:m + px] = np.clip(np.floor(t), 0, 255).astype(np.uint8)
    return drive, grey
