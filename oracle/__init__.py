"""Python face of the oracle (TEST INFRASTRUCTURE ONLY: tests, the smoke check and the benchmark's CPU-baseline leg).

`port()` is the plain-C restatement (oracle/_build/liboracle.so, built by `make -C oracle`); `ref()` is the
reference codec compiled from its own sources (oracle/_ref/libref.so, `make -C oracle ref`), present only where the
reference tree was available to build it. Neither is ever used by the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
REF_SCALAR_PATH = os.path.join(HERE, "_ref", "libref_scalar.so")
REF_DEVELOP_PATH = os.path.join(HERE, "_ref", "libref_develop.so")
# The reference tree's root is LIZARD_REF (default /root/reference); the tests pinned to the reference skip where it
# is absent or not built.
REF_ROOT = os.environ.get("LIZARD_REF", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "liblizard", "src")

_port = None
_ref = None
_ref_scalar = None
_ref_develop = None


class Code(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in "rate z mb kb n k m np nt edges".split()] + [
        ("rowptr", ctypes.c_int * 31), ("col", ctypes.c_int * 160), ("shift", ctypes.c_int * 160)]


def build(ref=True):
    """make the restatement, and the reference where its sources are present."""
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)
    if ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref", "LIZARD_REF=" + REF_ROOT], check=True)


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            build(ref=False)
        L = ctypes.CDLL(PORT_PATH)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.orc_code_init.argtypes = [P, I]
        L.orc_h_hash.argtypes = [P]
        L.orc_h_hash.restype = ctypes.c_uint32
        L.orc_ldpc_encode.argtypes = [P, P, P]
        L.orc_ldpc_decode.argtypes = [P, P, P, I, I, F]
        L.orc_crc32c.argtypes = [P, I]
        L.orc_crc32c.restype = ctypes.c_uint32
        L.orc_ldpc_batch.argtypes = [P, P, P, I, I, I, F, P, P, P, I]
        L.orc_anchor_find.argtypes = [I, P, I, I, P, P, P, P, P, P, P, P, P]
        L.orc_lens_fit.argtypes = [I, I, I, P, P, P, P, P]
        L.orc_anchor_register.argtypes = [I, P, P, I, I, P, P, F, P, P, P, P, P, P, P]
        U = ctypes.c_uint32
        L.orc_ingest_pixels.argtypes = [P, I, I, I, I, P]
        L.orc_gamma_lut.argtypes = [P]
        L.orc_develop.argtypes = [I, P, U, U, U, U, U, P, U, U, U, U, P, ctypes.c_size_t]
        _port = L
    return _port


def have_ref():
    return os.path.exists(REF_PATH)


def ref():
    """The reference compiled from its sources, or None where it could not be built here."""
    global _ref
    if _ref is None and have_ref():
        L = ctypes.CDLL(REF_PATH)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_crc32c.argtypes = [P, I]
        L.ref_crc32c.restype = ctypes.c_uint32
        L.ref_ldpc_shape.argtypes = [I, P]
        L.ref_ldpc_encode.argtypes = [I, P, P]
        L.ref_ldpc_decode_many.argtypes = [I, P, I, P, P, I, I, F]
        L.ref_ldpc_batch.argtypes = [P, P, P, I, I, I, F, P, P, P, I]
        _ref = L
    return _ref


def ref_scalar():
    """The reference's portable build (-DOB_SCALAR) with the anchor search's harness, or None where it could not be
    built here."""
    global _ref_scalar
    if _ref_scalar is None and os.path.exists(REF_SCALAR_PATH):
        L = ctypes.CDLL(REF_SCALAR_PATH)
        P, I = ctypes.c_void_p, ctypes.c_int
        L.refs_anchor_find.argtypes = [I, P, I, I, P, P, P, P, P, P, P, P, P]
        L.refs_anchor_model.argtypes = [I, I, I, P, P, P, P, P]
        L.refs_anchor_register.argtypes = [I, P, P, I, I, P, P, ctypes.c_float, P, P, P, P, P, P, P]
        _ref_scalar = L
    return _ref_scalar


def ref_develop():
    """The reference's own camera develop (develop.cpp) compiled here, or None where it could not be built."""
    global _ref_develop
    if _ref_develop is None and os.path.exists(REF_DEVELOP_PATH):
        L = ctypes.CDLL(REF_DEVELOP_PATH)
        P, I, U = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32
        L.refd_develop.argtypes = [I, P, U, U, U, U, U, P, U, U, U, U, P, ctypes.c_size_t]
        L.refd_gamma_lut.argtypes = [P]
        _ref_develop = L
    return _ref_develop


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def develop(lib, fn, fmt, plane, row_stride, pixel_stride, x0, y0, bin_, levels, ox, oy, w, h):
    """One develop through lib.fn (orc_develop or refd_develop): w x h luma bytes."""
    plane = np.ascontiguousarray(plane, np.uint8)
    lv = np.ascontiguousarray(levels, np.float32)
    out = np.zeros((h, w), np.uint8)
    rc = getattr(lib, fn)(fmt, _p(plane), row_stride, pixel_stride, x0, y0, bin_, _p(lv), ox, oy, w, h, _p(out), w)
    assert rc == 0
    return out


def lens_fit(lib, fn, span, iw, ih, H, ok, dx, dy):
    """The lens model from one frame's anchors through lib.fn (orc_lens_fit or refs_anchor_model): (fit, lens[15])."""
    Hf = np.ascontiguousarray(H, np.float32).ravel()[:9]
    ok, dx, dy = (np.ascontiguousarray(a, t) for a, t in ((ok, np.uint8), (dx, np.float32), (dy, np.float32)))
    lens = np.zeros(15, np.float64)
    fit = getattr(lib, fn)(span, iw, ih, _p(Hf), _p(ok), _p(dx), _p(dy), _p(lens))
    return fit, lens


def anchor_find(lib, fn, span, luma, H, lens=None, ok_in=None):
    """One frame's anchor search through lib.fn (the oracle's orc_anchor_find or the reference's refs_anchor_find):
    a dict of 49-entry arrays ok, peak, dx, dy, u, v, and found."""
    luma = np.ascontiguousarray(luma, np.uint8)
    h, w = luma.shape
    Hf = np.ascontiguousarray(H, np.float32).ravel()[:9]
    ln = None if lens is None else np.ascontiguousarray(lens, np.float64)
    oi = None if ok_in is None else np.ascontiguousarray(ok_in, np.uint8)
    out = {"ok": np.zeros(49, np.uint8)}
    for k in ("peak", "dx", "dy", "u", "v"):
        out[k] = np.zeros(49, np.float32)
    out["found"] = getattr(lib, fn)(span, _p(luma), w, h, _p(Hf), None if ln is None else _p(ln), None if oi is None else _p(oi),
                                    _p(out["ok"]), _p(out["peak"]), _p(out["dx"]), _p(out["dy"]), _p(out["u"]), _p(out["v"]))
    return out


def anchor_register(lib, fn, span, luma, H, quad, mpx, rim=None):
    """The code registered from the anchors through lib.fn (the oracle's orc_anchor_register or the reference's
    refs_anchor_register): a dict with held, H (9), quad (8), lens (15) and the 49-entry arrays ok, peak, dx, dy, u, v."""
    luma = np.ascontiguousarray(luma, np.uint8)
    h, w = luma.shape
    rm = None if rim is None else np.ascontiguousarray(rim, np.uint8)
    out = {"H": np.ascontiguousarray(H, np.float32).ravel()[:9].copy(), "quad": np.ascontiguousarray(quad, np.float32).ravel()[:8].copy(),
           "lens": np.zeros(15, np.float64), "ok": np.zeros(49, np.uint8)}
    for k in ("peak", "dx", "dy", "u", "v"):
        out[k] = np.zeros(49, np.float32)
    out["held"] = getattr(lib, fn)(span, _p(luma), None if rm is None else _p(rm), w, h, _p(out["H"]), _p(out["quad"]), float(mpx), _p(out["ok"]),
                                   _p(out["peak"]), _p(out["dx"]), _p(out["dy"]), _p(out["u"]), _p(out["v"]), _p(out["lens"]))
    return out


def code(rate):
    c = Code()
    if port().orc_code_init(ctypes.byref(c), rate):
        raise ValueError("no code at rate index %d" % rate)
    return c


def h_hash(rate):
    c = code(rate)
    return int(port().orc_h_hash(ctypes.byref(c)))


def crc32c(data):
    b = np.frombuffer(bytes(data), np.uint8).copy()
    return int(port().orc_crc32c(_p(b), b.size))


def ldpc_encode(rate, data):
    c = code(rate)
    data = np.ascontiguousarray(data, np.uint8)
    cw = np.zeros(c.n, np.uint8)
    port().orc_ldpc_encode(ctypes.byref(c), _p(data), _p(cw))
    return cw


def ldpc_decode(rate, llr, max_iter, stall_it=0, stall_ratio=0.0):
    c = code(rate)
    llr = np.ascontiguousarray(llr, np.int8)
    out = np.zeros(c.n, np.uint8)
    its = port().orc_ldpc_decode(ctypes.byref(c), _p(llr), _p(out), max_iter, stall_it, stall_ratio)
    return its, out


def ldpc_batch(lib, llr, offsets, rates, max_iter, stall_it, stall_ratio, threads=1):
    """The mixed-rate batch through the port (lib=port()) or the reference (lib=ref()): (packed bits, its, ok)."""
    llr = np.ascontiguousarray(llr, np.int8)
    offsets = np.ascontiguousarray(offsets, np.int64)
    rates = np.ascontiguousarray(rates, np.int32)
    bits = np.zeros(llr.size // 8, np.uint8)
    its = np.zeros(rates.size, np.int32)
    ok = np.zeros(rates.size, np.uint8)
    fn = lib.orc_ldpc_batch if hasattr(lib, "orc_ldpc_batch") else lib.ref_ldpc_batch
    rc = fn(_p(llr), _p(offsets), _p(rates), rates.size, max_iter, stall_it, stall_ratio, _p(bits), _p(its), _p(ok), threads)
    if rc:
        raise RuntimeError("oracle batch failed")
    return bits, its, ok


# ------------------------------------------------------------------ the receiver

SUB = 320


def _phy_sigs(L):
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.orc_fmt_new.argtypes = [I, I, I]
    L.orc_fmt_new.restype = P
    L.orc_fmt_free.argtypes = [P]
    L.orc_tiers_for.argtypes = [I, P, P, P]
    L.orc_fmt_info.argtypes = [P, P]
    L.orc_fmt_tables.argtypes = [P, P, P, P, P, P, P, P]
    L.orc_fmt_perm.argtypes = [P, I, P]
    L.orc_spectrum.argtypes = [P, P, P, P]
    L.orc_pilot_align.argtypes = [P, P, P]
    L.orc_demap.argtypes = [P, P, P, P, P, P]
    L.orc_blocks.argtypes = [P, P, P, P, P, P, I, P, P, P, P, P]
    L.orc_layout_nodes.argtypes = [I, P]
    L.orc_sample_grid.argtypes = [I, I, P, I, I, I, P, P]
    L.orc_sample_decode.argtypes = [I, I, P, I, I, I, P, P, P]


class Fmt:
    """The oracle's restatement of one format (n, subch, span)."""

    def __init__(self, n, subch, span=128):
        L = port()
        if not hasattr(L, "_phy"):
            _phy_sigs(L)
            L._phy = True
        self.L = L
        self.h = L.orc_fmt_new(n, subch, span)
        if not self.h:
            raise ValueError("no format at n=%d subch=%d span=%d" % (n, subch, span))
        info = np.zeros(20, np.int32)
        L.orc_fmt_info(self.h, _p(info))
        self.n, self.subch, self.span, self.blocks, self.used, self.bw, self.vblocks, self.tiers = (int(x) for x in info[:8])
        self.tier = [(int(info[8 + 3 * t]), int(info[9 + 3 * t]), int(info[10 + 3 * t])) for t in range(self.tiers)]
        need = self.subch * SUB
        self.pos = np.zeros(need, np.int32)
        self.uv = np.zeros(2 * need, np.int16)
        self.white = np.zeros(2 * need, np.uint8)
        self.block_tier = np.zeros(self.blocks, np.int32)
        self.block_slot = np.zeros(self.blocks, np.int32)
        self.erase = np.zeros(14, np.int32)
        self.hole_inv = np.zeros(36, np.float64)
        L.orc_fmt_tables(self.h, _p(self.pos), _p(self.uv), _p(self.white), _p(self.block_tier), _p(self.block_slot), _p(self.erase), _p(self.hole_inv))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_fmt_free(self.h)
            self.h = None

    def perm(self, t):
        out = np.zeros(7680, np.int32)
        nt = self.L.orc_fmt_perm(self.h, t, _p(out))
        return out[:nt]

    def spectrum(self, grid):
        """FP64 detrended spectrum (complex128, pos order) of a row-major n x n grid (grey / 255); also the erased grid
        and the 5 projections."""
        g = np.ascontiguousarray(grid, np.float32).copy()
        coef = np.zeros(2 * self.subch * SUB, np.float64)
        proj = np.zeros(5, np.float64)
        self.L.orc_spectrum(self.h, _p(g), _p(coef), _p(proj))
        return coef[0::2] + 1j * coef[1::2], g, proj

    def pilot_align(self, coef):
        c = np.ascontiguousarray(coef, np.float32)
        d = np.zeros(2, np.float32)
        used = self.L.orc_pilot_align(self.h, _p(c), _p(d))
        return d, used

    def demap(self, coef, turn=None):
        """coef: float32 pairs (2 a coefficient, pos order). Returns (llrf int8, sub_est float64, sub_rms float32)."""
        c = np.ascontiguousarray(coef, np.float32)
        llrf = np.zeros(2 * self.subch * SUB, np.int8)
        est = np.zeros(self.subch, np.float64)
        rms = np.zeros(self.subch, np.float32)
        t = None if turn is None else np.ascontiguousarray(turn, np.float32)
        self.L.orc_demap(self.h, _p(c), None if t is None else _p(t), _p(llrf), _p(est), _p(rms))
        return llrf, est, rms

    def blocks_stage(self, llrf, est, rms, coef, turn=None, max_iter=30):
        c = np.ascontiguousarray(coef, np.float32)
        blocks = np.zeros((self.blocks, 476), np.uint8)
        ok = np.zeros(self.blocks, np.uint8)
        its = np.zeros(self.blocks, np.int8)
        best = np.zeros(self.blocks, np.float32)
        pil = np.zeros(self.blocks, np.float32)
        t = None if turn is None else np.ascontiguousarray(turn, np.float32)
        self.L.orc_blocks(self.h, _p(np.ascontiguousarray(llrf, np.int8)), _p(np.ascontiguousarray(est, np.float64)),
                          _p(np.ascontiguousarray(rms, np.float32)), _p(c), None if t is None else _p(t), max_iter,
                          _p(blocks), _p(ok), _p(its), _p(best), _p(pil))
        return {"blocks": blocks, "ok": ok, "its": its, "est": best, "pilot": pil}

    def sample(self, luma, reg):
        """The picture grid (n x n float32) of a luma frame through a registration (H then the mesh)."""
        luma = np.ascontiguousarray(luma, np.uint8)
        h, w = luma.shape
        g = np.zeros(self.n * self.n, np.float32)
        self.L.orc_sample_grid(self.n, self.span, _p(luma), w, h, w, _p(np.ascontiguousarray(reg, np.float32)), _p(g))
        return g.reshape(self.n, self.n)

    def sample_decode(self, luma, reg):
        """The grid as the x86-64 decode samples it (strips of 64 columns, the integer read) and the shading fit's
        samples: (grid n x n, shade n/8 x n/8)."""
        luma = np.ascontiguousarray(luma, np.uint8)
        h, w = luma.shape
        g = np.zeros(self.n * self.n, np.float32)
        c = self.n // 8
        s = np.zeros(c * c, np.float32)
        self.L.orc_sample_decode(self.n, self.span, _p(luma), w, h, w, _p(np.ascontiguousarray(reg, np.float32)), _p(g), _p(s))
        return g.reshape(self.n, self.n), s.reshape(c, c)

    def receive(self, grid, fp64_spectrum=True):
        """The whole finish on a grid: spectrum (FP64, narrowed to float), pilots, soft values, blocks."""
        spec, _, _ = self.spectrum(grid)
        coef = np.empty(2 * spec.size, np.float32)
        coef[0::2] = spec.real
        coef[1::2] = spec.imag
        d, used = self.pilot_align(coef)
        turn = d if (used and (d[0] != 0 or d[1] != 0)) else None
        llrf, est, rms = self.demap(coef, turn)
        out = self.blocks_stage(llrf, est, rms, coef, turn)
        out.update({"coef": coef, "llrf": llrf, "sub_est": est, "sub_rms": rms, "align": d if turn is not None else np.zeros(2, np.float32)})
        return out


class RefFmt:
    """The reference codec at one format (only where oracle/_ref was built)."""

    def __init__(self, n, subch, span=128):
        L = ref()
        if L is None:
            raise RuntimeError("the reference is not built here")
        if not hasattr(L, "_phy"):
            P, I = ctypes.c_void_p, ctypes.c_int
            L.ref_fmt_new.argtypes = [I, I, I]
            L.ref_fmt_new.restype = P
            L.ref_fmt_free.argtypes = [P]
            L.ref_fmt_info.argtypes = [P, P]
            L.ref_fmt_tables.argtypes = [P, P, P, P, P, P, P]
            L.ref_fmt_perm.argtypes = [P, I, P]
            L.ref_encode.argtypes = [P, P, I, P, P]
            L.ref_finish_grid.argtypes = [P] + [P] * 11
            L.ref_decode_frame.argtypes = [P, P, I, I, P, P, P, P, P, P]
            L.ref_sample_grid.argtypes = [P, P, I, I, P, I, P]
            L.ref_sample_decode.argtypes = [P, P, I, I, P, P, P]
            L._phy = True
        self.L = L
        self.h = L.ref_fmt_new(n, subch, span)
        if not self.h:
            raise ValueError("no format")
        info = np.zeros(21, np.int32)
        L.ref_fmt_info(self.h, _p(info))
        self.n, self.subch, self.blocks, self.used, self.bw, self.vblocks, self.tiers, self.pxm, self.px = (int(x) for x in info[:9])
        self.tier = [(int(info[9 + 3 * t]), int(info[10 + 3 * t]), int(info[11 + 3 * t])) for t in range(self.tiers)]

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_fmt_free(self.h)
            self.h = None

    def tables(self):
        need = self.subch * SUB
        pos = np.zeros(need, np.int32)
        white = np.zeros(2 * need, np.uint8)
        bt = np.zeros(self.blocks, np.int32)
        bs = np.zeros(self.blocks, np.int32)
        er = np.zeros(14, np.int32)
        hi = np.zeros(36, np.float64)
        self.L.ref_fmt_tables(self.h, _p(pos), _p(white), _p(bt), _p(bs), _p(er), _p(hi))
        return {"pos": pos, "white": white, "block_tier": bt, "block_slot": bs, "erase": er, "hole_inv": hi}

    def perm(self, t):
        out = np.zeros(7680, np.int32)
        nt = self.L.ref_fmt_perm(self.h, t, _p(out))
        return out[:nt]

    def encode(self, blocks, c=0):
        """(drive px x px float32, grey W x W uint8)."""
        blocks = np.ascontiguousarray(blocks, np.uint8)
        drive = np.zeros(self.px * self.px, np.float32)
        W = self.px + 4 * self.pxm
        grey = np.zeros(W * W, np.uint8)
        self.L.ref_encode(self.h, _p(blocks), c, _p(drive), _p(grey))
        return drive.reshape(self.px, self.px), grey.reshape(W, W)

    def finish_grid(self, grid):
        g = np.ascontiguousarray(grid, np.float32)
        need = self.subch * SUB
        out = {"coef": np.zeros(2 * need, np.float32), "llrf": np.zeros(2 * need, np.int8), "sub_est": np.zeros(self.subch, np.float64),
               "sub_rms": np.zeros(self.subch, np.float32), "align": np.zeros(2, np.float32), "its": np.zeros(self.blocks, np.int8),
               "est": np.zeros(self.blocks, np.float32), "pilot": np.zeros(self.blocks, np.float32),
               "blocks": np.zeros((self.blocks, 476), np.uint8), "ok": np.zeros(self.blocks, np.uint8)}
        good = self.L.ref_finish_grid(self.h, _p(g), *[_p(out[k]) for k in ("coef", "llrf", "sub_est", "sub_rms", "align", "its", "est", "pilot", "blocks", "ok")])
        out["good"] = good
        return out

    def decode_frame(self, luma):
        luma = np.ascontiguousarray(luma, np.uint8)
        ih, iw = luma.shape
        blocks = np.zeros((self.blocks, 476), np.uint8)
        ok = np.zeros(self.blocks, np.uint8)
        its = np.zeros(self.blocks, np.int8)
        reg = np.zeros(9 + 2 * 40 * 40, np.float32)
        nxy = np.zeros(80, np.float32)
        nn = np.zeros(2, np.int32)
        good = self.L.ref_decode_frame(self.h, _p(luma), iw, ih, _p(blocks), _p(ok), _p(its), _p(reg), _p(nxy), _p(nn))
        nx, ny = int(nn[0]), int(nn[1])
        return {"good": good, "blocks": blocks, "ok": ok, "its": its, "H": reg[:9].copy(),
                "nodes": reg[9:9 + 2 * nx * ny].reshape(ny, nx, 2).copy(), "node_x": nxy[:nx].copy(), "node_y": nxy[nx:nx + ny].copy()}

    def sample_grid(self, luma, H, nodes, fast):
        luma = np.ascontiguousarray(luma, np.uint8)
        ih, iw = luma.shape
        reg = np.concatenate([np.asarray(H, np.float32).ravel(), np.asarray(nodes, np.float32).ravel()]).astype(np.float32)
        g = np.zeros(self.n * self.n, np.float32)
        self.L.ref_sample_grid(self.h, _p(luma), iw, ih, _p(reg), int(fast), _p(g))
        return g.reshape(self.n, self.n)

    def sample_decode(self, luma, H, nodes):
        """The grid as the reference's decode samples it (strips of 64, its integer read at gamma 1) and the shading
        fit's samples; (grid n x n, shade n/8 x n/8, lin) where lin says the integer read ran."""
        luma = np.ascontiguousarray(luma, np.uint8)
        ih, iw = luma.shape
        reg = np.concatenate([np.asarray(H, np.float32).ravel(), np.asarray(nodes, np.float32).ravel()]).astype(np.float32)
        g = np.zeros(self.n * self.n, np.float32)
        c = self.n // 8
        s = np.zeros(c * c, np.float32)
        lin = self.L.ref_sample_decode(self.h, _p(luma), iw, ih, _p(reg), _p(g), _p(s))
        return g.reshape(self.n, self.n), s.reshape(c, c), bool(lin)


def spec_blocks(count, seed=None):
    """Blocks as the spec's test vector makes them (id LE, byte j = j mod 256), or seeded random payloads."""
    b = np.zeros((count, 476), np.uint8)
    b[:, :4] = np.arange(count, dtype="<u4").view(np.uint8).reshape(count, 4)
    if seed is None:
        b[:, 4:] = np.arange(472, dtype=np.int64) & 255
    else:
        b[:, 4:] = np.random.default_rng(seed).integers(0, 256, (count, 472), dtype=np.uint8)
    return b


def picture_grid(grey, n, pxm, quiet_modules=2, margin=15):
    """The n x n picture grid (grey / 255) out of a painted grey square at an exact-copy scale (pxm = n / span)."""
    o = (quiet_modules + margin) * pxm
    return grey[o:o + n, o:o + n].astype(np.float32) / 255.0
