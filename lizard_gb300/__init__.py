"""lizard_gb300: the LIZARD receive hot path on one GB300, behind a C ABI (include/lizard_gb300.h).

This module is the Python face of that ABI, for tests, the benchmark and Python callers. It loads the in-tree
library lizard_gb300/liblizard_gb300.so (built by lizard_gb300/build.py) and fails loudly when it is missing: there
is no CPU fallback for any decode here.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblizard_gb300.so")

# The reference's rate indices (liblizard/src/ldpc.h:30-33) and their codes' shapes.
RATES = (6, 4, 3, 2)
RATE_NAME = {6: "7/8", 4: "3/4", 3: "2/3", 2: "1/2"}
CODE_N = {6: 4608, 4: 5120, 3: 5760, 2: 7680}
CODE_K = {6: 3968, 4: 3840, 3: 3840, 2: 3840}
CODE_NT = {6: 4480, 4: 5120, 3: 5760, 2: 7680}
# Entries of H (liblizard/test/ldpc_table.c prints them; the oracle derives them from the tables).
CODE_EDGES = {6: 14463, 4: 19455, 3: 22527, 2: 26879}
BLOCK_BYTES = 476
INFO_BITS = 3840

_lib = None


class LizgError(RuntimeError):
    pass


def lib():
    """The loaded C library. Raises if it has not been built: the decode has no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LizgError("lizard_gb300: %s is not built (run `python lizard_gb300/build.py`)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.lizg_last_error.restype = ctypes.c_char_p
    L.lizg_version.restype = ctypes.c_char_p
    L.lizg_ldpc_n.argtypes = [I]
    L.lizg_ldpc_encode.argtypes = [I, P, P]
    L.lizg_ldpc_encode_many.argtypes = [I, P, I, P]
    L.lizg_crc32c.argtypes = [P, ctypes.c_size_t]
    L.lizg_crc32c.restype = ctypes.c_uint32
    L.lizg_ldpc_decode_stall.argtypes = [I, P, P, I, I, F]
    L.lizg_ldpc_plan_new.argtypes = [P, I, I, I, F]
    L.lizg_ldpc_plan_new.restype = P
    L.lizg_ldpc_plan_free.argtypes = [P]
    L.lizg_ldpc_plan_llr_bytes.argtypes = [P]
    L.lizg_ldpc_plan_llr_bytes.restype = ctypes.c_int64
    L.lizg_ldpc_plan_run_dev.argtypes = [P, P, P, P, P, P]
    L.lizg_ldpc_plan_run.argtypes = [P, P, P, P, P, P]
    L.lizg_ldpc_plan_set_chunks.argtypes = [P, ctypes.c_int]
    L.lizg_ldpc_plan_set_transfer.argtypes = [P, ctypes.c_int]
    L.lizg_ldpc_plan_transfer.argtypes = [P]
    L.lizg_ldpc_plan_launches.argtypes = [P]
    L.lizg_ldpc_autotune.argtypes = [I, P, I, P]
    L.lizg_ldpc_variants.argtypes = [I]
    L.lizg_ldpc_variant.argtypes = [I, P, P]
    L.lizg_ldpc_set_variant.argtypes = [I, I]
    _lib = L
    return L


def _check(rc, what):
    if rc < 0:
        raise LizgError("%s failed (%d): %s" % (what, rc, lib().lizg_last_error().decode()))
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def crc32c(data):
    b = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8))
    return int(lib().lizg_crc32c(_ptr(b), b.size))


def ldpc_encode(rate, data):
    """k data bits (one a byte) -> n codeword bits, the reference's ldpc_encode."""
    data = np.ascontiguousarray(data, np.uint8)
    cw = np.zeros(CODE_N.get(rate, 8), np.uint8)
    _check(lib().lizg_ldpc_encode(rate, _ptr(data), _ptr(cw)), "lizg_ldpc_encode")
    return cw


def ldpc_encode_many(rate, data):
    """(count, k) data bits -> (count, n) codewords."""
    data = np.ascontiguousarray(data, np.uint8)
    cw = np.zeros((data.shape[0], CODE_N[rate]), np.uint8)
    _check(lib().lizg_ldpc_encode_many(rate, _ptr(data), data.shape[0], _ptr(cw)), "lizg_ldpc_encode_many")
    return cw


def ldpc_autotune(count=8192, ebn0_db=(1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0)):
    """Times every decoder variant of every code on the current device over count codewords a code (codeword c at
    ebn0_db[c % len]) and keeps the fastest per code; returns the chosen variant indices in code order 7/8, 3/4,
    2/3, 1/2."""
    e = np.ascontiguousarray(np.atleast_1d(ebn0_db), np.float32)
    ch = np.zeros(4, np.int32)
    _check(lib().lizg_ldpc_autotune(count, _ptr(e), e.size, _ptr(ch)), "lizg_ldpc_autotune")
    return [int(x) for x in ch]


def ldpc_variants(rate):
    """How many decoder variants the code of this rate has."""
    return _check(lib().lizg_ldpc_variants(rate), "lizg_ldpc_variants")


def ldpc_variant(rate):
    """The current device's variant of this rate's code: (index, warps a codeword, loop form, pair form)."""
    w, lf = np.zeros(1, np.int32), np.zeros(1, np.int32)
    v = _check(lib().lizg_ldpc_variant(rate, _ptr(w), _ptr(lf)), "lizg_ldpc_variant")
    return v, int(w[0]), bool(lf[0] & 1), bool(lf[0] & 2)


def ldpc_set_variant(rate, index):
    _check(lib().lizg_ldpc_set_variant(rate, index), "lizg_ldpc_set_variant")


def ldpc_decode_stall(rate, llr, max_iter, stall_it=0, stall_ratio=0.0):
    """The reference's ldpc_decode_stall on the GPU: (iterations or -1/-3, n hard bits)."""
    llr = np.ascontiguousarray(llr, np.int8)
    out = np.zeros(CODE_N[rate], np.uint8)
    rc = lib().lizg_ldpc_decode_stall(rate, _ptr(llr), _ptr(out), max_iter, stall_it, stall_ratio)
    if rc <= -100:
        raise LizgError("lizg_ldpc_decode_stall failed (%d): %s" % (rc + 100, lib().lizg_last_error().decode()))
    return rc, out


class LdpcPlan:
    """A planned batch of mixed-rate codewords laid back to back (include/lizard_gb300.h lizg_ldpc_plan_*)."""

    def __init__(self, rates, max_iter=30, stall_it=9, stall_ratio=0.95):
        self.rates = np.ascontiguousarray(rates, np.int32)
        self.count = int(self.rates.size)
        h = lib().lizg_ldpc_plan_new(_ptr(self.rates), self.count, max_iter, stall_it, stall_ratio)
        if not h:
            raise LizgError("lizg_ldpc_plan_new: " + lib().lizg_last_error().decode())
        self._h = ctypes.c_void_p(h)
        self.llr_bytes = int(lib().lizg_ldpc_plan_llr_bytes(self._h))
        n = np.array([CODE_N[int(r)] for r in self.rates], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)

    def close(self):
        if getattr(self, "_h", None):
            lib().lizg_ldpc_plan_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def launches(self):
        return int(lib().lizg_ldpc_plan_launches(self._h))

    def set_transfer(self, in_place):
        """1: page-locked host buffers are read and written in place by the decoder; 0: always staged."""
        _check(lib().lizg_ldpc_plan_set_transfer(self._h, int(in_place)), "lizg_ldpc_plan_set_transfer")

    @property
    def transfer(self):
        """The route the last run took: 1 in place, 0 staged."""
        return int(lib().lizg_ldpc_plan_transfer(self._h))

    def set_chunks(self, chunks):
        """Chunk count of the pipelined host-memory run (1..16); returns the count set."""
        return _check(lib().lizg_ldpc_plan_set_chunks(self._h, int(chunks)), "lizg_ldpc_plan_set_chunks")

    def run(self, llr, bits=None, its=None, ok=None, stream=0):
        """Host memory in and out: returns (packed bits, its, ok)."""
        llr = np.ascontiguousarray(llr, np.int8)
        if llr.size != self.llr_bytes:
            raise ValueError("llr holds %d bytes, the plan %d" % (llr.size, self.llr_bytes))
        bits = np.empty(self.llr_bytes // 8, np.uint8) if bits is None else bits
        its = np.empty(self.count, np.int32) if its is None else its
        ok = np.empty(self.count, np.uint8) if ok is None else ok
        _check(lib().lizg_ldpc_plan_run(self._h, _ptr(llr), _ptr(bits), _ptr(its), _ptr(ok), ctypes.c_void_p(stream)), "lizg_ldpc_plan_run")
        return bits, its, ok

    def run_dev(self, d_llr, d_bits, d_its, d_ok, stream=0):
        """Device pointers (ints) in and out, queued on `stream` (a cudaStream_t as an int)."""
        _check(lib().lizg_ldpc_plan_run_dev(self._h, ctypes.c_void_p(d_llr), ctypes.c_void_p(d_bits), ctypes.c_void_p(d_its),
                                            ctypes.c_void_p(d_ok), ctypes.c_void_p(stream)), "lizg_ldpc_plan_run_dev")


def iterations_run(its, rates, max_iter, stall_it):
    """Iterations each codeword actually ran: its return when positive, max_iter at -1, stall_it at -3."""
    its = np.asarray(its)
    return np.where(its > 0, its, np.where(its == -3, stall_it, max_iter))


def edge_updates(its, rates, max_iter, stall_it):
    e = np.array([CODE_EDGES[int(r)] for r in rates], np.int64)
    return int((iterations_run(its, rates, max_iter, stall_it).astype(np.int64) * e).sum())


# ---------------------------------------------------------------- the receiver

SUB = 320
PICTURES = (384, 512, 768, 1024, 1152, 1280, 1536)


def _rx_sigs(L):
    P, I = ctypes.c_void_p, ctypes.c_int
    L.lizg_format_tables.argtypes = [I, I, I, P, P, P, P, P, P, P, P, P]
    L.lizg_rx_new.argtypes = [I, I, I, I]
    L.lizg_rx_new.restype = P
    L.lizg_rx_free.argtypes = [P]
    L.lizg_rx_info.argtypes = [P, P]
    L.lizg_rx_perm.argtypes = [P, I, P]
    L.lizg_rx_launches.argtypes = [P]
    L.lizg_rx_set_read.argtypes = [P, I]
    L.lizg_rx_fault.argtypes = [P]
    L.lizg_rx_autotune.argtypes = [P, P, I, I, I, ctypes.c_int64, P, I, P, P]
    L.lizg_rx_variant.argtypes = [P, I]
    L.lizg_rx_set_ldpc_mixed.argtypes = [P, I]
    L.lizg_layout_nodes.argtypes = [I, P, P, P]
    L.lizg_rx_finish_luma_host.argtypes = [P, P, I, I, I, ctypes.c_int64, P, I, P, P, P]
    L.lizg_rx_finish_coef_dev.argtypes = [P, P, I, P, P]
    L.lizg_rx_finish_grid_dev.argtypes = [P, P, I, P, P, P]
    L.lizg_rx_finish_luma_dev.argtypes = [P, P, I, I, I, ctypes.c_int64, P, I, P, P, P, P]
    L.lizg_rx_finish_luma_graph.argtypes = [P, P, I, I, I, ctypes.c_int64, P, I, P, P, P, P]
    L.lizg_anchor_find_dev.argtypes = [I, P, I, I, ctypes.c_int64, P, I, P, P, I, P, P]
    L.lizg_engine_new.argtypes = []
    L.lizg_engine_new.restype = P
    L.lizg_engine_free.argtypes = [P]
    L.lizg_engine_add_format.argtypes = [P, I, I, I, I]
    L.lizg_engine_rx.argtypes = [P, I]
    L.lizg_engine_rx.restype = P
    L.lizg_engine_run_dev.argtypes = [P, P, I, P]
    L.lizg_engine_launches.argtypes = [P]
    L.lizg_engine_set_mixed.argtypes = [P, I]
    L.lizg_engine_autotune.argtypes = [P, P, I, P, ctypes.POINTER(ctypes.c_float)]
    L.lizg_ingest_pixels_dev.argtypes = [P, I, I, I, ctypes.c_int64, I, I, P, P]
    L.lizg_develop_dev.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, I, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, P, P]
    L.lizg_refiner_new.argtypes = [I, I]
    L.lizg_refiner_new.restype = P
    L.lizg_refiner_free.argtypes = [P]
    L.lizg_refine_dev.argtypes = [P, P, I, I, ctypes.c_int64, P, I, I, P, P, P]
    L.lizg_anchor_register_dev.argtypes = [P, P, P, I, I, ctypes.c_int64, P, P, I, P, P, P, P]
    L.lizg_encoder_new.argtypes = [I, I, I, I]
    L.lizg_encoder_new.restype = P
    L.lizg_encoder_free.argtypes = [P]
    L.lizg_encoder_fps.argtypes = [P, I]
    L.lizg_encoder_info.argtypes = [P, P]
    L.lizg_encode_dev.argtypes = [P, P, I, I, P, P, P]
    L.lizg_layout_kind.argtypes = [I, I, I, P]
    L.lizg_border_nodes_dev.argtypes = [I, P, I, I, ctypes.c_int64, P, I, P, I, P, P]
    L.lizg_rx_spectrum_grid_dev.argtypes = [P, P, I, P, P]
    L.lizg_gn_new.argtypes = [I, I, I, I]
    L.lizg_gn_new.restype = P
    L.lizg_gn_free.argtypes = [P]
    L.lizg_gn_refine_dev.argtypes = [P, P, I, I, ctypes.c_int64, P, I, I, P, P, P]
    L.lizg_gn_pictures_dev.argtypes = [P, P, I, I, ctypes.c_int64, P, I, P, P]
    L.lizg_fmt_geometry.argtypes = [I, P, P]
    L.lizg_fmt_read_dev.argtypes = [I, P, I, I, ctypes.c_int64, P, I, I, P, P, P]
    L.lizg_fmt_decode_dev.argtypes = [I, P, I, P, P]


class RxOut(ctypes.Structure):
    """lizg_rx_out: device pointers."""
    _fields_ = [("blocks", ctypes.c_void_p), ("ok", ctypes.c_void_p), ("its", ctypes.c_void_p), ("est", ctypes.c_void_p),
                ("pilot", ctypes.c_void_p), ("align", ctypes.c_void_p), ("llrf", ctypes.c_void_p), ("sub_est", ctypes.c_void_p),
                ("sub_rms", ctypes.c_void_p)]


class Format:
    """A format's host-side tables (lizg_format_tables): no device needed."""

    def __init__(self, n, subch, span=128):
        L = lib()
        if not hasattr(L, "_rx"):
            _rx_sigs(L)
            L._rx = True
        info = np.zeros(22, np.int32)
        _check(L.lizg_format_tables(n, subch, span, _ptr(info), None, None, None, None, None, None, None, None), "lizg_format_tables")
        self.n, self.subch, self.span, self.blocks, self.used, self.bw, self.vblocks, self.tiers, self.V, self.npilot = (int(x) for x in info[:10])
        self.tier = [(int(info[10 + 3 * t]), int(info[11 + 3 * t]), int(info[12 + 3 * t])) for t in range(self.tiers)]
        need = self.subch * SUB
        self.uv = np.zeros(2 * need, np.int16)
        self.white = np.zeros(2 * need, np.uint8)
        self.block_tier = np.zeros(self.blocks, np.int32)
        self.block_slot = np.zeros(self.blocks, np.int32)
        self.erase = np.zeros(14, np.int32)
        self.hole_inv = np.zeros(36, np.float64)
        self.detrend = np.zeros(6 * self.n + 2, np.float32)
        nts = [CODE_NT[r] for r, _, _ in self.tier]
        perm = np.zeros(sum(nts), np.int16)
        _check(L.lizg_format_tables(n, subch, span, None, _ptr(self.uv), _ptr(self.white), _ptr(self.block_tier), _ptr(self.block_slot),
                                    _ptr(self.erase), _ptr(self.hole_inv), _ptr(self.detrend), _ptr(perm)), "lizg_format_tables")
        self.perm = np.split(perm, np.cumsum(nts)[:-1])
        self.scale = np.float32(n) / np.float32(span)

    def tix(self):
        u, v = self.uv[0::2].astype(np.int64), self.uv[1::2].astype(np.int64)
        return v * self.n + (u + self.n) % self.n


def rx_outputs(fmt, frames, keep=False):
    """Device output buffers of a receive call for frames frames of a format (torch tensors) and the lizg_rx_out
    naming them."""
    import torch
    f = fmt
    o = {"blocks": torch.zeros((frames, f.blocks, BLOCK_BYTES), dtype=torch.uint8, device="cuda"),
         "ok": torch.zeros((frames, f.blocks), dtype=torch.uint8, device="cuda"),
         "its": torch.zeros((frames, f.blocks), dtype=torch.int32, device="cuda"),
         "est": torch.zeros((frames, f.blocks), dtype=torch.float32, device="cuda"),
         "pilot": torch.zeros((frames, f.blocks), dtype=torch.float32, device="cuda"),
         "align": torch.zeros((frames, 3), dtype=torch.float32, device="cuda")}
    if keep:
        o["llrf"] = torch.zeros((frames, 2 * f.subch * SUB), dtype=torch.int8, device="cuda")
        o["sub_est"] = torch.zeros((frames, f.subch), dtype=torch.float64, device="cuda")
        o["sub_rms"] = torch.zeros((frames, f.subch), dtype=torch.float32, device="cuda")
    s = RxOut(*[o[k].data_ptr() if k in o else None for k in ("blocks", "ok", "its", "est", "pilot", "align", "llrf", "sub_est", "sub_rms")])
    return o, s


READ_DECODE, READ_EXACT = 0, 1


class Receiver:
    """A receiver handle (lizg_rx_*) for one format and up to max_frames frames a call. read: "decode" (the reference
    decoder's integer read, the default) or "exact" (the exact float walk)."""

    def __init__(self, n, subch, span=128, max_frames=1, read="decode"):
        self.fmt = Format(n, subch, span)
        L = lib()
        h = L.lizg_rx_new(n, subch, span, max_frames)
        if not h:
            raise LizgError("lizg_rx_new: " + L.lizg_last_error().decode())
        self._h = ctypes.c_void_p(h)
        self.max_frames = max_frames
        self.set_read(read)

    def set_read(self, read):
        """The picture read of later finishes from captured frames: "decode" or "exact"."""
        code = {"decode": READ_DECODE, "exact": READ_EXACT}[read]
        _check(lib().lizg_rx_set_read(self._h, code), "lizg_rx_set_read")
        self.read = read

    def close(self):
        if getattr(self, "_h", None):
            lib().lizg_rx_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def launches(self):
        return int(lib().lizg_rx_launches(self._h))

    def fault(self):
        """1 where a pass's bounded wait gave up (never expected), else 0."""
        return _check(lib().lizg_rx_fault(self._h), "lizg_rx_fault")

    def autotune_dev(self, d_luma, w, h, pitch, frame_stride, d_reg, frames, stream=None):
        """lizg_rx_autotune on device buffers (pointers): each tier's LDPC kernel variant timed on these frames and
        kept by the handle. Returns the 4 choices (-1 past the format's tiers)."""
        import torch
        choice = np.full(4, -1, np.int32)
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_rx_autotune(self._h, ctypes.c_void_p(d_luma), w, h, pitch, frame_stride, ctypes.c_void_p(d_reg), frames,
                                      _ptr(choice), ctypes.c_void_p(st)), "lizg_rx_autotune")
        return [int(c) for c in choice]

    def set_ldpc_mixed(self, mixed):
        """The decode stage: 0 a launch a tier (the default), 1 one persistent launch across the tiers; the previous."""
        return _check(lib().lizg_rx_set_ldpc_mixed(self._h, int(mixed)), "lizg_rx_set_ldpc_mixed")

    def variant(self, tier):
        """Tier's LDPC kernel variant as the handle's finishes launch it (its own after autotune, else the device's)."""
        return _check(lib().lizg_rx_variant(self._h, tier), "lizg_rx_variant")

    def _outputs(self, frames, torch, keep):
        return rx_outputs(self.fmt, frames, keep)

    def finish_coef(self, coef, keep=True, stream=None):
        """coef: frames x subch x 320 complex64 (or float32 pairs). Returns a dict of numpy arrays."""
        import torch
        c = np.ascontiguousarray(np.asarray(coef).view(np.float32) if np.iscomplexobj(coef) else coef, np.float32)
        frames = c.size // (2 * self.fmt.subch * SUB)
        d = torch.from_numpy(c.reshape(frames, -1)).cuda()
        o, s = self._outputs(frames, torch, keep)
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_rx_finish_coef_dev(self._h, ctypes.c_void_p(d.data_ptr()), frames, ctypes.byref(s), ctypes.c_void_p(st)), "lizg_rx_finish_coef_dev")
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in o.items()}

    def spectrum_grid(self, grids, stream=None):
        """The transform alone on grids (frames x n x n float32): frames x subch*320 complex64 (pos order)."""
        import torch
        g = np.ascontiguousarray(grids, np.float32)
        frames = g.shape[0]
        d = torch.from_numpy(g).cuda()
        c = torch.zeros((frames, 2 * self.fmt.subch * SUB), dtype=torch.float32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_rx_spectrum_grid_dev(self._h, ctypes.c_void_p(d.data_ptr()), frames, ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(st)),
               "lizg_rx_spectrum_grid_dev")
        torch.cuda.synchronize()
        out = c.cpu().numpy()
        return out[:, 0::2] + 1j * out[:, 1::2]

    def finish_grid(self, grids, keep=True, coef=True, stream=None):
        """grids: frames x n x n float32 (grey / 255). Returns a dict of numpy arrays (coef: frames x subch*320 complex64)."""
        import torch
        g = np.ascontiguousarray(grids, np.float32)
        frames = g.shape[0]
        d = torch.from_numpy(g).cuda()
        o, s = self._outputs(frames, torch, keep)
        c = torch.zeros((frames, 2 * self.fmt.subch * SUB), dtype=torch.float32, device="cuda") if coef else None
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_rx_finish_grid_dev(self._h, ctypes.c_void_p(d.data_ptr()), frames, ctypes.byref(s),
                                              ctypes.c_void_p(c.data_ptr()) if coef else None, ctypes.c_void_p(st)), "lizg_rx_finish_grid_dev")
        torch.cuda.synchronize()
        out = {k: v.cpu().numpy() for k, v in o.items()}
        if coef:
            out["coef"] = c.cpu().numpy()
        return out

    def finish_luma(self, luma, reg, keep=True, grid=True, stream=None):
        """luma: frames x h x w uint8; reg: frames x (9 + 2 nx ny) float32 (H then the node mesh). Returns a dict of
        numpy arrays including the sampled grids and the spectra."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        frames, h, w = lu.shape
        d = torch.from_numpy(lu).cuda()
        dr = torch.from_numpy(np.ascontiguousarray(reg, np.float32)).cuda()
        o, s = self._outputs(frames, torch, keep)
        n = self.fmt.n
        g = torch.zeros((frames, n, n), dtype=torch.float32, device="cuda") if grid else None
        c = torch.zeros((frames, 2 * self.fmt.subch * SUB), dtype=torch.float32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_rx_finish_luma_dev(self._h, ctypes.c_void_p(d.data_ptr()), w, h, w, h * w, ctypes.c_void_p(dr.data_ptr()), frames,
                                              ctypes.byref(s), ctypes.c_void_p(g.data_ptr()) if grid else None, ctypes.c_void_p(c.data_ptr()),
                                              ctypes.c_void_p(st)), "lizg_rx_finish_luma_dev")
        torch.cuda.synchronize()
        out = {k: v.cpu().numpy() for k, v in o.items()}
        if grid:
            out["grid"] = g.cpu().numpy()
        out["coef"] = c.cpu().numpy()
        return out

    def finish_luma_host(self, luma, reg):
        """lizg_rx_finish_luma_host: frames x h x w uint8 and frames x (9 + 2 nx ny) float32 from host memory;
        (blocks, ok, its, verified)."""
        lu = np.ascontiguousarray(luma, np.uint8)
        rg = np.ascontiguousarray(reg, np.float32)
        frames, h, w = lu.shape
        nb = frames * self.fmt.blocks
        blocks = np.zeros((frames, self.fmt.blocks, BLOCK_BYTES), np.uint8)
        ok = np.zeros((frames, self.fmt.blocks), np.uint8)
        its = np.zeros((frames, self.fmt.blocks), np.int32)
        v = _check(lib().lizg_rx_finish_luma_host(self._h, _ptr(lu), w, h, w, h * w, _ptr(rg), frames, _ptr(blocks), _ptr(ok), _ptr(its)),
                   "lizg_rx_finish_luma_host")
        assert ok.size == nb
        return blocks, ok, its, v


FRAME_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint8), ctypes.c_int,
                            ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32), ctypes.c_int)
LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p)
RELEASE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64)


class FrontConfig(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("subch", ctypes.c_int), ("span", ctypes.c_int), ("max_w", ctypes.c_int), ("max_h", ctypes.c_int),
                ("batch_cap", ctypes.c_int), ("slots", ctypes.c_int), ("read", ctypes.c_int), ("frame", FRAME_FN), ("log", LOG_FN),
                ("user", ctypes.c_void_p)]


class FrontReceiver:
    """The batching front (lizg_receiver_*): frames pushed from host memory with their registrations, decoded in
    batches on the front's own thread. on_frame(tag, ts_ns, verified bytes, ok, its) and on_release(tag) are called
    from C (the front's thread, or inside push)."""

    def __init__(self, n, subch, span, max_w, max_h, batch_cap=0, slots=0, read="decode", on_frame=None, on_release=None, on_log=None):
        L = lib()
        if not hasattr(L, "_front"):
            P, I = ctypes.c_void_p, ctypes.c_int
            L.lizg_receiver_new.argtypes = [ctypes.POINTER(FrontConfig), RELEASE_FN]
            L.lizg_receiver_new.restype = P
            L.lizg_receiver_free.argtypes = [P]
            L.lizg_receiver_push.argtypes = [P, P, I, I, I, ctypes.c_int64, ctypes.c_uint64, P]
            L.lizg_receiver_batch_cap.argtypes = [P, I]
            L.lizg_receiver_wants_luma.argtypes = [P]
            L.lizg_receiver_flush.argtypes = [P]
            L.lizg_receiver_stats.argtypes = [P]
            L.lizg_receiver_stats.restype = ctypes.c_char_p
            L.lizg_receiver_series.argtypes = [P, ctypes.c_double, P, I]
            L._front = True

        def frame(user, tag, ts, verified, count, ok, its, blocks):
            if on_frame:
                on_frame(int(tag), int(ts), bytes(ctypes.string_at(verified, count * BLOCK_BYTES)) if count else b"",
                         np.ctypeslib.as_array(ok, (blocks,)).copy(), np.ctypeslib.as_array(its, (blocks,)).copy())

        self._frame = FRAME_FN(frame)
        self._log = LOG_FN(lambda user, line: on_log(line.decode()) if on_log else None)
        self._release = RELEASE_FN(lambda user, tag: on_release(int(tag)) if on_release else None)
        cfg = FrontConfig(n, subch, span, max_w, max_h, batch_cap, slots, {"decode": READ_DECODE, "exact": READ_EXACT}[read],
                          self._frame, self._log, None)
        h = L.lizg_receiver_new(ctypes.byref(cfg), self._release)
        if not h:
            raise LizgError("lizg_receiver_new: " + L.lizg_last_error().decode())
        self._h = ctypes.c_void_p(h)

    def push(self, luma, ts_ns, tag, reg):
        lu = np.ascontiguousarray(luma, np.uint8)
        rg = np.ascontiguousarray(reg, np.float32)
        h, w = lu.shape
        return _check(lib().lizg_receiver_push(self._h, _ptr(lu), w, h, w, int(ts_ns), int(tag), _ptr(rg)), "lizg_receiver_push")

    def batch_cap(self, frames):
        lib().lizg_receiver_batch_cap(self._h, frames)

    def flush(self):
        return _check(lib().lizg_receiver_flush(self._h), "lizg_receiver_flush")

    def stats(self):
        import json
        return json.loads(lib().lizg_receiver_stats(self._h).decode())

    def series(self, since_ms=-1e300, cap=1 << 16):
        out = np.zeros(cap, np.float64)
        k = _check(lib().lizg_receiver_series(self._h, since_ms, _ptr(out), cap), "lizg_receiver_series")
        return out[:k]

    def close(self):
        if getattr(self, "_h", None):
            lib().lizg_receiver_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class AnchorOut(ctypes.Structure):
    _fields_ = [("ok", ctypes.c_void_p), ("peak", ctypes.c_void_p), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("u", ctypes.c_void_p), ("v", ctypes.c_void_p)]


def anchor_find(span, luma, H, lens=None, skip=None, stream=None):
    """The anchor search on the GPU for a batch of frames: luma frames x h x w uint8, H frames x 9 (or frames x
    stride: a receiver's registrations), lens frames x 15 float64 or None, skip frames x 49 or None. Returns a dict of
    frames x 49 arrays ok, peak, dx, dy, u, v."""
    import torch
    lib()
    lu = np.ascontiguousarray(luma, np.uint8)
    if lu.ndim == 2:
        lu = lu[None]
    frames, h, w = lu.shape
    Hf = np.ascontiguousarray(np.asarray(H, np.float32).reshape(frames, -1))
    d_l, d_h = torch.from_numpy(lu).cuda(), torch.from_numpy(Hf).cuda()
    d_lens = None if lens is None else torch.from_numpy(np.ascontiguousarray(np.asarray(lens, np.float64).reshape(frames, 15))).cuda()
    d_skip = None if skip is None else torch.from_numpy(np.ascontiguousarray(np.asarray(skip, np.uint8).reshape(frames, 49))).cuda()
    o = {"ok": torch.zeros((frames, 49), dtype=torch.uint8, device="cuda")}
    for k in ("peak", "dx", "dy", "u", "v"):
        o[k] = torch.zeros((frames, 49), dtype=torch.float32, device="cuda")
    s = AnchorOut(*[o[k].data_ptr() for k in ("ok", "peak", "dx", "dy", "u", "v")])
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _check(lib().lizg_anchor_find_dev(span, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_h.data_ptr()), Hf.shape[1],
                                      None if d_lens is None else ctypes.c_void_p(d_lens.data_ptr()),
                                      None if d_skip is None else ctypes.c_void_p(d_skip.data_ptr()), frames, ctypes.byref(s), ctypes.c_void_p(st)),
           "lizg_anchor_find_dev")
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in o.items()}


class Encoder:
    """The sender on the GPU (lizg_encoder_*): blocks (frames x blocks x 476 bytes) to the drive (frames x px x px
    floats) and the grey page (frames x W x W)."""

    def __init__(self, n, subch, span, max_frames=8):
        self._h = lib().lizg_encoder_new(n, subch, span, max_frames)
        if not self._h:
            raise LizgError("lizg_encoder_new: " + lib().lizg_last_error().decode())
        info = np.zeros(5, np.int32)
        _check(lib().lizg_encoder_info(self._h, _ptr(info)), "lizg_encoder_info")
        self.blocks, self.pxm, self.px, self.W, self.max_frames = (int(v) for v in info)

    def set_fps(self, fps):
        _check(lib().lizg_encoder_fps(self._h, fps), "lizg_encoder_fps")

    def encode(self, blocks, pilots=0, drive=True, stream=None):
        """blocks: frames x blocks x 476 uint8. Returns (drive or None, grey)."""
        import torch
        b = np.ascontiguousarray(blocks, np.uint8).reshape(-1, self.blocks, BLOCK_BYTES)
        frames = b.shape[0]
        d_b = torch.from_numpy(b).cuda()
        d_g = torch.zeros((frames, self.W, self.W), dtype=torch.uint8, device="cuda")
        d_d = torch.zeros((frames, self.px, self.px), dtype=torch.float32, device="cuda") if drive else None
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_encode_dev(self._h, ctypes.c_void_p(d_b.data_ptr()), frames, pilots,
                                     None if d_d is None else ctypes.c_void_p(d_d.data_ptr()), ctypes.c_void_p(d_g.data_ptr()), ctypes.c_void_p(st)),
               "lizg_encode_dev")
        torch.cuda.synchronize()
        return (None if d_d is None else d_d.cpu().numpy()), d_g.cpu().numpy()

    def __del__(self):
        if getattr(self, "_h", None):
            lib().lizg_encoder_free(self._h)
            self._h = None


def layout_kind(span, version, fps):
    """The border's cell kinds, (span + 30)^2 (2 dark, 1 light, 0 the picture's), with the word (version, fps)."""
    side = span + 30
    k = np.zeros(side * side, np.uint8)
    rc = lib().lizg_layout_kind(span, version, fps, _ptr(k))
    _check(rc if rc < 0 else 0, "lizg_layout_kind")
    return k.reshape(side, side)


def fmt_geometry(span):
    """(cells a side, codeword bytes) of the format word in a ring of span modules."""
    c, b = ctypes.c_int32(), ctypes.c_int32()
    _check(lib().lizg_fmt_geometry(span, ctypes.byref(c), ctypes.byref(b)), "lizg_fmt_geometry")
    return c.value, b.value


def fmt_read(span, luma, regs, stream=None):
    """The format word read and decoded on the GPU for a batch of registered frames: luma frames x h x w uint8, regs
    frames x (9 + 2 nodes) float32 (H then the mesh). Returns (q frames x 4 cells soft values, word frames x 4:
    read, ok, version, fps)."""
    import torch
    lu = np.ascontiguousarray(luma, np.uint8)
    if lu.ndim == 2:
        lu = lu[None]
    frames, h, w = lu.shape
    rg = np.ascontiguousarray(np.asarray(regs, np.float32).reshape(frames, -1))
    cells, _ = fmt_geometry(span)
    d_l, d_r = torch.from_numpy(lu).cuda(), torch.from_numpy(rg).cuda()
    d_q = torch.zeros((frames, 4 * cells), dtype=torch.float32, device="cuda")
    d_w = torch.zeros((frames, 4), dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _check(lib().lizg_fmt_read_dev(span, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_r.data_ptr()), rg.shape[1], frames,
                                   ctypes.c_void_p(d_q.data_ptr()), ctypes.c_void_p(d_w.data_ptr()), ctypes.c_void_p(st)), "lizg_fmt_read_dev")
    torch.cuda.synchronize()
    return d_q.cpu().numpy(), d_w.cpu().numpy()


def fmt_decode(span, q, stream=None):
    """The format word's soft decode alone on the GPU: q frames x 4 cells. Returns frames x 4 (1, ok, version, fps)."""
    import torch
    qq = np.ascontiguousarray(np.asarray(q, np.float32))
    if qq.ndim == 1:
        qq = qq[None]
    d_q = torch.from_numpy(qq).cuda()
    d_w = torch.zeros((qq.shape[0], 4), dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _check(lib().lizg_fmt_decode_dev(span, ctypes.c_void_p(d_q.data_ptr()), qq.shape[0], ctypes.c_void_p(d_w.data_ptr()), ctypes.c_void_p(st)),
           "lizg_fmt_decode_dev")
    torch.cuda.synchronize()
    return d_w.cpu().numpy()


def border_nodes(span, luma, H, lens=None, stream=None):
    """The registration's border nodes on the GPU for a batch of frames: luma frames x h x w uint8, H frames x 9 (or
    frames x stride, H first), lens frames x 15 float64 or None. Returns frames x nn x nn x 4 (dx, dy, score, done)."""
    import torch
    lu = np.ascontiguousarray(luma, np.uint8)
    if lu.ndim == 2:
        lu = lu[None]
    frames, h, w = lu.shape
    Hf = np.ascontiguousarray(np.asarray(H, np.float32).reshape(frames, -1))
    nn = int(lib().lizg_layout_nodes(span, None, None, None))
    d_l, d_h = torch.from_numpy(lu).cuda(), torch.from_numpy(Hf).cuda()
    d_lens = None if lens is None else torch.from_numpy(np.ascontiguousarray(np.asarray(lens, np.float64).reshape(frames, 15))).cuda()
    d_n = torch.zeros((frames, nn, nn, 4), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _check(lib().lizg_border_nodes_dev(span, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_h.data_ptr()), Hf.shape[1],
                                       None if d_lens is None else ctypes.c_void_p(d_lens.data_ptr()), frames, ctypes.c_void_p(d_n.data_ptr()),
                                       ctypes.c_void_p(st)), "lizg_border_nodes_dev")
    torch.cuda.synchronize()
    return d_n.cpu().numpy()


class PilotRefiner:
    """Gauss-Newton on H against the known pilots (lizg_gn_*), chunk frames at once."""

    def __init__(self, n, subch, span, chunk=8):
        self._h = lib().lizg_gn_new(n, subch, span, chunk)
        if not self._h:
            raise LizgError("lizg_gn_new: " + lib().lizg_last_error().decode())
        self.n, self.chunk = n, chunk

    def refine(self, luma, reg, steps=3, stream=None):
        """luma frames x h x w uint8, reg frames x (9 + 2 nodes) float32. Returns (reg refined, loss, improved)."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(reg, np.float32).copy()).cuda()
        d_loss = torch.zeros(frames, dtype=torch.float32, device="cuda")
        d_imp = torch.zeros(frames, dtype=torch.int32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_gn_refine_dev(self._h, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_r.data_ptr()), frames, steps,
                                        ctypes.c_void_p(d_loss.data_ptr()), ctypes.c_void_p(d_imp.data_ptr()), ctypes.c_void_p(st)), "lizg_gn_refine_dev")
        torch.cuda.synchronize()
        return d_r.cpu().numpy(), d_loss.cpu().numpy(), d_imp.cpu().numpy()

    def pictures(self, luma, reg, stream=None):
        """The sampled picture and its 8 tangents: frames x 9 x n x n float32."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(reg, np.float32)).cuda()
        d_p = torch.zeros((frames, 9, self.n, self.n), dtype=torch.float32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _check(lib().lizg_gn_pictures_dev(self._h, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_r.data_ptr()), frames,
                                          ctypes.c_void_p(d_p.data_ptr()), ctypes.c_void_p(st)), "lizg_gn_pictures_dev")
        torch.cuda.synchronize()
        return d_p.cpu().numpy()

    def __del__(self):
        if getattr(self, "_h", None):
            lib().lizg_gn_free(self._h)
            self._h = None


class EngineBatch(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int), ("d_luma", ctypes.c_void_p), ("w", ctypes.c_int), ("h", ctypes.c_int), ("pitch", ctypes.c_int),
                ("frame_stride", ctypes.c_int64), ("d_reg", ctypes.c_void_p), ("frames", ctypes.c_int), ("out", RxOut)]


class Engine:
    """The multi-stream engine: one receiver handle per picture format; run() decodes one batch per format, each on
    its format's own stream from its own CUDA graph, together."""

    def __init__(self):
        self._h = lib().lizg_engine_new()
        if not self._h:
            raise LizgError("lizg_engine_new failed: %s" % lib().lizg_last_error().decode())
        self.formats = []

    def add_format(self, n, subch, span, max_frames):
        i = _check(lib().lizg_engine_add_format(self._h, n, subch, span, max_frames), "lizg_engine_add_format")
        self.formats.append(Format(n, subch, span))
        return i

    def run_dev(self, batches, stream):
        """batches: list of (format, d_luma ptr, w, h, pitch, frame_stride, d_reg ptr, frames, RxOut)."""
        arr = (EngineBatch * len(batches))(*[EngineBatch(*b) for b in batches])
        _check(lib().lizg_engine_run_dev(self._h, ctypes.cast(arr, ctypes.c_void_p), len(batches), ctypes.c_void_p(stream)), "lizg_engine_run_dev")

    def set_mixed(self, mixed):
        """1: stage-wise across formats (one column pass, row pass and decode grid over every format's items, the
        whole run one graph); 0: a graph a format on its own stream. Returns the previous setting."""
        return _check(lib().lizg_engine_set_mixed(self._h, int(mixed)), "lizg_engine_set_mixed")

    def autotune(self, batches, stream):
        """Runs the batches both ways, keeps the faster: (mode, [ms a graph a format, ms stage-wise])."""
        arr = (EngineBatch * len(batches))(*[EngineBatch(*b) for b in batches])
        ms = (ctypes.c_float * 2)()
        mode = _check(lib().lizg_engine_autotune(self._h, ctypes.cast(arr, ctypes.c_void_p), len(batches), ctypes.c_void_p(stream), ms),
                      "lizg_engine_autotune")
        return mode, [ms[0], ms[1]]

    @property
    def launches(self):
        return lib().lizg_engine_launches(self._h)

    def rx_variant(self, format, tier):
        """Tier `tier`'s LDPC kernel variant in format `format`'s receiver (lizg_rx_variant)."""
        return _check(lib().lizg_rx_variant(ctypes.c_void_p(lib().lizg_engine_rx(self._h, format)), tier), "lizg_rx_variant")

    def close(self):
        if self._h:
            lib().lizg_engine_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


FIELD_PARAMS = 8 + 2 * 49


class FieldRefiner:
    """The registration refined by its adjoint (lizg_field_*): Gauss-Newton over H and the 7 x 7 anchor field against
    the pilots, the timing track and the anchors' centres, chunk frames a pass."""

    def __init__(self, n, subch, span, chunk=8):
        L = lib()
        if not hasattr(L, "_field"):
            P, I = ctypes.c_void_p, ctypes.c_int
            L.lizg_field_new.argtypes = [I, I, I, I]
            L.lizg_field_new.restype = P
            L.lizg_field_free.argtypes = [P]
            L.lizg_field_refine_dev.argtypes = [P, P, I, I, ctypes.c_int64, P, I, I, P, P, P, P, P]
            L.lizg_field_terms_dev.argtypes = [P, P, I, I, ctypes.c_int64, P, P, I, P, P, P]
            L._field = True
        self._h = L.lizg_field_new(n, subch, span, chunk)
        if not self._h:
            raise LizgError("lizg_field_new: " + L.lizg_last_error().decode())
        self._h = ctypes.c_void_p(self._h)
        self.n, self.span, self.chunk = n, span, chunk

    def refine_dev(self, d_luma, w, h, frame_stride, d_reg, frames, steps=3, anchors=None, d_gate=None, d_loss=None, d_improved=None, stream=0):
        """Device pointers; anchors: an AnchorOut of device pointers (frames x 49) or None."""
        _check(lib().lizg_field_refine_dev(self._h, ctypes.c_void_p(d_luma), w, h, frame_stride, ctypes.c_void_p(d_reg), frames, steps,
                                           None if anchors is None else ctypes.byref(anchors), None if d_gate is None else ctypes.c_void_p(d_gate),
                                           None if d_loss is None else ctypes.c_void_p(d_loss),
                                           None if d_improved is None else ctypes.c_void_p(d_improved), ctypes.c_void_p(stream)),
               "lizg_field_refine_dev")

    def terms(self, luma, reg, theta, anchors=None):
        """The three terms (pilots, track, anchors) at parameters theta (frames x FIELD_PARAMS) about reg: frames x 3 x
        (1 + FIELD_PARAMS) float64, each term's loss then its gradient. anchors: a dict of numpy ok, u, v (frames x 49)."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(reg, np.float32).reshape(frames, -1)).cuda()
        d_t = torch.from_numpy(np.ascontiguousarray(theta, np.float32).reshape(frames, FIELD_PARAMS)).cuda()
        d_o = torch.zeros((frames, 3, 1 + FIELD_PARAMS), dtype=torch.float64, device="cuda")
        keep = None
        if anchors is not None:
            keep = {k: torch.from_numpy(np.ascontiguousarray(anchors[k], np.uint8 if k == "ok" else np.float32)).cuda() for k in ("ok", "u", "v")}
            z = keep["u"]
            ao = AnchorOut(keep["ok"].data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), keep["u"].data_ptr(), keep["v"].data_ptr())
        _check(lib().lizg_field_terms_dev(self._h, ctypes.c_void_p(d_l.data_ptr()), w, h, h * w, ctypes.c_void_p(d_r.data_ptr()),
                                          ctypes.c_void_p(d_t.data_ptr()), frames, None if keep is None else ctypes.byref(ao),
                                          ctypes.c_void_p(d_o.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "lizg_field_terms_dev")
        torch.cuda.synchronize()
        return d_o.cpu().numpy()

    def refine(self, luma, reg, steps=3, anchors=None, gate=None):
        """luma frames x h x w uint8, reg frames x (9 + 2 nodes): (refined reg, loss, improved)."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(reg, np.float32).reshape(frames, -1).copy()).cuda()
        d_loss = torch.zeros(frames, dtype=torch.float32, device="cuda")
        d_imp = torch.zeros(frames, dtype=torch.int32, device="cuda")
        d_g = None if gate is None else torch.from_numpy(np.ascontiguousarray(gate, np.uint8)).cuda()
        keep = None
        if anchors is not None:
            keep = {k: torch.from_numpy(np.ascontiguousarray(anchors[k], np.uint8 if k == "ok" else np.float32)).cuda() for k in ("ok", "u", "v")}
            z = keep["u"]
            keep["out"] = AnchorOut(keep["ok"].data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), keep["u"].data_ptr(), keep["v"].data_ptr())
        self.refine_dev(d_l.data_ptr(), w, h, h * w, d_r.data_ptr(), frames, steps, None if keep is None else keep["out"],
                        None if d_g is None else d_g.data_ptr(), d_loss.data_ptr(), d_imp.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return d_r.cpu().numpy(), d_loss.cpu().numpy(), d_imp.cpu().numpy()

    def close(self):
        if getattr(self, "_h", None):
            lib().lizg_field_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Refiner:
    """The registration's refinement from the anchors (lizg_refine_*) for frames of one ring span."""

    def __init__(self, span, max_frames):
        self._h = lib().lizg_refiner_new(span, max_frames)
        if not self._h:
            raise LizgError("lizg_refiner_new failed: %s" % lib().lizg_last_error().decode())

    def refine_dev(self, d_luma, w, h, frame_stride, d_reg, frames, rounds, d_found=None, d_lens=None, stream=0):
        _check(lib().lizg_refine_dev(self._h, ctypes.c_void_p(d_luma), w, h, frame_stride, ctypes.c_void_p(d_reg), frames, rounds,
                                     None if d_found is None else ctypes.c_void_p(d_found), None if d_lens is None else ctypes.c_void_p(d_lens),
                                     ctypes.c_void_p(stream)), "lizg_refine_dev")

    def refine(self, luma, reg, rounds=3):
        """luma frames x h x w uint8, reg frames x (9 + 2 nx ny): returns (refined reg, anchors found, lens frames x 15)."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        if lu.ndim == 2:
            lu = lu[None]
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(np.asarray(reg, np.float32).reshape(frames, -1))).cuda()
        d_f = torch.zeros(frames, dtype=torch.int32, device="cuda")
        d_lens = torch.zeros((frames, 15), dtype=torch.float64, device="cuda")
        self.refine_dev(d_l.data_ptr(), w, h, w * h, d_r.data_ptr(), frames, rounds, d_f.data_ptr(), d_lens.data_ptr(),
                        torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return d_r.cpu().numpy(), d_f.cpu().numpy(), d_lens.cpu().numpy()

    def register_dev(self, d_luma, w, h, frame_stride, d_reg, frames, d_rim=None, d_quad=None, d_held=None, d_lens=None, anchors=None, stream=0):
        """lizg_anchor_register_dev on device pointers; anchors: an AnchorOut or None."""
        p = lambda x: None if x is None else ctypes.c_void_p(x)
        _check(lib().lizg_anchor_register_dev(self._h, ctypes.c_void_p(d_luma), p(d_rim), w, h, frame_stride, ctypes.c_void_p(d_reg), p(d_quad),
                                              frames, p(d_held), p(d_lens), None if anchors is None else ctypes.byref(anchors),
                                              ctypes.c_void_p(stream)), "lizg_anchor_register_dev")

    def register(self, luma, reg, quad=None, rim=None):
        """The reference's registration from the anchors for frames x h x w uint8 and their registrations (H the corners';
        frames x (9 + 2 nx ny)): a dict of reg, quad, held, lens and the anchors' ok, peak, dx, dy, u, v."""
        import torch
        lu = np.ascontiguousarray(luma, np.uint8)
        if lu.ndim == 2:
            lu = lu[None]
        frames, h, w = lu.shape
        d_l = torch.from_numpy(lu).cuda()
        d_rim = None if rim is None else torch.from_numpy(np.ascontiguousarray(rim, np.uint8).reshape(lu.shape)).cuda()
        d_r = torch.from_numpy(np.ascontiguousarray(np.asarray(reg, np.float32).reshape(frames, -1))).cuda()
        d_q = torch.from_numpy(np.ascontiguousarray(np.asarray(quad, np.float32).reshape(frames, 8))).cuda() if quad is not None else \
            torch.zeros((frames, 8), dtype=torch.float32, device="cuda")
        d_held = torch.zeros(frames, dtype=torch.int32, device="cuda")
        d_lens = torch.zeros((frames, 15), dtype=torch.float64, device="cuda")
        ao = {"ok": torch.zeros((frames, 49), dtype=torch.uint8, device="cuda")}
        for k in ("peak", "dx", "dy", "u", "v"):
            ao[k] = torch.zeros((frames, 49), dtype=torch.float32, device="cuda")
        out = AnchorOut(*[ao[k].data_ptr() for k in ("ok", "peak", "dx", "dy", "u", "v")])
        # with no quad given the corners come from H; the buffer then only receives them
        self.register_dev(d_l.data_ptr(), w, h, w * h, d_r.data_ptr(), frames, None if d_rim is None else d_rim.data_ptr(),
                          d_q.data_ptr() if quad is not None else None, d_held.data_ptr(), d_lens.data_ptr(), out,
                          torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        res = {"reg": d_r.cpu().numpy(), "held": d_held.cpu().numpy(), "lens": d_lens.cpu().numpy()}
        res["quad"] = d_q.cpu().numpy() if quad is not None else None
        for k, v in ao.items():
            res[k] = v.cpu().numpy()
        return res

    def close(self):
        if self._h:
            lib().lizg_refiner_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RawFrame(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int), ("row_stride", ctypes.c_uint32), ("pixel_stride", ctypes.c_uint32), ("x0", ctypes.c_uint32),
                ("y0", ctypes.c_uint32), ("bin", ctypes.c_uint32), ("levels", ctypes.c_float * 9)]


def ingest_pixels(px, fmt, w=None):
    """frames x h x stride bytes of liz_pixfmt fmt (or one frame, 2-D), w pixels a row (default the stride's worth), to
    luma on the GPU: frames x h x w."""
    import torch
    a = np.ascontiguousarray(px, np.uint8)
    if a.ndim == 2:
        a = a[None]
    frames, h, stride = a.shape
    bpp = 1 if fmt == LIZG_PIX_GREY8 else 4
    w = stride // bpp if w is None else w
    d = torch.from_numpy(a).cuda()
    o = torch.zeros((frames, h, w), dtype=torch.uint8, device="cuda")
    _check(lib().lizg_ingest_pixels_dev(ctypes.c_void_p(d.data_ptr()), w, h, stride, h * stride, fmt, frames, ctypes.c_void_p(o.data_ptr()),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "lizg_ingest_pixels_dev")
    torch.cuda.synchronize()
    return o.cpu().numpy()


LIZG_PIX_GREY8, LIZG_PIX_RGBX8, LIZG_PIX_RGBA8, LIZG_PIX_BGRA8 = 1, 2, 3, 4


def develop(fmt, planes, row_stride, pixel_stride, x0, y0, bin_, levels, ox, oy, w, h):
    """frames x plane bytes (or one plane, 1-D) developed on the GPU: frames x h x w luma."""
    import torch
    a = np.ascontiguousarray(planes, np.uint8)
    if a.ndim == 1:
        a = a[None]
    frames, nbytes = a.shape
    r = RawFrame(fmt, row_stride, pixel_stride, x0, y0, bin_, (ctypes.c_float * 9)(*[float(v) for v in levels]))
    d = torch.from_numpy(a).cuda()
    o = torch.zeros((frames, h, w), dtype=torch.uint8, device="cuda")
    _check(lib().lizg_develop_dev(ctypes.byref(r), ctypes.c_void_p(d.data_ptr()), nbytes, nbytes, frames, ox, oy, w, h,
                                  ctypes.c_void_p(o.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "lizg_develop_dev")
    torch.cuda.synchronize()
    return o.cpu().numpy()
