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
REF_SRC = "/root/reference/liblizard/src"

_port = None
_ref = None


class Code(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in "rate z mb kb n k m np nt edges".split()] + [
        ("rowptr", ctypes.c_int * 31), ("col", ctypes.c_int * 160), ("shift", ctypes.c_int * 160)]


def build(ref=True):
    """make the restatement, and the reference where its sources are present."""
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)
    if ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref"], check=True)


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


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


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
