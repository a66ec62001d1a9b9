"""The reference's own PartConvFilter, compiled from the reference sources
into oracle/_ref/libpcref.so (Makefile.ref; TEST INFRASTRUCTURE ONLY).

It pins the oracle: tests run the oracle restatement and the reference's
code on the same inputs and compare them.  The reference sources are only
present where the reference checkout is (``PARTCONV_REF_SRC``, default the
checkout this build was made beside), and its MAC is SSE3, so the library
builds on x86_64 hosts only; ``available()`` says whether it can be used.
Fixtures it produced are committed under tests/golden/ for hosts without it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import threading

import numpy as np

from .oracle import _f32, _f32p, _fp, _i32, _ip

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libpcref.so")
_lock = threading.Lock()
_lib = None


def ref_src() -> str:
    return os.environ.get("PARTCONV_REF_SRC", "/root/reference")


def buildable() -> bool:
    src = os.path.join(ref_src(), "src")
    return (platform.machine() in ("x86_64", "AMD64") and os.path.exists(os.path.join(src, "partconv.cpp"))
            and os.path.exists(os.path.join(src, "buffers.cpp")))


def build(force: bool = False) -> str | None:
    """Compile oracle/_ref/libpcref.so when the reference sources are here."""
    if not buildable():
        return LIB_PATH if os.path.exists(LIB_PATH) else None
    args = ["make", "-s", "-f", os.path.join(_HERE, "Makefile.ref"), f"REF={ref_src()}"]
    if force:
        args.insert(2, "-B")
    subprocess.run(args, check=True)
    return LIB_PATH


def available() -> bool:
    return buildable() or (platform.machine() in ("x86_64", "AMD64") and os.path.exists(LIB_PATH))


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            L.ref_layout_check.argtypes = [C.c_int, _i32p_t(), _i32p_t(), C.c_int]
            L.ref_layout_check.restype = C.c_int
            L.ref_multi_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p_t(), _i32p_t(), _i32p_t(),
                                           C.POINTER(_f32p), _i32p_t(), _i32p_t(), _i32p_t(), _f32p, _i32p_t(),
                                           C.c_int, C.c_char_p, C.c_int]
            L.ref_multi_create.restype = C.c_void_p
            L.ref_multi_run.argtypes = [C.c_void_p, _f32p, _f32p, C.c_long]
            L.ref_multi_run.restype = C.c_int
            L.ref_multi_reset.argtypes = [C.c_void_p]
            L.ref_multi_destroy.argtypes = [C.c_void_p]
            _lib = L
    return _lib


def _i32p_t():
    return C.POINTER(C.c_int)


def layout_check(N, P, ir_len):
    """PartConvFilter::setup's verdict: (status, P with the last level
    recomputed); status 0 accepted, 1 rejected."""
    N = _i32(N)
    P = _i32(P).copy()
    st = lib().ref_layout_check(len(N), _ip(N), _ip(P), int(ir_len))
    return st, P


class RefMulti:
    """PartConvMulti / PartConvMultiRelaxed callbacks over the reference's
    PartConvFilter instances; same arguments as oracle.OracleMulti."""

    def __init__(self, buffer_size, n_in, n_out, pcs, relaxed=False):
        self.buffer_size, self.n_in, self.n_out = buffer_size, n_in, n_out
        irs = [_f32(p["ir"]) for p in pcs]
        self._irs = irs
        M = _i32([len(p["N"]) for p in pcs])
        Nf = _i32(np.concatenate([np.asarray(p["N"]) for p in pcs]))
        Pf = _i32(np.concatenate([np.asarray(p.get("P", [1] * len(p["N"]))) for p in pcs]))
        ptrs = (_f32p * len(irs))(*[_fp(a) for a in irs])
        lens = _i32([len(a) for a in irs])
        msg = C.create_string_buffer(512)
        self._h = lib().ref_multi_create(
            buffer_size, n_in, n_out, len(pcs), _ip(M), _ip(Nf), _ip(Pf), ptrs, _ip(lens),
            _ip(_i32([p.get("in_ch", 0) for p in pcs])), _ip(_i32([p.get("out_ch", 0) for p in pcs])),
            _fp(_f32([p.get("scale", 1.0) for p in pcs])), _ip(_i32([p.get("mute", 0) for p in pcs])),
            int(bool(relaxed)), msg, 512)
        if not self._h:
            raise ValueError(msg.value.decode())

    def run(self, x: np.ndarray) -> np.ndarray:
        """x: [frames, n_in] interleaved (frames a multiple of buffer_size)."""
        x = _f32(x).reshape(-1, self.n_in)
        out = np.zeros((x.shape[0], self.n_out), np.float32)
        if lib().ref_multi_run(self._h, _fp(out), _fp(x), x.shape[0]):
            raise RuntimeError("frames must be a multiple of buffer_size")
        return out

    def reset(self):
        lib().ref_multi_reset(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().ref_multi_destroy(h)
            self._h = None
