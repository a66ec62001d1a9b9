"""ctypes wrapper over liboracle.so (test infrastructure only; see __init__)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    srcs = [os.path.join(_HERE, f) for f in ("pc_oracle.cpp", "orc_fft.h")]
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(map(os.path.getmtime, srcs)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            L.orc_layout_check.argtypes = [C.c_int, _i32p, _i32p, C.c_int, C.c_int, _i32p, C.c_char_p, C.c_int]
            L.orc_layout_check.restype = C.c_int
            L.orc_multi_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _i32p,
                                           C.POINTER(_f32p), _i32p, _i32p, _i32p, _f32p, _i32p,
                                           C.c_int, C.c_int, C.c_char_p, C.c_int]
            L.orc_multi_create.restype = C.c_void_p
            L.orc_multi_run.argtypes = [C.c_void_p, _f32p, _f32p, C.c_long]
            L.orc_multi_run.restype = C.c_int
            L.orc_multi_reset.argtypes = [C.c_void_p]
            L.orc_multi_destroy.argtypes = [C.c_void_p]
            L.orc_filter_create.argtypes = [C.c_int, _i32p, _i32p, _f32p, C.c_int, C.c_int, C.c_char_p, C.c_int]
            L.orc_filter_create.restype = C.c_void_p
            for name in ("sync_levels", "sync_levels_relaxed", "reset", "destroy"):
                getattr(L, "orc_filter_" + name).argtypes = [C.c_void_p]
            L.orc_filter_input.argtypes = [C.c_void_p, _f32p]
            L.orc_filter_output.argtypes = [C.c_void_p, _f32p]
            L.orc_filter_output_relaxed.argtypes = [C.c_void_p, _f32p]
            L.orc_filter_run_level.argtypes = [C.c_void_p, C.c_int]
            L.orc_filter_run_level.restype = C.c_int
            L.orc_filter_error.argtypes = [C.c_void_p]
            L.orc_filter_error.restype = C.c_int
            L.orc_filter_parts.argtypes = [C.c_void_p, _i32p]
            L.orc_filter_spectra.argtypes = [C.c_void_p, C.c_int, _f32p]
            L.orc_rfft.argtypes = [C.c_int, _f32p, _f32p]
            L.orc_irfft.argtypes = [C.c_int, _f32p, _f32p]
            L.orc_conv_direct_f64.argtypes = [_f32p, C.c_long, _f32p, C.c_long, C.POINTER(C.c_long),
                                              C.c_long, C.POINTER(C.c_double), C.c_int]
            L.orc_run_streams.argtypes = [C.c_int, _i32p, _i32p, _i32p, C.POINTER(_f32p), _i32p, _f32p,
                                          _f32p, C.c_long, C.c_int, C.c_int, C.c_char_p, C.c_int]
            L.orc_run_streams.restype = C.c_double
            _lib = L
    return _lib


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f32p)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_i32p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def layout_check(N, P, ir_len, relaxed=False):
    """Returns (status, P_with_last_recomputed, delays, message)."""
    N = _i32(N)
    P = _i32(P).copy()
    M = len(N)
    delays = np.zeros(M, np.int32)
    msg = C.create_string_buffer(256)
    st = lib().orc_layout_check(M, _ip(N), _ip(P), int(ir_len), int(bool(relaxed)), _ip(delays), msg, 256)
    return st, P, delays, msg.value.decode()


class OracleMulti:
    """PartConvMulti / PartConvMultiRelaxed restatement.

    pcs: list of dicts {ir, N, P, in_ch, out_ch, scale, mute}.
    schedule: 0 auto (strict restatement if the layout passes the strict
    check, else minimum-latency), 1 strict only, 2 minimum-latency.
    """

    def __init__(self, buffer_size, n_in, n_out, pcs, relaxed=False, schedule=0):
        self.buffer_size, self.n_in, self.n_out = buffer_size, n_in, n_out
        irs = [_f32(p["ir"]) for p in pcs]
        self._irs = irs
        M = _i32([len(p["N"]) for p in pcs])
        Nf = _i32(np.concatenate([np.asarray(p["N"]) for p in pcs]))
        Pf = _i32(np.concatenate([np.asarray(p.get("P", [1] * len(p["N"]))) for p in pcs]))
        ptrs = (_f32p * len(irs))(*[_fp(a) for a in irs])
        lens = _i32([len(a) for a in irs])
        msg = C.create_string_buffer(512)
        self._h = lib().orc_multi_create(
            buffer_size, n_in, n_out, len(pcs), _ip(M), _ip(Nf), _ip(Pf), ptrs, _ip(lens),
            _ip(_i32([p.get("in_ch", 0) for p in pcs])), _ip(_i32([p.get("out_ch", 0) for p in pcs])),
            _fp(_f32([p.get("scale", 1.0) for p in pcs])), _ip(_i32([p.get("mute", 0) for p in pcs])),
            int(bool(relaxed)), int(schedule), msg, 512)
        if not self._h:
            raise ValueError(msg.value.decode())

    def run(self, x: np.ndarray) -> np.ndarray:
        """x: [frames, n_in] interleaved (frames a multiple of buffer_size)."""
        x = _f32(x).reshape(-1, self.n_in)
        out = np.zeros((x.shape[0], self.n_out), np.float32)
        r = lib().orc_multi_run(self._h, _fp(out), _fp(x), x.shape[0])
        if r:
            raise RuntimeError(f"oracle run failed ({r})")
        return out

    def reset(self):
        lib().orc_multi_reset(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_multi_destroy(h)
            self._h = None


class OracleFilter:
    """PartConvFilter restatement with the fine-grained per-level API."""

    def __init__(self, N, P, ir=None, relaxed_check=False):
        N = _i32(N)
        P = _i32(P)
        if ir is None:
            ir = np.ones(int(np.sum(N.astype(np.int64) * P)), np.float32)
        self._ir = _f32(ir)
        msg = C.create_string_buffer(256)
        self._h = lib().orc_filter_create(len(N), _ip(N), _ip(P), _fp(self._ir), len(self._ir),
                                          int(bool(relaxed_check)), msg, 256)
        if not self._h:
            raise ValueError(msg.value.decode())
        self.M = len(N)
        self.N = N.copy()
        self.num_parts = np.zeros(self.M, np.int32)
        lib().orc_filter_parts(self._h, _ip(self.num_parts))

    def sync_levels(self):
        lib().orc_filter_sync_levels(self._h)

    def sync_levels_relaxed(self):
        lib().orc_filter_sync_levels_relaxed(self._h)

    def input(self, x):
        x = _f32(x)
        lib().orc_filter_input(self._h, _fp(x))

    def output(self):
        y = np.zeros(int(self.N[0]), np.float32)
        lib().orc_filter_output(self._h, _fp(y))
        return y

    def output_relaxed(self):
        y = np.zeros(int(self.N[0]), np.float32)
        lib().orc_filter_output_relaxed(self._h, _fp(y))
        return y

    def runLevel(self, L):
        return lib().orc_filter_run_level(self._h, int(L))

    def reset(self):
        lib().orc_filter_reset(self._h)

    def error(self):
        return bool(lib().orc_filter_error(self._h))

    def spectra(self, L):
        n = int(self.N[L])
        out = np.zeros((int(self.num_parts[L]), n + 1, 2), np.float32)
        lib().orc_filter_spectra(self._h, int(L), _fp(out))
        return out[..., 0] + 1j * out[..., 1]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_filter_destroy(h)
            self._h = None


def rfft(x: np.ndarray) -> np.ndarray:
    x = _f32(x)
    n = len(x)
    out = np.zeros((n // 2 + 1, 2), np.float32)
    if lib().orc_rfft(n, _fp(x), _fp(out)):
        raise ValueError("length must be a power of two")
    return out[:, 0] + 1j * out[:, 1]


def irfft(X: np.ndarray, nfft: int) -> np.ndarray:
    Xi = np.zeros((nfft // 2 + 1, 2), np.float32)
    Xi[:, 0] = np.real(X)
    Xi[:, 1] = np.imag(X)
    y = np.zeros(nfft, np.float32)
    if lib().orc_irfft(nfft, _fp(Xi), _fp(y)):
        raise ValueError("length must be a power of two")
    return y


def conv_direct_f64(x, h, idx=None, threads=None) -> np.ndarray:
    """FP64 direct convolution y[n] = sum_k h[k] x[n-k] at indices idx."""
    x = _f32(x)
    h = _f32(h)
    if threads is None:
        threads = os.cpu_count() or 1
    if idx is None:
        n = len(x) + len(h) - 1
        y = np.zeros(n, np.float64)
        lib().orc_conv_direct_f64(_fp(x), len(x), _fp(h), len(h), None, n,
                                  y.ctypes.data_as(C.POINTER(C.c_double)), threads)
        return y
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    y = np.zeros(len(idx), np.float64)
    lib().orc_conv_direct_f64(_fp(x), len(x), _fp(h), len(h), idx.ctypes.data_as(C.POINTER(C.c_long)),
                              len(idx), y.ctypes.data_as(C.POINTER(C.c_double)), threads)
    return y


def run_streams(layouts, irs, x_planar, buffer_size, threads=None):
    """Minimum-latency schedule over independent mono streams on host threads.

    layouts: list of (N, P); irs: list of arrays; x_planar: [S, frames].
    Returns (y [S, frames], wall seconds)."""
    S = len(layouts)
    x = _f32(x_planar)
    frames = x.shape[1]
    irs = [_f32(h) for h in irs]
    M = _i32([len(N) for N, _ in layouts])
    Nf = _i32(np.concatenate([np.asarray(N) for N, _ in layouts]))
    Pf = _i32(np.concatenate([np.asarray(P) for _, P in layouts]))
    ptrs = (_f32p * S)(*[_fp(a) for a in irs])
    lens = _i32([len(a) for a in irs])
    y = np.zeros_like(x)
    msg = C.create_string_buffer(256)
    if threads is None:
        threads = os.cpu_count() or 1
    t = lib().orc_run_streams(S, _ip(M), _ip(Nf), _ip(Pf), ptrs, _ip(lens), _fp(x), _fp(y), frames,
                              buffer_size, threads, msg, 256)
    if t < 0:
        raise ValueError(msg.value.decode())
    return y, t


def run_leveled(N, P, ir, x):
    """One worker thread per level over a mono signal (the reference's
    thread-per-level shape); returns (y, wall seconds).  Bit-identical to the
    sequential minimum-latency restatement."""
    L = lib()
    if not hasattr(L, "_leveled"):
        L.orc_run_leveled.argtypes = [C.c_int, _i32p, _i32p, _f32p, C.c_int, _f32p, _f32p, C.c_long, C.c_char_p,
                                      C.c_int]
        L.orc_run_leveled.restype = C.c_double
        L._leveled = True
    N = _i32(N)
    P = _i32(P).copy()
    ir = _f32(ir)
    x = _f32(x).reshape(-1)
    y = np.zeros_like(x)
    msg = C.create_string_buffer(256)
    t = L.orc_run_leveled(len(N), _ip(N), _ip(P), _fp(ir), len(ir), _fp(x), _fp(y), len(x), msg, 256)
    if t < 0:
        raise ValueError(msg.value.decode())
    return y, t
