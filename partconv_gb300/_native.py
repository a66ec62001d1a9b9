"""ctypes binding of libpartconv_gb300.so (the C ABI in include/partconv_gb300.h).

Loading never falls back to anything else: if the library is missing or a
call needs a GPU that is not there, the error propagates.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

PC_OK = 0
PC_ERR_ARG = 1
PC_ERR_LAYOUT = 2
PC_ERR_CONFIG = 3
PC_ERR_IO = 4
PC_ERR_CUDA = 5
PC_ERR_NOMEM = 6
PC_ERR_STATE = 7
PC_ERR_LIMIT = 8
PC_INTERLEAVED = 0
PC_PLANAR = 1
PC_MAX_BLOCK = 65536
PC_MAX_LEVELS = 16
PC_NOALLOC_SCRATCH_BYTES = 32 << 20

_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int)


class PCInfo(C.Structure):
    _fields_ = [
        ("fs", C.c_int),
        ("buffer_size", C.c_int),
        ("num_input_channels", C.c_int),
        ("num_output_channels", C.c_int),
        ("num_pcs", C.c_int),
        ("max_block_size", C.c_int),
        ("relaxed", C.c_int),
        ("hyperperiod", C.c_int),
        ("frame_num", C.c_longlong),
        ("device_bytes", C.c_longlong),
        ("step_blocks", C.c_int),
        ("spread_bins", C.c_int),
        ("spread_parts", C.c_int),
    ]


class PCKernelStats(C.Structure):
    _fields_ = [
        ("name", C.c_char * 32),
        ("launches", C.c_longlong),
        ("total_ms", C.c_double),
        ("alg_bytes", C.c_double),
    ]


class PCRtStats(C.Structure):
    _fields_ = [
        ("callbacks", C.c_longlong),
        ("misses", C.c_longlong),
        ("period_us", C.c_double),
        ("compute_mean_us", C.c_double),
        ("latency_p50_us", C.c_double),
        ("latency_p99_us", C.c_double),
        ("latency_max_us", C.c_double),
        ("wall_s", C.c_double),
    ]


PCS_LOAD_MAX_POOLS = 8


class PCSLoadStats(C.Structure):
    _fields_ = [
        ("requests", C.c_longlong), ("finished", C.c_longlong), ("peak_concurrent", C.c_longlong),
        ("steps", C.c_longlong), ("blocks", C.c_longlong),
        ("wall_s", C.c_double), ("audio_s", C.c_double),
        ("latency_p50_us", C.c_double), ("latency_p99_us", C.c_double), ("latency_max_us", C.c_double),
        ("miss_rate", C.c_double),
        ("n_pools", C.c_int),
        ("pool_block", C.c_int * PCS_LOAD_MAX_POOLS),
        ("pool_steps", C.c_longlong * PCS_LOAD_MAX_POOLS), ("pool_blocks", C.c_longlong * PCS_LOAD_MAX_POOLS),
        ("pool_p50_us", C.c_double * PCS_LOAD_MAX_POOLS), ("pool_p99_us", C.c_double * PCS_LOAD_MAX_POOLS),
        ("pool_miss_rate", C.c_double * PCS_LOAD_MAX_POOLS),
    ]


# name -> (restype, argtypes); mirrors include/partconv_gb300.h
SIGNATURES = {
    "pc_check_layout": (C.c_int, [C.c_int, _i32p, _i32p, C.c_int, C.c_int, _i32p, C.c_char_p, C.c_int]),
    "pc_create": (C.c_void_p, [C.c_int]),
    "pc_setup_config": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_double]),
    "pc_setup_layout": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _i32p,
                                  C.POINTER(_f32p), _i32p, _i32p, _i32p, _f32p, _i32p]),
    "pc_set_relaxed": (C.c_int, [C.c_void_p, C.c_int]),
    "pc_set_step_blocks": (C.c_int, [C.c_void_p, C.c_int]),
    "pc_set_tiles": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "pc_run": (C.c_int, [C.c_void_p, _f32p, _f32p, C.c_int]),
    "pc_process": (C.c_int, [C.c_void_p, _f32p, _f32p, C.c_longlong, C.c_int]),
    "pc_process_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p]),
    "pc_reset": (C.c_int, [C.c_void_p]),
    "pc_cleanup": (C.c_int, [C.c_void_p]),
    "pc_destroy": (None, [C.c_void_p]),
    "pc_last_error": (C.c_char_p, [C.c_void_p]),
    "pc_get_info": (C.c_int, [C.c_void_p, C.POINTER(PCInfo)]),
    "pc_get_layout": (C.c_int, [C.c_void_p, C.c_int, _i32p, _i32p, _i32p]),
    "pc_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "pc_profile_kernels": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(PCKernelStats), C.c_int,
                                     C.POINTER(C.c_int)]),
    "pc_rt_drive": (C.c_int, [C.c_void_p, _f32p, _f32p, C.c_longlong, C.c_double, C.c_int, C.POINTER(PCRtStats)]),
    "pc_convolve_noalloc": (C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                      C.c_void_p]),
    "pcf_create": (C.c_void_p, [C.c_int, C.c_int]),
    "pcf_setup": (C.c_int, [C.c_void_p, C.c_int, _i32p, _i32p, _f32p, C.c_int, C.c_int]),
    "pcf_sync_levels": (C.c_int, [C.c_void_p, C.c_int]),
    "pcf_input": (C.c_int, [C.c_void_p, _f32p]),
    "pcf_run_level": (C.c_int, [C.c_void_p, C.c_int]),
    "pcf_output": (C.c_int, [C.c_void_p, _f32p, C.c_int]),
    "pcf_reset": (C.c_int, [C.c_void_p]),
    "pcf_bench": (C.c_double, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]),
    "pcf_cleanup": (C.c_int, [C.c_void_p]),
    "pcf_destroy": (None, [C.c_void_p]),
    "pcf_last_error": (C.c_char_p, [C.c_void_p]),
    "pcf_get_parts": (C.c_int, [C.c_void_p, _i32p]),
    "pcf_overlap_error": (C.c_int, [C.c_void_p]),
    "pcm_create": (C.c_void_p, [C.c_int]),
    "pcm_setup": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _f32p, C.c_int]),
    "pcm_process_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p]),
    "pcm_reset": (C.c_int, [C.c_void_p]),
    "pcm_profile_kernels": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(PCKernelStats), C.c_int,
                                      C.POINTER(C.c_int)]),
    "pcm_device_bytes": (C.c_longlong, [C.c_void_p]),
    "pcm_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "pcm_last_error": (C.c_char_p, [C.c_void_p]),
    "pcm_destroy": (None, [C.c_void_p]),
    "pcd_create": (C.c_void_p, [C.c_int, _i32p, _i32p, C.c_int, C.c_int, C.c_longlong, C.c_char_p, C.c_int]),
    "pcd_workspace_bytes": (C.c_longlong, [C.c_void_p]),
    "pcd_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pcd_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_int, C.c_void_p]),
    "pcd_destroy": (None, [C.c_void_p]),
    "pcd_last_error": (C.c_char_p, [C.c_void_p]),
    "pcd_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "pcs_create": (C.c_void_p, [C.c_int, C.c_longlong, C.c_int]),
    "pcs_admit": (C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int, _i32p, _i32p, C.POINTER(C.c_int)]),
    "pcs_admit_async": (C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int, _i32p, _i32p, C.POINTER(C.c_int)]),
    "pcs_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "pcs_is_live": (C.c_int, [C.c_void_p, C.c_int]),
    "pcs_release": (C.c_int, [C.c_void_p, C.c_int]),
    "pcs_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "pcs_query": (C.c_int, [C.c_void_p]),
    "pcs_sync": (C.c_int, [C.c_void_p]),
    "pcs_bytes_in_use": (C.c_longlong, [C.c_void_p]),
    "pcs_live": (C.c_int, [C.c_void_p]),
    "pcs_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "pcs_last_error": (C.c_char_p, [C.c_void_p]),
    "pcs_destroy": (None, [C.c_void_p]),
    "pcs_run_load": (C.c_int, [C.POINTER(C.c_void_p), _i32p, C.c_int, C.c_int, C.POINTER(C.c_double), _i32p, _i32p,
                               C.POINTER(C.c_longlong), C.POINTER(_f32p), _i32p, _i32p, _i32p, _i32p, _f32p,
                               C.c_longlong, C.c_ulonglong, C.c_int, C.c_double, C.c_double,
                               C.POINTER(PCSLoadStats)]),
}

_lock = threading.Lock()
_lib = None


def lib(build: bool = True):
    """Load the in-tree library (building it first when sources changed), or
    the library named by $PARTCONV_GB300_LIB (a build with other options)."""
    global _lib
    with _lock:
        if _lib is None:
            path = os.environ.get("PARTCONV_GB300_LIB") or (_build.build() if build else _build.LIB_PATH)
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def lib_path() -> str:
    return _build.LIB_PATH


class PartConvError(RuntimeError):
    """A failing C-ABI call: .code is the PC_ERR_* status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(handle, code: int) -> None:
    if code != PC_OK:
        msg = lib().pc_last_error(handle)
        raise PartConvError(code, msg.decode() if msg else "")
