"""PartConvMulti / PartConvMultiRelaxed on the GB300 engine.

Mirrors the reference class of src/partconvMulti.h:52-165
(ebattenberg/partconv): ``setup(config_file, max_threads_per_level,
max_level0_threads, min_work)``, ``run(output, input, frameCount)``,
``reset()``, ``cleanup()`` and the public fields ``FS``, ``buffer_size``,
``max_block_size``, ``verbosity``, ``numInputChannels``,
``numOutputChannels``, ``frameNum``, ``output_mix``, ``input_mix``,
``doneWaiter``, ``lastFrame``.  Where the reference calls ``exit(-1)``
(bad config, wrong frame count) these methods raise ``PartConvError``;
success returns 0 like the C++ methods.

Beyond the reference: ``setup_layout`` (no config file), ``process`` (many
callbacks per call from host arrays) and ``process_device`` (device
tensors/pointers on a CUDA stream).
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _native as nat
from ._native import PartConvError  # noqa: F401  (re-export)


class Waiter:
    """src/partconvMulti.h:152-165: wait until a value reaches a target."""

    def __init__(self, inVal: int = 0):
        self._cv = threading.Condition()
        self._val = inVal
        self._init = inVal

    def waitFor(self, target: int, timeout: float | None = None) -> bool:
        with self._cv:
            return self._cv.wait_for(lambda: self._val == target, timeout)

    def changeAndSignal(self, newVal: int) -> None:
        with self._cv:
            self._val = newVal
            self._cv.notify_all()


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class PartConvMulti:
    relaxed = 0

    def __init__(self, verbosity: int = 0, step_blocks: int = 1, tiles=None):
        """step_blocks > 1: offline throughput mode, `step_blocks` base blocks
        per step (pc_set_step_blocks); run() is then unavailable and process()
        wants a multiple of step_blocks * buffer_size frames.
        tiles: (bins, parts) per spread task (pc_set_tiles), e.g. the
        autotuner's choice; None keeps the default."""
        self.verbosity = verbosity
        self._lib = nat.lib()
        self._h = self._lib.pc_create(int(verbosity))
        if not self._h:
            raise PartConvError(nat.PC_ERR_NOMEM, "pc_create failed")
        if step_blocks != 1:
            nat.check(self._h, self._lib.pc_set_step_blocks(self._h, int(step_blocks)))
        if tiles:
            nat.check(self._h, self._lib.pc_set_tiles(self._h, int(tiles[0]), int(tiles[1])))
        self.FS = 0
        self.buffer_size = 0
        self.max_block_size = 0
        self.numInputChannels = 0
        self.numOutputChannels = 0
        self.output_mix = None
        self.input_mix = None
        self.doneWaiter = None
        self.lastFrame = 0
        self._frame_num = 0

    # -- setup ---------------------------------------------------------------
    def setup(self, config_file_name: str, max_threads_per_level: int = 1, max_level0_threads: int = 0,
              min_work: float = 0) -> int:
        """PartConvMulti::setup (src/partconvMulti.cpp:23-718) from a pc.config file."""
        nat.check(self._h, self._lib.pc_setup_config(self._h, str(config_file_name).encode(),
                                                     int(max_threads_per_level), int(max_level0_threads),
                                                     float(min_work)))
        self._after_setup()
        return 0

    def setup_layout(self, FS: int, buffer_size: int, numInputChannels: int, numOutputChannels: int,
                     pcs: list[dict]) -> int:
        """Setup without a file.  pcs: dicts with keys ir, N, P (last level's
        count ignored), in_ch, out_ch, scale (1.0), mute (0)."""
        irs = [_f32(p["ir"]) for p in pcs]
        self._keep = irs
        M = _i32([len(p["N"]) for p in pcs])
        Nf = _i32(np.concatenate([np.asarray(p["N"]) for p in pcs]))
        Pf = _i32(np.concatenate([np.asarray(p.get("P", [0] * len(p["N"]))) for p in pcs]))
        ptrs = (nat._f32p * len(irs))(*[a.ctypes.data_as(nat._f32p) for a in irs])
        lens = _i32([len(a) for a in irs])
        inc = _i32([p.get("in_ch", 0) for p in pcs])
        outc = _i32([p.get("out_ch", 0) for p in pcs])
        sc = _f32([p.get("scale", 1.0) for p in pcs])
        mu = _i32([p.get("mute", 0) for p in pcs])
        ip = lambda a: a.ctypes.data_as(nat._i32p)  # noqa: E731
        nat.check(self._h, self._lib.pc_setup_layout(
            self._h, int(FS), int(buffer_size), int(numInputChannels), int(numOutputChannels), len(pcs),
            ip(M), ip(Nf), ip(Pf), ptrs, ip(lens), ip(inc), ip(outc), sc.ctypes.data_as(nat._f32p), ip(mu)))
        self._after_setup()
        return 0

    def _after_setup(self):
        if self.relaxed:
            nat.check(self._h, self._lib.pc_set_relaxed(self._h, 1))
        info = self.info()
        self.FS = info.fs
        self.buffer_size = info.buffer_size
        self.max_block_size = info.max_block_size
        self.numInputChannels = info.num_input_channels
        self.numOutputChannels = info.num_output_channels
        self.step_blocks = info.step_blocks
        self.output_mix = np.zeros(self.buffer_size * self.numOutputChannels, np.float32)
        self.input_mix = np.zeros(self.buffer_size * self.numInputChannels, np.float32)
        self._frame_num = 0

    # -- processing ------------------------------------------------------------
    @property
    def frameNum(self) -> int:
        return self._frame_num

    def run(self, output: np.ndarray, input: np.ndarray, frameCount: int) -> int:
        """PartConvMulti::run: one callback of interleaved float32 frames.
        ``output`` must be a writable float32 C-contiguous array."""
        if output.dtype != np.float32 or not output.flags.c_contiguous:
            raise PartConvError(nat.PC_ERR_ARG, "output must be a C-contiguous float32 array")
        x = _f32(input)
        if x.size < frameCount * self.numInputChannels or output.size < frameCount * self.numOutputChannels:
            raise PartConvError(nat.PC_ERR_ARG, "buffer smaller than frameCount frames")
        nat.check(self._h, self._lib.pc_run(self._h, output.ctypes.data_as(nat._f32p),
                                            x.ctypes.data_as(nat._f32p), int(frameCount)))
        self._frame_num += 1
        if self.doneWaiter is not None and self._frame_num == self.lastFrame:
            self.doneWaiter.changeAndSignal(1)
        return 0

    def process(self, x: np.ndarray, layout: int = nat.PC_INTERLEAVED) -> np.ndarray:
        """Many callbacks at once.  Interleaved x: [frames, nIn] -> [frames, nOut];
        planar x: [nIn, frames] -> [nOut, frames]."""
        x = _f32(x)
        if layout == nat.PC_INTERLEAVED:
            x = x.reshape(-1, self.numInputChannels)
            frames = x.shape[0]
            y = np.empty((frames, self.numOutputChannels), np.float32)
        else:
            x = x.reshape(self.numInputChannels, -1)
            frames = x.shape[1]
            y = np.empty((self.numOutputChannels, frames), np.float32)
        nat.check(self._h, self._lib.pc_process(self._h, y.ctypes.data_as(nat._f32p), x.ctypes.data_as(nat._f32p),
                                                int(frames), int(layout)))
        self._frame_num += frames // self.buffer_size
        return y

    def process_into(self, y, x, frames: int, layout: int = nat.PC_INTERLEAVED) -> int:
        """pc_process into caller-owned host buffers (numpy arrays or host
        pointers, e.g. pinned memory); no allocation on the Python side."""
        py = y.ctypes.data if hasattr(y, "ctypes") else int(y)
        px = x.ctypes.data if hasattr(x, "ctypes") else int(x)
        nat.check(self._h, self._lib.pc_process(self._h, C.cast(py, nat._f32p), C.cast(px, nat._f32p), int(frames),
                                                int(layout)))
        self._frame_num += frames // self.buffer_size
        return 0

    def process_device(self, d_out, d_in, frames: int, layout: int = nat.PC_INTERLEAVED, stream=None) -> int:
        """Device buffers (torch tensors or integer device pointers) on a
        CUDA stream (torch stream, raw handle int; None means torch's current
        stream).  Enqueues only; the caller synchronises."""
        po = d_out.data_ptr() if hasattr(d_out, "data_ptr") else int(d_out)
        pi = d_in.data_ptr() if hasattr(d_in, "data_ptr") else int(d_in)
        if stream is None:
            import torch

            stream = torch.cuda.current_stream()
        if hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        nat.check(self._h, self._lib.pc_process_device(self._h, C.c_void_p(po), C.c_void_p(pi), int(frames),
                                                       int(layout), C.c_void_p(int(stream))))
        self._frame_num += frames // self.buffer_size
        return 0

    def reset(self) -> None:
        nat.check(self._h, self._lib.pc_reset(self._h))
        self._frame_num = 0

    def cleanup(self) -> int:
        nat.check(self._h, self._lib.pc_cleanup(self._h))
        return 0

    # -- introspection -----------------------------------------------------------
    def info(self) -> nat.PCInfo:
        inf = nat.PCInfo()
        nat.check(self._h, self._lib.pc_get_info(self._h, C.byref(inf)))
        return inf

    def layout(self, pc: int):
        M = C.c_int(0)
        N = (C.c_int * nat.PC_MAX_LEVELS)()
        P = (C.c_int * nat.PC_MAX_LEVELS)()
        nat.check(self._h, self._lib.pc_get_layout(self._h, int(pc), C.byref(M), N, P))
        return list(N[:M.value]), list(P[:M.value])

    def kernel_launches(self) -> int:
        return int(self._lib.pc_kernel_launches(self._h))

    def profile_kernels(self, nsteps: int) -> list[dict]:
        """pc_profile_kernels: per-kernel CUDA-event time and algorithmic
        bytes over nsteps further base steps."""
        recs = (nat.PCKernelStats * 8)()
        n = C.c_int(0)
        nat.check(self._h, self._lib.pc_profile_kernels(self._h, int(nsteps), recs, 8, C.byref(n)))
        self._frame_num += nsteps
        return [dict(name=r.name.decode(), launches=r.launches, total_ms=r.total_ms, alg_bytes=r.alg_bytes)
                for r in recs[: n.value]]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.pc_destroy(h)
            except Exception:
                pass
            self._h = None


class PartConvMultiRelaxed(PartConvMulti):
    """src/partconvMulti.h:142-148: output is one base block later."""

    relaxed = 1


def check_layout(N, P, ir_len, relaxed=True):
    """pc_check_layout: returns (status, P with last level recomputed, delays, message)."""
    N = _i32(N)
    P = _i32(P).copy()
    d = np.zeros(len(N), np.int32)
    msg = C.create_string_buffer(256)
    st = nat.lib().pc_check_layout(len(N), N.ctypes.data_as(nat._i32p), P.ctypes.data_as(nat._i32p),
                                   int(ir_len), int(bool(relaxed)), d.ctypes.data_as(nat._i32p), msg, 256)
    return st, P, d, msg.value.decode()
