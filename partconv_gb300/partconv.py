"""The ``partconv`` Python module surface on the GB300 engine.

Mirrors the SWIG module of ebattenberg/partconv (src/partconv.i:3-12, which
wraps src/partconv.h): ``PartConvFilter``, ``PartConvMax``, ``DelayBuffer``,
``DoubleBuffer``, ``intArray`` and ``doubleArray``, plus ``PartConvMulti``
(not wrapped by the reference's SWIG file; added here for the multi-instance
drop-in).  Scripts written against the reference module, e.g. src/tune.py,
run after ``import partconv`` (the top-level module of this repository) or
``from partconv_gb300 import partconv``.

Error behaviour follows the reference where it returns codes
(``PartConvFilter.setup`` returns 1 for a rejected layout); where the
reference calls ``exit(-1)`` these classes raise ``PartConvError``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from ._native import PartConvError
from .multi import PartConvMulti, PartConvMultiRelaxed, Waiter  # noqa: F401


# --------------------------------------------------------------------------
# SWIG carrays helpers (src/partconv.i:10-12: %array_class(int, intArray),
# %array_class(double, doubleArray))
# --------------------------------------------------------------------------
class _CArray:
    _dtype = None

    def __init__(self, nelements: int):
        self._a = np.zeros(int(nelements), dtype=self._dtype)

    def __getitem__(self, i):
        return self._a[i].item()

    def __setitem__(self, i, v):
        self._a[i] = v

    def __len__(self):
        return len(self._a)

    def cast(self):
        return self._a

    def __array__(self, dtype=None, copy=None):
        return self._a if dtype is None else self._a.astype(dtype)

    @classmethod
    def frompointer(cls, arr):
        out = cls(0)
        out._a = np.asarray(arr, dtype=cls._dtype)
        return out


class intArray(_CArray):
    _dtype = np.int32


class doubleArray(_CArray):
    _dtype = np.float64


def _as_ints(v, n=None):
    a = np.asarray(v.cast() if isinstance(v, _CArray) else v, dtype=np.int32)
    return np.ascontiguousarray(a[:n] if n is not None else a)


# --------------------------------------------------------------------------
class PartConvFilter:
    """src/partconv.h:40-114 / src/partconv.cpp:70-648 on the GPU."""

    def __init__(self, inVerbosity: int = 0, inSampleRate: int = 44100):
        self._lib = nat.lib()
        self.verbosity = inVerbosity
        self.FS = inSampleRate
        self._h = None
        self.M = 0
        self.N = None
        self.num_parts = None

    def _check(self, code):
        if code != nat.PC_OK:
            raise PartConvError(code, self._lib.pcf_last_error(self._h).decode())

    def setup(self, M, N_in, num_parts_in, impulse=None, fftwOptLevel=1, wisdom=None) -> int:
        """Returns 0, or 1 when the layout is rejected (like the reference).
        fftwOptLevel and wisdom are accepted for compatibility (no FFTW)."""
        if self._h is not None:
            self.cleanup()
        M = int(M)
        N = _as_ints(N_in, M)
        P = _as_ints(num_parts_in, M).copy()
        self._h = self._lib.pcf_create(int(self.verbosity), int(self.FS))
        if impulse is None:
            ir_p, ir_len = None, 0
        else:
            self._ir = np.ascontiguousarray(np.asarray(impulse, dtype=np.float32).ravel())
            ir_p, ir_len = self._ir.ctypes.data_as(nat._f32p), len(self._ir)
        r = self._lib.pcf_setup(self._h, M, N.ctypes.data_as(nat._i32p), P.ctypes.data_as(nat._i32p), ir_p, ir_len, 0)
        if r == nat.PC_ERR_LAYOUT or r == nat.PC_ERR_LIMIT:
            self.last_error = self._lib.pcf_last_error(self._h).decode()
            if self.verbosity:
                print("PartConvFilter ERROR:", self.last_error)
            self._lib.pcf_destroy(self._h)
            self._h = None
            return 1
        self._check(r)
        self.M = M
        self.N = N
        self.num_parts = P
        if isinstance(num_parts_in, _CArray):
            num_parts_in[M - 1] = int(P[M - 1])
        if self.verbosity > 0:
            lay = ", ".join(f"{n}x{p}" for n, p in zip(N, P))
            print(f"\nPartitioning Specs:\npartitioning: {lay}\nfilter latency: {1000.0 * N[0] / self.FS:g} ms")
        return 0

    def bench(self, L, trials=100, pollute_every=0, max_time=0.1, benchData=None) -> float:
        bd = None
        if benchData is not None:
            bd_arr = np.zeros(2 * self.M, np.float64)
            bd = bd_arr.ctypes.data_as(C.POINTER(C.c_double))
        t = self._lib.pcf_bench(self._h, int(L), int(trials), int(pollute_every), float(max_time), bd)
        if t < 0:
            raise PartConvError(nat.PC_ERR_CUDA, self._lib.pcf_last_error(self._h).decode() or "bench failed")
        if benchData is not None:
            benchData[2 * L] = bd_arr[2 * L]
            benchData[2 * L + 1] = bd_arr[2 * L + 1]
        return t

    def reset(self):
        self._check(self._lib.pcf_reset(self._h))

    def sync_levels(self):
        self._check(self._lib.pcf_sync_levels(self._h, 0))

    def sync_levels_relaxed(self):
        self._check(self._lib.pcf_sync_levels(self._h, 1))

    def input(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.size < int(self.N[0]):
            raise PartConvError(nat.PC_ERR_ARG, "input holds fewer than N[0] samples")
        self._check(self._lib.pcf_input(self._h, x.ctypes.data_as(nat._f32p)))

    def _output(self, y, relaxed):
        out = np.zeros(int(self.N[0]), np.float32) if y is None else y
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < int(self.N[0]):
            raise PartConvError(nat.PC_ERR_ARG, "output must be a C-contiguous float32 array of N[0] samples")
        self._check(self._lib.pcf_output(self._h, out.ctypes.data_as(nat._f32p), int(relaxed)))
        return out

    def output(self, y=None):
        return self._output(y, 0)

    def output_relaxed(self, y=None):
        return self._output(y, 1)

    def runLevel(self, L) -> int:
        self._check(self._lib.pcf_run_level(self._h, int(L)))
        return 0

    def cleanup(self) -> int:
        if self._h is not None:
            self._lib.pcf_destroy(self._h)
            self._h = None
        return 0

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass


# --------------------------------------------------------------------------
class PartConvMax:
    """src/partconv.h:117-204 / src/partconv.cpp:653-1396: n inputs, m outputs,
    k impulse responses in one float array, three channel modes
    (partconv.cpp:661-708) and part counts derived from the block sizes
    (partconv.cpp:718-728).  Runs on the batched GB300 engine."""

    def __init__(self, inVerbosity: int = 0):
        self.verbosity = inVerbosity
        self._m = None
        self.frameNum = 0

    def setup(self, inSampleRate, n, m, k, impulses, filterLength, stride, blockSizes, levels, fftwOptLevel=1,
              wisdom=None, max_threads_per_level=1, max_level0_threads=0) -> int:
        n, m, k = int(n), int(m), int(k)
        if n == m and n == k:            # parallel filtering, distinct IRs
            pairs = [(i, i, i) for i in range(k)]
        elif n == m and k == 1:          # parallel, identical IR
            pairs = [(0, j, j) for j in range(n)]
        elif m == n * k:                 # filterbank
            pairs = [(i, j, i * n + j) for i in range(k) for j in range(n)]
        else:
            if self.verbosity:
                print("PartConvMax::setup() does not support requested channel configuration")
            return 1
        bs = _as_ints(blockSizes, int(levels))
        nlev = int(levels)
        P = np.zeros(nlev, np.int32)
        total = 0
        for i in range(nlev - 1):
            P[i] = 2 * bs[i + 1] // bs[i] - 2
            total += int(bs[i]) * int(P[i])
            if total >= filterLength:
                nlev = i + 1
                break
        N = [int(v) for v in bs[:nlev]]
        P = [int(v) for v in P[:nlev]]
        imp = np.asarray(impulses, dtype=np.float32).ravel()
        irs = []
        for i in range(k):
            if stride == 1:
                irs.append(imp[filterLength * i: filterLength * (i + 1)])
            else:
                irs.append(imp[stride * (filterLength * i + np.arange(filterLength))])
        pcs = [dict(ir=irs[ir_i], N=N, P=P, in_ch=ic, out_ch=oc) for ir_i, ic, oc in pairs]
        self._m = PartConvMulti(self.verbosity)
        self._m.setup_layout(int(inSampleRate), N[0], n, m, pcs)
        self.FS = int(inSampleRate)
        self.buffer_size = N[0]
        self.max_block_size = max(N)
        self.numInputChannels = n
        self.numOutputChannels = m
        self.outbuffers = [np.zeros(N[0], np.float32) for _ in range(m)]
        self.inbuffers = [np.zeros(N[0], np.float32) for _ in range(n)]
        self.frameNum = 0
        return 0

    def run(self, output=None, input=None) -> int:
        """output / input: sequences of per-channel float32 arrays (float**);
        default to self.outbuffers / self.inbuffers."""
        output = self.outbuffers if output is None else output
        input = self.inbuffers if input is None else input
        x = np.stack([np.asarray(c, np.float32)[: self.buffer_size] for c in input], axis=1)
        y = np.zeros((self.buffer_size, self.numOutputChannels), np.float32)
        self._m.run(y, np.ascontiguousarray(x), self.buffer_size)
        for o in range(self.numOutputChannels):
            output[o][: self.buffer_size] = y[:, o]
        self.frameNum += 1
        return 0

    def reset(self):
        self._m.reset()

    def cleanup(self) -> int:
        if self._m is not None:
            self._m.cleanup()
        return 0


# --------------------------------------------------------------------------
def _device_zeros(n):
    import torch

    if not torch.cuda.is_available():
        raise PartConvError(nat.PC_ERR_CUDA, "DelayBuffer/DoubleBuffer need a CUDA device")
    return torch.zeros(int(n), dtype=torch.float32, device="cuda")


class DelayBuffer:
    """src/partconv.cpp:1401-1472: a frame ring that returns whole blocks
    delayed by `delay` frames; kept in device memory."""

    def __init__(self, frameSize: int, blockSize: int, delay: int):
        self.frameSize = int(frameSize)
        self.framesPerBlock = int(blockSize)
        self.readFrameDelay = int(delay) - self.framesPerBlock - 1
        rem = (self.readFrameDelay + 1) % self.framesPerBlock
        size = self.readFrameDelay + 1 + (self.framesPerBlock - rem)
        self.numBlocks = size // self.framesPerBlock + 1
        self.bufferSize = self.numBlocks * self.framesPerBlock
        self._mem = _device_zeros(self.bufferSize * self.frameSize)
        self._init()

    def _init(self):
        self.readBlock = self.numBlocks - 1
        self.writeBlock = self.readFrameDelay // self.framesPerBlock
        self.writeFrame = self.readFrameDelay % self.framesPerBlock

    def write(self, x):
        import torch

        f = self.writeBlock * self.framesPerBlock + self.writeFrame
        src = torch.as_tensor(np.asarray(x, np.float32)[: self.frameSize])
        self._mem[f * self.frameSize:(f + 1) * self.frameSize].copy_(src)
        self.writeFrame += 1
        if self.writeFrame == self.framesPerBlock:
            self.writeFrame = 0
            self.writeBlock = (self.writeBlock + 1) % self.numBlocks

    def read(self, y=None):
        if self.readBlock == self.writeBlock:   # the reference exits here (partconv.cpp:1449-1455)
            raise PartConvError(nat.PC_ERR_STATE,
                                f"readBlock ({self.readBlock}) == writeBlock ({self.writeBlock})")
        f = self.readBlock * self.framesPerBlock
        blk = self._mem[f * self.frameSize:(f + self.framesPerBlock) * self.frameSize].cpu().numpy()
        if y is not None:
            y[: blk.size] = blk
            return y
        return blk

    def prepNextRead(self):
        self.readBlock = (self.readBlock + 1) % self.numBlocks

    def reset(self):
        self._mem.zero_()
        self._init()


class DoubleBuffer:
    """src/partconv.cpp:1477-1511: read/write buffer pair in device memory."""

    def __init__(self, inSize: int):
        self.size = int(inSize)
        self._bufs = [_device_zeros(self.size), _device_zeros(self.size)]
        self._rd = 0

    def swap(self):
        self._rd = 1 - self._rd

    def getReadBuffer(self):
        return self._bufs[self._rd]

    def getWriteBuffer(self):
        return self._bufs[1 - self._rd]

    def reset(self):
        for b in self._bufs:
            b.zero_()
