"""MIMO partitioned convolution: y_o = sum_i x_i * h_{i,o} with per-bin
channel sums (one FFT per input and level block, one inverse FFT per output
and level block).  Wraps the pcm_* C ABI (include/partconv_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from ._native import PartConvError


class PartConvMIMO:
    def __init__(self, verbosity: int = 0):
        self._lib = nat.lib()
        self._h = self._lib.pcm_create(int(verbosity))
        if not self._h:
            raise PartConvError(nat.PC_ERR_NOMEM, "pcm_create failed")

    def _check(self, code):
        if code != nat.PC_OK:
            raise PartConvError(code, self._lib.pcm_last_error(self._h).decode())

    def setup(self, irs, N, P, fs: int = 48000):
        """irs: [n_in, n_out, ir_len] float array; N/P: level layout (last
        level's part count recomputed)."""
        irs = np.ascontiguousarray(irs, dtype=np.float32)
        self.n_in, self.n_out, L = irs.shape
        Nv = np.ascontiguousarray(N, dtype=np.int32)
        Pv = np.ascontiguousarray(P, dtype=np.int32).copy()
        self._check(self._lib.pcm_setup(self._h, int(fs), int(Nv[0]), self.n_in, self.n_out, len(Nv),
                                        Nv.ctypes.data_as(nat._i32p), Pv.ctypes.data_as(nat._i32p),
                                        irs.ctypes.data_as(nat._f32p), int(L)))
        self.N, self.P, self.buffer_size = list(Nv), list(Pv), int(Nv[0])
        return 0

    def process_device(self, d_out, d_in, frames: int, layout: int = nat.PC_PLANAR, stream=None):
        po = d_out.data_ptr() if hasattr(d_out, "data_ptr") else int(d_out)
        pi = d_in.data_ptr() if hasattr(d_in, "data_ptr") else int(d_in)
        if stream is None:
            import torch

            stream = torch.cuda.current_stream()
        if hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        self._check(self._lib.pcm_process_device(self._h, C.c_void_p(po), C.c_void_p(pi), int(frames), int(layout),
                                                 C.c_void_p(int(stream))))

    def process(self, x: np.ndarray) -> np.ndarray:
        """Planar host arrays: x [n_in, frames] -> y [n_out, frames]."""
        import torch

        x = np.ascontiguousarray(x, dtype=np.float32)
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty((self.n_out, x.shape[1]), dtype=torch.float32, device="cuda")
        self.process_device(yd, xd, x.shape[1], nat.PC_PLANAR)
        torch.cuda.synchronize()
        return yd.cpu().numpy()

    def reset(self):
        self._check(self._lib.pcm_reset(self._h))

    def profile_kernels(self, nsteps: int):
        recs = (nat.PCKernelStats * 4)()
        n = C.c_int(0)
        self._check(self._lib.pcm_profile_kernels(self._h, int(nsteps), recs, 4, C.byref(n)))
        return [dict(name=r.name.decode(), launches=r.launches, total_ms=r.total_ms, alg_bytes=r.alg_bytes)
                for r in recs[: n.value]]

    def device_bytes(self) -> int:
        return int(self._lib.pcm_device_bytes(self._h))

    def kernel_launches(self) -> int:
        return int(self._lib.pcm_kernel_launches(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.pcm_destroy(h)
            except Exception:
                pass
            self._h = None
