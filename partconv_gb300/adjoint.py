"""Differentiable partitioned convolution for torch.

``PartitionedConvFunction`` is a ``torch.autograd.Function`` whose forward
and backward are the hand-written CUDA kernels of the pcd_* C ABI: the
forward pass is the FDL over all blocks of every level, dL/dx uses the
conjugated filter spectra anti-causally, and dL/dh is a partitioned
cross-correlation of the input with dL/dy in the same level layout.
``PartitionedConv`` is a module holding a learnable impulse response.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as nat
from ._native import PartConvError


class DiffPlan:
    """Layout, batch and length of one differentiable convolution."""

    def __init__(self, N, P, ir_len: int, batch: int, length: int):
        self._lib = nat.lib()
        Nv = np.ascontiguousarray(N, dtype=np.int32)
        Pv = np.ascontiguousarray(P, dtype=np.int32).copy()
        msg = C.create_string_buffer(256)
        self._p = self._lib.pcd_create(len(Nv), Nv.ctypes.data_as(nat._i32p), Pv.ctypes.data_as(nat._i32p),
                                       int(ir_len), int(batch), int(length), msg, 256)
        if not self._p:
            raise PartConvError(nat.PC_ERR_LAYOUT, msg.value.decode())
        self.N, self.P = list(Nv), list(Pv)
        self.ir_len, self.batch, self.length = int(ir_len), int(batch), int(length)
        self.workspace_bytes = int(self._lib.pcd_workspace_bytes(self._p))

    def _check(self, code):
        if code != nat.PC_OK:
            raise PartConvError(code, self._lib.pcd_last_error(self._p).decode())

    def new_workspace(self, device):
        return torch.empty(self.workspace_bytes, dtype=torch.uint8, device=device)

    def forward(self, x, h, y, ws, stream):
        self._check(self._lib.pcd_forward(self._p, C.c_void_p(x.data_ptr()), C.c_void_p(h.data_ptr()),
                                          C.c_void_p(y.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_void_p(stream)))

    def backward(self, x, h, gy, gx, gh, ws, recompute: bool, stream):
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        self._check(self._lib.pcd_backward(self._p, ptr(x), ptr(h), ptr(gy), ptr(gx), ptr(gh),
                                           C.c_void_p(ws.data_ptr()), int(bool(recompute)), C.c_void_p(stream)))

    def kernel_launches(self) -> int:
        return int(self._lib.pcd_kernel_launches(self._p))

    def __del__(self):
        p = getattr(self, "_p", None)
        if p:
            try:
                self._lib.pcd_destroy(p)
            except Exception:
                pass
            self._p = None


class PartitionedConvFunction(torch.autograd.Function):
    """y = (x * h)[..., :T] for x [batch, T] and h [ir_len], float32 CUDA.

    recompute=True frees the spectra between forward and backward (the
    backward pass rebuilds them from x and h) when memory matters."""

    @staticmethod
    def forward(ctx, x, h, plan: DiffPlan, recompute: bool = False):
        x = x.contiguous()
        h = h.contiguous()
        if x.dtype != torch.float32 or h.dtype != torch.float32 or not x.is_cuda:
            raise PartConvError(nat.PC_ERR_ARG, "float32 CUDA tensors expected")
        if tuple(x.shape) != (plan.batch, plan.length) or h.numel() != plan.ir_len:
            raise PartConvError(nat.PC_ERR_ARG, "shapes do not match the plan")
        stream = torch.cuda.current_stream(x.device).cuda_stream
        ws = plan.new_workspace(x.device)
        y = torch.empty_like(x)
        plan.forward(x, h, y, ws, stream)
        ctx.plan = plan
        ctx.recompute = recompute
        ctx.ws = None if recompute else ws
        ctx.save_for_backward(x, h)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, h = ctx.saved_tensors
        plan = ctx.plan
        gy = gy.contiguous()
        stream = torch.cuda.current_stream(gy.device).cuda_stream
        ws = ctx.ws if ctx.ws is not None else plan.new_workspace(gy.device)
        gx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        gh = torch.zeros_like(h) if ctx.needs_input_grad[1] else None
        plan.backward(x, h, gy, gx, gh, ws, ctx.ws is None, stream)
        ctx.ws = None
        return gx, gh, None, None


class PartitionedConv(torch.nn.Module):
    """A learnable impulse response applied by partitioned convolution."""

    def __init__(self, h_init, N, P, batch: int, length: int, recompute: bool = False):
        super().__init__()
        self.h = torch.nn.Parameter(torch.as_tensor(np.asarray(h_init, np.float32)).clone())
        self.plan = DiffPlan(N, P, self.h.numel(), batch, length)
        self.recompute = recompute

    def forward(self, x):
        return PartitionedConvFunction.apply(x, self.h, self.plan, self.recompute)
