"""pc_convolve_noalloc: the entry point for callers that cannot allocate
device memory (plug-ins in hosts that own all GPU memory, code under an
allocator that forbids cudaMalloc, real-time threads that must not block in
the driver).  Its result must match the allocating engine (a handle with the
same one-level layout, run through pc_process_device) within the parity
tolerance, on two calls in a row (the second call must clear the state the
first one left in the shared static scratch array).

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

from partconv_gb300 import PC_PLANAR, PartConvMulti
from partconv_gb300 import _native as nat
from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _noalloc(x_d, h_d, y_d, frames, h_len, n0, stream):
    return nat.lib().pc_convolve_noalloc(C.c_void_p(x_d.data_ptr()), frames, C.c_void_p(h_d.data_ptr()), h_len,
                                         C.c_void_p(y_d.data_ptr()), n0, C.c_void_p(stream))


def test_noalloc_matches_engine_on_two_calls(gpu):
    import torch

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(1234)
    for call, (n0, h_len) in enumerate([(128, 7000), (256, 20000)]):
        h = wl.decaying_ir(rng, h_len, 0.3)
        frames = n0 * (h_len // n0 + 48)
        x = (0.1 * rng.standard_normal(frames)).astype(np.float32)
        x_d = torch.from_numpy(x).to(dev)
        h_d = torch.from_numpy(h).to(dev)

        m = PartConvMulti()
        m.setup_layout(48000, n0, 1, 1, [dict(ir=h, N=[n0], P=[0])])
        y_ref = torch.empty_like(x_d)
        m.process_device(y_ref.view(1, -1), x_d.view(1, -1), frames, PC_PLANAR)

        y = torch.full_like(x_d, float("nan"))
        rc = _noalloc(x_d, h_d, y, frames, h_len, n0, stream)
        assert rc == nat.PC_OK, nat.lib().pc_last_error(None)
        torch.cuda.synchronize()
        a = y.cpu().numpy()
        b = y_ref.cpu().numpy()
        assert np.all(np.isfinite(a)), f"call {call}: unwritten output"
        assert wl.rel_l2(a, b) <= TOL, f"call {call}: rel L2 {wl.rel_l2(a, b):.3e}"
        assert wl.rel_l2(a, wl.conv_fp64(x, h, frames)) <= TOL


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import torch

    dev = torch.device("cuda", 0)
    n0 = 64
    h_len = 4_000_000   # needs ~2 x 8 B per tap of spectra: more than the 32 MiB array
    x_d = torch.zeros(n0 * 4, device=dev)
    h_d = torch.zeros(h_len, device=dev)
    y_d = torch.zeros_like(x_d)
    rc = _noalloc(x_d, h_d, y_d, n0 * 4, h_len, n0, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == nat.PC_ERR_LIMIT
    assert b"static array" in nat.lib().pc_last_error(None)
    rc = _noalloc(x_d, h_d, y_d, n0 * 4 + 1, 100, n0, 0)
    assert rc == nat.PC_ERR_ARG
