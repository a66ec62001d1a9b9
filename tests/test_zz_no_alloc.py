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


# (block size, IR taps): two multi-part layouts with spread tasks (P >= 3),
# then the smallest and largest block sizes with P = 2 and a one-part IR, so
# the path without spread tasks runs too
CASES = [(128, 7000), (256, 20000), (16, 20), (1024, 1500), (64, 50)]


def test_noalloc_matches_engine_on_consecutive_calls(gpu):
    import torch

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(1234)
    for call, (n0, h_len) in enumerate(CASES):
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
        assert wl.rel_l2(a, b) <= TOL, f"call {call} ({n0}, {h_len}): rel L2 {wl.rel_l2(a, b):.3e}"
        assert wl.rel_l2(a, wl.conv_fp64(x, h, frames)) <= TOL


def test_noalloc_call_leaves_device_memory_unchanged(gpu):
    """After a first call on the device, a call takes no device memory: the
    free memory the driver reports is the same before and after it, and the
    repeated call gives the same bits."""
    import torch

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(99)
    n0, h_len = 256, 30000
    h_d = torch.from_numpy(wl.decaying_ir(rng, h_len, 0.5)).to(dev)
    frames = n0 * 200
    x_d = torch.from_numpy((0.1 * rng.standard_normal(frames)).astype(np.float32)).to(dev)
    y1 = torch.empty_like(x_d)
    y2 = torch.empty_like(x_d)
    assert _noalloc(x_d, h_d, y1, frames, h_len, n0, stream) == nat.PC_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    assert _noalloc(x_d, h_d, y2, frames, h_len, n0, stream) == nat.PC_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
    assert torch.equal(y1, y2)


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
