"""Differentiable partitioned convolution (config 4): forward against FP64,
hand-written adjoints against dense torch FFT-conv autograd (float64) and
FP64 central finite differences (step 1e-3) on 64 random coordinates.

Tolerances: forward relative L2 <= 1e-5 (the forward parity bar); dL/dh and
dL/dx relative L2 <= 1e-6 against FP64 central finite differences on 64
coordinates each (the adjoint target) and against float64 dense autograd."""
import numpy as np
import pytest

from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_GRAD = 1e-6


def _dense_conv(x, h):
    """(x * h)[..., :T] by FFT in the dtype of the inputs (torch autograd)."""
    import torch

    T, L = x.shape[-1], h.shape[-1]
    n = 1 << (T + L - 1 - 1).bit_length()
    return torch.fft.irfft(torch.fft.rfft(x, n) * torch.fft.rfft(h, n), n)[..., :T]


def _case(B, T, L, seed):
    rng = np.random.default_rng(seed)
    x = (0.1 * rng.standard_normal((B, T))).astype(np.float32)
    h = (0.01 * rng.standard_normal(L)).astype(np.float32)
    ht = wl.decaying_ir(rng, L, 1.0)
    return x, h, ht


@pytest.mark.parametrize("N,P,B,T,L", [
    ([64, 256], [4, 0], 2, 64 * 40, 1500),
    ([128, 1024], [8, 0], 3, 128 * 64, 9000),
    ([256], [0], 2, 256 * 20, 700),
])
def test_forward_and_gradients_small(gpu, N, P, B, T, L):
    import torch

    from partconv_gb300.adjoint import PartitionedConv

    x, h0, ht = _case(B, T, L, L)
    dev = torch.device("cuda")
    xd = torch.from_numpy(x).to(dev).requires_grad_(True)
    mod = PartitionedConv(h0, N, P, B, T).to(dev)
    y = mod(xd)
    y64 = np.stack([wl.conv_fp64(x[b], h0, T) for b in range(B)])
    assert wl.rel_l2(y.detach().cpu().numpy(), y64) <= TOL
    target = _dense_conv(torch.from_numpy(x).double().to(dev), torch.from_numpy(ht).double().to(dev)).float()
    loss = torch.mean((y - target) ** 2)
    loss.backward()
    # dense autograd in float64
    xr = torch.from_numpy(x).double().to(dev).requires_grad_(True)
    hr = torch.from_numpy(h0).double().to(dev).requires_grad_(True)
    lr = torch.mean((_dense_conv(xr, hr) - target.double()) ** 2)
    lr.backward()
    assert wl.rel_l2(mod.h.grad.cpu().numpy(), hr.grad.cpu().numpy()) <= TOL_GRAD
    assert wl.rel_l2(xd.grad.cpu().numpy(), xr.grad.cpu().numpy()) <= TOL_GRAD


def test_recompute_matches_stored_spectra(gpu):
    import torch

    from partconv_gb300.adjoint import PartitionedConv

    x, h0, _ = _case(2, 128 * 50, 4000, 5)
    outs = []
    for recompute in (False, True):
        xd = torch.from_numpy(x).cuda().requires_grad_(True)
        mod = PartitionedConv(h0, [128, 1024], [8, 0], 2, 128 * 50, recompute=recompute).cuda()
        mod(xd).pow(2).sum().backward()
        outs.append((mod.h.grad.cpu().numpy(), xd.grad.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_config4_adjoint(gpu):
    """Config 4: batch 8 x 2^18 samples, learnable 2^16-tap IR from
    N(0, 0.01^2), target IR T60 1 s, MSE loss, layout 512x8 | 4096x15.
    Both gradients against FP64 central differences (step 1e-3, 64 random
    coordinates each) and float64 dense autograd, relative L2 <= 1e-6."""
    import torch

    from partconv_gb300.adjoint import PartitionedConv

    c = wl.cfg4()
    x, h0, ht = c["x"], c["h_init"], c["h_target"]
    B, T = x.shape
    L = len(h0)
    dev = torch.device("cuda")
    xd = torch.from_numpy(x).to(dev).requires_grad_(True)
    mod = PartitionedConv(h0, c["N"], c["P"], B, T).to(dev)
    t64 = np.stack([wl.conv_fp64(x[b], ht, T) for b in range(B)])
    y64 = np.stack([wl.conv_fp64(x[b], h0, T) for b in range(B)])
    target = torch.from_numpy(t64.astype(np.float32)).to(dev)
    y = mod(xd)
    assert wl.rel_l2(y.detach().cpu().numpy(), y64) <= TOL
    loss = torch.mean((y - target) ** 2)
    loss.backward()
    gh = mod.h.grad.cpu().numpy().astype(np.float64)
    gx = xd.grad.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(77)
    coords_h = np.sort(rng.choice(L, 64, replace=False))
    coords_x = [(int(b), int(i)) for b, i in zip(rng.integers(0, B, 64), rng.choice(T, 64, replace=False))]
    fd_h, fd_x = wl.fd_grads_fp64(x, h0, t64, coords_h, coords_x, 1e-3)
    err_h = wl.rel_l2(gh[coords_h], fd_h)
    err_x = wl.rel_l2(np.array([gx[b, i] for b, i in coords_x]), fd_x)
    print(f"config 4 vs FP64 central differences: dL/dh {err_h:.2e}, dL/dx {err_x:.2e}")
    assert err_h <= TOL_GRAD
    assert err_x <= TOL_GRAD
    # and against float64 dense autograd on every tap and sample
    xr = torch.from_numpy(x).double().to(dev).requires_grad_(True)
    hr = torch.from_numpy(h0).double().to(dev).requires_grad_(True)
    lr = torch.mean((_dense_conv(xr, hr) - torch.from_numpy(t64).to(dev)) ** 2)
    lr.backward()
    assert wl.rel_l2(gh, hr.grad.cpu().numpy()) <= TOL_GRAD
    assert wl.rel_l2(gx, xr.grad.cpu().numpy()) <= TOL_GRAD
