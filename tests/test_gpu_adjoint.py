"""Differentiable partitioned convolution (config 4): forward against FP64,
hand-written adjoints against dense torch FFT-conv autograd (float64) and
FP64 central finite differences (step 1e-3) on 64 random coordinates.

Tolerances: forward relative L2 <= 1e-5; gradients relative L2 <= 1e-5
against float64 autograd; the finite-difference comparison is reported and
held to 1e-5 (float32 accumulation over 2^21 products bounds it)."""
import numpy as np
import pytest

from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5


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
    assert wl.rel_l2(mod.h.grad.cpu().numpy(), hr.grad.cpu().numpy()) <= TOL
    assert wl.rel_l2(xd.grad.cpu().numpy(), xr.grad.cpu().numpy()) <= TOL


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
    N(0, 0.01^2), target IR T60 1 s, MSE loss, layout 512x8 | 4096x15."""
    import torch

    from partconv_gb300.adjoint import PartitionedConv

    c = wl.cfg4()
    x, h0, ht = c["x"], c["h_init"], c["h_target"]
    B, T = x.shape
    L = len(h0)
    dev = torch.device("cuda")
    xd = torch.from_numpy(x).to(dev)
    mod = PartitionedConv(h0, c["N"], c["P"], B, T).to(dev)
    # targets and the FP64 residual
    x64 = x.astype(np.float64)
    t64 = np.stack([wl.conv_fp64(x[b], ht, T) for b in range(B)])
    y64 = np.stack([wl.conv_fp64(x[b], h0, T) for b in range(B)])
    target = torch.from_numpy(t64.astype(np.float32)).to(dev)
    y = mod(xd)
    assert wl.rel_l2(y.detach().cpu().numpy(), y64) <= TOL
    loss = torch.mean((y - target) ** 2)
    loss.backward()
    gh = mod.h.grad.cpu().numpy().astype(np.float64)
    # FP64 central differences at 64 coordinates: L is quadratic in h, and
    # y(h +- d e_j) = y(h) +- d x shifted by j, so both loss values are exact
    r = y64 - t64
    M = r.size
    rng = np.random.default_rng(77)
    coords = np.sort(rng.choice(L, 64, replace=False))
    d = 1e-3
    fd = np.empty(64)
    for n, j in enumerate(coords):
        xs = np.zeros_like(x64)
        xs[:, j:] = x64[:, : T - j]
        lp = np.sum((r + d * xs) ** 2) / M
        lm = np.sum((r - d * xs) ** 2) / M
        fd[n] = (lp - lm) / (2 * d)
    err_fd = float(np.linalg.norm(gh[coords] - fd) / np.linalg.norm(fd))
    print(f"config 4 dL/dh vs FP64 central differences: relative L2 {err_fd:.2e}")
    assert err_fd <= TOL
    # and against float64 dense autograd on all taps
    hr = torch.from_numpy(h0).double().to(dev).requires_grad_(True)
    lr = torch.mean((_dense_conv(torch.from_numpy(x64).to(dev), hr) - torch.from_numpy(t64).to(dev)) ** 2)
    lr.backward()
    assert wl.rel_l2(gh, hr.grad.cpu().numpy()) <= TOL
