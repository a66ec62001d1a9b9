"""MIMO per-bin channel-sum engine (config 3) against the oracle run as one
PartConvMulti PC per path with the reference's time-domain mix
(src/partconvMulti.cpp:911-921).  Tolerance: relative L2 <= 1e-5 per output."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PC_INTERLEAVED, PC_PLANAR
from partconv_gb300 import workloads as wl
from partconv_gb300.mimo import PartConvMIMO

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _oracle_mimo(irs, x, N, P, threads=None):
    """Per output: run every input's path as an independent mono stream and
    sum in input order."""
    n_in, n_out, _ = irs.shape
    y = np.zeros((n_out, x.shape[1]), np.float64)
    for o in range(n_out):
        ys, _ = oracle.run_streams([(N, P)] * n_in, [irs[i, o] for i in range(n_in)], x, N[0], threads)
        acc = np.zeros(x.shape[1], np.float32)
        for i in range(n_in):
            acc += ys[i]
        y[o] = acc
    return y


@pytest.mark.parametrize("N,P,n_in,n_out,L", [
    ([64, 256, 1024], [4, 3, 0], 3, 4, 5000),
    ([128, 2048], [16, 15], 2, 3, 1 << 15),
    ([256], [0], 4, 1, 3000),
    # 398 older parts per spread task (one input each): long MAC term lists
    ([64], [400], 8, 2, 25600),
])
def test_mimo_matches_oracle(gpu, N, P, n_in, n_out, L):
    rng = np.random.default_rng(L + n_in)
    irs = np.stack([wl.decaying_ir(rng, L, 0.3) for _ in range(n_in * n_out)]).reshape(n_in, n_out, L)
    frames = N[0] * ((L + 2 * N[-1]) // N[0] + 16)
    x = (0.1 * rng.standard_normal((n_in, frames))).astype(np.float32)
    m = PartConvMIMO()
    m.setup(irs, N, P)
    y = m.process(x)
    ref = _oracle_mimo(irs, x, N, P)
    for o in range(n_out):
        assert wl.rel_l2(y[o], ref[o]) <= TOL, o
        ref64 = sum(wl.conv_fp64(x[i], irs[i, o], frames) for i in range(n_in))
        assert wl.rel_l2(y[o], ref64) <= TOL
    # interleaved layout and a second call from reset give the same samples
    import torch

    m.reset()
    xi = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    yi = torch.empty((frames, n_out), dtype=torch.float32, device="cuda")
    m.process_device(yi, xi, frames, PC_INTERLEAVED)
    torch.cuda.synchronize()
    assert np.array_equal(yi.cpu().numpy().T, y)
    assert m.kernel_launches() > 0


def test_mimo_config3_full_size(gpu):
    """Config 3: 64 x 64 paths of 2^15 taps (T60 0.5 s, x 1/64), 2^18 input
    frames plus the IR flush, layout 128x16 | 2048x15."""
    c = wl.cfg3()
    irs, N, P = c["irs"], c["N"], c["P"]
    L = irs.shape[2]
    frames = c["x"].shape[1] + L
    x = np.zeros((c["x"].shape[0], frames), np.float32)
    x[:, : c["x"].shape[1]] = c["x"]
    m = PartConvMIMO()
    m.setup(irs, N, P)
    y = m.process(x)
    # the oracle on a sample of outputs keeps the test to seconds
    for o in (0, 17, 63):
        ys, _ = oracle.run_streams([(N, P)] * irs.shape[0], [irs[i, o] for i in range(irs.shape[0])], x, N[0])
        ref = np.sum(ys, axis=0, dtype=np.float32)
        assert wl.rel_l2(y[o], ref) <= TOL, o
