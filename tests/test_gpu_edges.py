"""Edge cases of the CUDA path through the C ABI: the alignment known
answer (impulse in, impulse response out, at zero added latency; one block
later for the Relaxed variant), zero input, one-tap and shorter-than-a-block
IRs, linearity, layout invariance, and the most levels a PC may have
(beyond the four whose output slices level 0 prefetches)."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PartConvMulti, PartConvMultiRelaxed
from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _run(pcs, N0, x, relaxed=False, n_in=1, n_out=1):
    m = PartConvMultiRelaxed() if relaxed else PartConvMulti()
    m.setup_layout(48000, N0, n_in, n_out, pcs)
    y = m.process(x.reshape(-1, n_in))
    m.cleanup()
    return y


@pytest.mark.parametrize("relaxed", [False, True])
@pytest.mark.parametrize("N,P", [([64, 512, 4096], [8, 7, 0]), ([64, 512, 4096], [14, 14, 0]), ([256], [0])])
def test_impulse_gives_the_impulse_response_at_zero_latency(gpu, N, P, relaxed):
    rng = np.random.default_rng(1)
    h = wl.decaying_ir(rng, 9000, 0.2)
    N0 = N[0]
    frames = N0 * ((len(h) + 3 * N0) // N0 + 2)
    x = np.zeros(frames, np.float32)
    at = 3 * N0 + 5
    x[at] = 1.0
    y = _run([dict(ir=h, N=N, P=P)], N0, x, relaxed)[:, 0]
    d = at + (N0 if relaxed else 0)
    blk = d // N0 * N0   # blocks before the impulse's see only zeros
    assert not np.any(y[:blk])
    assert np.abs(y[blk:d]).max() <= 1e-6 * np.abs(h).max()
    assert wl.rel_l2(y[d:d + len(h)], h) <= 1e-6
    assert np.abs(y[d + len(h):]).max() <= 1e-6 * np.abs(h).max()


def test_zero_input_gives_zero_output(gpu):
    rng = np.random.default_rng(2)
    h = wl.decaying_ir(rng, 20000, 0.5)
    y = _run([dict(ir=h, N=[128, 1024, 8192], P=[14, 14, 0])], 128, np.zeros(128 * 300, np.float32))
    assert not np.any(y)


@pytest.mark.parametrize("L", [1, 100])
def test_ir_shorter_than_a_block(gpu, L):
    rng = np.random.default_rng(L)
    h = wl.decaying_ir(rng, L, 0.1)
    x = (0.1 * rng.standard_normal(256 * 40)).astype(np.float32)
    y = _run([dict(ir=h, N=[256], P=[0])], 256, x)[:, 0]
    ref = wl.conv_fp64(x, h, len(x))
    assert wl.rel_l2(y, ref) <= 1e-6


def test_linearity(gpu):
    rng = np.random.default_rng(4)
    h = wl.decaying_ir(rng, 40000, 0.4)
    pcs = [dict(ir=h, N=[256, 2048, 16384], P=[14, 14, 0])]
    n = 256 * 400
    x1 = (0.1 * rng.standard_normal(n)).astype(np.float32)
    x2 = (0.1 * rng.standard_normal(n)).astype(np.float32)
    y1, y2 = _run(pcs, 256, x1)[:, 0], _run(pcs, 256, x2)[:, 0]
    y12 = _run(pcs, 256, (0.75 * x1 - 1.5 * x2).astype(np.float32))[:, 0]
    assert wl.rel_l2(y12, 0.75 * y1.astype(np.float64) - 1.5 * y2) <= 1e-6


def test_layout_invariance(gpu):
    rng = np.random.default_rng(5)
    h = wl.decaying_ir(rng, 50000, 0.5)
    x = (0.1 * rng.standard_normal(256 * 500)).astype(np.float32)
    ya = _run([dict(ir=h, N=[256, 2048, 16384], P=[8, 7, 0])], 256, x)[:, 0]        # every level in step
    yb = _run([dict(ir=h, N=[256, 2048, 16384], P=[14, 14, 0])], 256, x)[:, 0]      # larger levels deferred
    yc = _run([dict(ir=h, N=[256, 1024, 4096], P=[6, 6, 0])], 256, x)[:, 0]
    assert wl.rel_l2(yb, ya) <= 1e-6 and wl.rel_l2(yc, ya) <= 1e-6


def test_eleven_levels(gpu):
    """Block sizes 16 .. 16384 (doubling): six levels beyond the four whose
    output slices the level-0 fire prefetches."""
    rng = np.random.default_rng(6)
    N = [16 << k for k in range(11)]
    P = [2] + [1] * 9 + [0]
    h = wl.decaying_ir(rng, 60000, 0.6)
    x = (0.1 * rng.standard_normal(16 * 6000)).astype(np.float32)
    y = _run([dict(ir=h, N=N, P=P)], 16, x)[:, 0]
    ref = oracle.OracleMulti(16, 1, 1, [dict(ir=h, N=N, P=P)]).run(x[:, None])[:, 0]
    assert wl.rel_l2(y, ref) <= 1e-5
