"""Several base blocks per step (pc_set_step_blocks): one launch transforms
and convolves K consecutive level-0 blocks of every PC, larger levels run
beside the steps.  Through the C ABI: the same convolution as one-block
steps to float32 rounding, against the oracle at the parity tolerance, with
the state carried across calls and the argument rules enforced."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PC_PLANAR, PartConvError, PartConvMulti, PartConvMultiRelaxed
from partconv_gb300 import _native as nat
from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5      # relative L2 per output channel vs the oracle (as the one-block path)
TOL_ONE = 1e-6  # vs this engine's one-block steps (same partitions, other sum order)


def _ir(rng, n, t60=0.3):
    return wl.decaying_ir(rng, n, t60)


LAYOUTS = [   # N, P, IR length, K
    ([256, 2048, 16384], [14, 14, 0], 131072, 4),   # minimum-slack chain of the batched workload
    ([256, 2048], [14, 0], 40000, 4),
    ([256, 1024, 4096], [4, 4, 0], 20000, 4),       # level 1: slack 0, one step per block
    ([128, 1024, 8192], [8, 7, 0], 60000, 4),       # slack 0 everywhere
    ([64, 256, 1024], [4, 3, 0], 5000, 2),
    ([256], [0], 3000, 4),                          # one level, 12 parts: a partial-sum row
    ([256], [0], 1500, 4),                          # one level, 6 parts: all in the fire
    ([256], [0], 500, 4),                           # one level, 2 parts < K: ring keeps the newest 2
    ([128, 512], [40, 0], 12000, 4),                # 40 level-0 parts: two rows
    ([512, 4096], [8, 15], 65536, 2),               # base block 512, K = 2
]


def _calls(m, x, sizes):
    out, at = [], 0
    for n in sizes:
        out.append(m.process(x[at:at + n]))
        at += n
    return np.concatenate(out)


@pytest.mark.parametrize("N,P,L,K", LAYOUTS)
def test_step_blocks_match_oracle_and_one_block_steps(gpu, N, P, L, K):
    rng = np.random.default_rng(L + K)
    h = _ir(rng, L)
    N0 = N[0]
    step = K * N0
    blocks = (L + 4 * N[-1]) // step + 6
    frames = step * blocks
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    x[frames - L - N0:] = 0.0
    pcs = [dict(ir=h, N=N, P=P)]
    m = PartConvMulti(step_blocks=K)
    m.setup_layout(48000, N0, 1, 1, pcs)
    assert m.step_blocks == K
    # three calls: each call's first step takes its older input from the ring
    cut = [step * (blocks // 3), step * (blocks // 3 + 1)]
    y = _calls(m, x, [cut[0], cut[1], frames - cut[0] - cut[1]])
    ref = oracle.OracleMulti(N0, 1, 1, pcs).run(x)
    one = PartConvMulti()
    one.setup_layout(48000, N0, 1, 1, pcs)
    y1 = one.process(x)
    e_or, e_one = wl.rel_l2(y[:, 0], ref[:, 0]), wl.rel_l2(y[:, 0], y1[:, 0])
    assert e_or <= TOL, e_or
    assert e_one <= TOL_ONE, e_one
    m.reset()
    assert np.array_equal(m.process(x), y)   # call boundaries do not change a bit


def test_step_blocks_mixing_and_reduction(gpu):
    """Mixed outputs, a muted PC and PC-less outputs; a level with N_L = 2 N0
    lowers the requested K = 8 to 2."""
    rng = np.random.default_rng(31)
    N0 = 64
    hs = [_ir(rng, 700 + 900 * i) for i in range(5)]
    pcs = [
        dict(ir=hs[0], N=[64, 256], P=[4, 0], in_ch=0, out_ch=1, scale=0.5),
        dict(ir=hs[1], N=[64], P=[0], in_ch=1, out_ch=1, scale=2.0),
        dict(ir=hs[2], N=[64, 128], P=[2, 0], in_ch=1, out_ch=0, scale=1.0, mute=1),
        dict(ir=hs[3], N=[64, 256, 1024], P=[4, 3, 0], in_ch=2, out_ch=2, scale=-1.0),
        dict(ir=hs[4], N=[64, 512], P=[8, 0], in_ch=0, out_ch=1, scale=1.5),
    ]
    frames = N0 * 256
    x = (0.1 * rng.standard_normal((frames, 3))).astype(np.float32)
    ref = oracle.OracleMulti(N0, 3, 4, pcs).run(x)
    m = PartConvMulti(step_blocks=8)
    m.setup_layout(48000, N0, 3, 4, pcs)
    assert m.step_blocks == 2
    y = m.process(x)
    for o in (1, 2):
        assert wl.rel_l2(y[:, o], ref[:, o]) <= TOL
    assert np.all(y[:, 0] == 0) and np.all(y[:, 3] == 0)
    m.reset()
    yp = m.process(np.ascontiguousarray(x.T), PC_PLANAR)
    assert np.array_equal(y, yp.T)
    # without the 2 N0 level the smallest larger level is 4 N0: K = 4
    m8 = PartConvMulti(step_blocks=8)
    m8.setup_layout(48000, N0, 3, 4, [p for i, p in enumerate(pcs) if i != 2])
    assert m8.step_blocks == 4
    y8 = m8.process(x)
    ref8 = oracle.OracleMulti(N0, 3, 4, [p for i, p in enumerate(pcs) if i != 2]).run(x)
    for o in (1, 2):
        assert wl.rel_l2(y8[:, o], ref8[:, o]) <= TOL


def test_step_blocks_relaxed(gpu):
    rng = np.random.default_rng(32)
    N, P, L = [128, 512, 2048], [4, 3, 0], 7000
    h = _ir(rng, L)
    frames = 128 * 200
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    ref = oracle.OracleMulti(128, 1, 1, [dict(ir=h, N=N, P=P)], relaxed=True).run(x)
    m = PartConvMultiRelaxed(step_blocks=4)
    m.setup_layout(48000, 128, 1, 1, [dict(ir=h, N=N, P=P)])
    assert m.step_blocks == 4
    y = np.concatenate([m.process(x[:128 * 80]), m.process(x[128 * 80:])])
    assert np.all(y[:128] == 0)
    assert wl.rel_l2(y[:, 0], ref[:, 0]) <= TOL


def test_step_blocks_argument_rules(gpu):
    m = PartConvMulti(step_blocks=4)
    m.setup_layout(48000, 256, 1, 1, [dict(ir=np.ones(8000, np.float32), N=[256, 2048], P=[14, 0])])
    assert m.step_blocks == 4
    with pytest.raises(PartConvError) as ei:
        m.run(np.zeros(256, np.float32), np.zeros(256, np.float32), 256)
    assert ei.value.code == nat.PC_ERR_STATE
    with pytest.raises(PartConvError) as ei:
        m.process(np.zeros((256 * 6, 1), np.float32))
    assert ei.value.code == nat.PC_ERR_ARG
    assert m._lib.pc_set_step_blocks(m._h, 2) == nat.PC_ERR_STATE
    # at most 4 blocks per step
    m4 = PartConvMulti(step_blocks=8)
    m4.setup_layout(48000, 128, 1, 1, [dict(ir=np.ones(5000, np.float32), N=[128, 1024], P=[8, 0])])
    assert m4.step_blocks == 4
    # base block 1024: the level-0 kernel takes one block per step
    m1 = PartConvMulti(step_blocks=4)
    m1.setup_layout(48000, 1024, 1, 1, [dict(ir=np.ones(5000, np.float32), N=[1024], P=[0])])
    assert m1.step_blocks == 1


def test_config2_step_blocks_full_size(gpu):
    """The 32 streams of the batched workload with K = 4 vs the oracle."""
    c = wl.cfg2()
    S = len(c["irs"])
    N0 = c["N0"]
    K = 4
    tail = max(len(h) for h in c["irs"])
    frames = (c["x"].shape[1] + tail + K * N0 - 1) // (K * N0) * (K * N0)
    x = np.zeros((S, frames), np.float32)
    x[:, : c["x"].shape[1]] = c["x"]
    pcs = [dict(ir=h, N=N, P=P, in_ch=s, out_ch=s) for s, (h, (N, P)) in enumerate(zip(c["irs"], c["layouts"]))]
    m = PartConvMulti(step_blocks=K)
    m.setup_layout(48000, N0, S, S, pcs)
    assert m.step_blocks == K
    y = m.process(x, PC_PLANAR)
    ref, _ = oracle.run_streams(c["layouts"], c["irs"], x, N0)
    for s in range(S):
        assert wl.rel_l2(y[s], ref[s]) <= TOL, s
