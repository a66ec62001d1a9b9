"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the
same seeded inputs, and against FP64 convolution.  Tolerance: relative L2
error per output channel <= 1e-5 (float32 FFTs of different design)."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PC_INTERLEAVED, PC_PLANAR, PartConvError, PartConvMulti, PartConvMultiRelaxed
from partconv_gb300 import _native as nat
from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _ir(rng, n, t60=0.3):
    return wl.decaying_ir(rng, n, t60)


def _run_callbacks(m, x, N0):
    frames, nin = x.shape
    out = np.zeros((frames, m.numOutputChannels), np.float32)
    buf = np.zeros(N0 * m.numOutputChannels, np.float32)
    for b in range(frames // N0):
        m.run(buf, x[b * N0:(b + 1) * N0], N0)
        out[b * N0:(b + 1) * N0] = buf.reshape(N0, -1)
    return out


LAYOUTS = [
    ([16], [0], 700),                      # single level, ragged IR
    ([64, 256, 1024], [6, 6, 0], 9000),    # strict-valid
    ([64, 256, 1024], [4, 3, 0], 5000),    # relaxed slack 0
    ([128, 2048], [16, 15], 32768),        # config 3 layout
    ([512, 4096], [8, 15], 65536),         # config 4 layout
    ([32, 64, 128, 256], [2, 1, 1, 0], 1500),
    ([1024, 8192], [8, 3], 30000),         # class-2 FFT size
    # layouts with slack: larger levels' fires are deferred off the step chain
    ([64, 512, 4096], [14, 14, 0], 40000),        # strict ratio 8: windows 6 and 62 steps
    ([128, 1024], [40, 0], 12000),                # slack 32 steps, window capped at T - 2 = 6
    ([64, 512], [9, 0], 6000),                    # window of one step
    ([256, 2048, 16384], [14, 14, 0], 131072),    # config-1 IR length, strict chain
    # many parts: spread tasks split into several partial-sum rows
    ([64, 512], [40, 0], 12000),                  # level 0: 38 parts beyond the first two (3 rows)
    ([64, 512], [8, 0], 64 * 8 + 512 * 40),       # in-step level 1 with 40 parts (3 rows)
    ([32], [0], 3200),                            # one level, 100 parts (7 rows)
    ([2048, 16384], [8, 0], 60000),               # base block in the 4096 class (no prefetch path)
]
DEFERRED = LAYOUTS[7:]


@pytest.mark.parametrize("N,P,L", LAYOUTS)
def test_single_pc_run_matches_oracle(gpu, N, P, L):
    rng = np.random.default_rng(L)
    h = _ir(rng, L)
    N0 = N[0]
    frames = N0 * ((L + 4 * N[-1]) // N0 + 8)
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    x[frames - L - N0:] = 0.0
    m = PartConvMulti()
    m.setup_layout(48000, N0, 1, 1, [dict(ir=h, N=N, P=P)])
    y = _run_callbacks(m, x, N0)
    ref = oracle.OracleMulti(N0, 1, 1, [dict(ir=h, N=N, P=P)]).run(x)
    ref64 = wl.conv_fp64(x[:, 0], h, frames)
    assert wl.rel_l2(y[:, 0], ref[:, 0]) <= TOL
    assert wl.rel_l2(y[:, 0], ref64) <= TOL
    assert m.kernel_launches() > 0


@pytest.mark.parametrize("N,P,L", LAYOUTS[1:4] + DEFERRED)
def test_process_graph_path_equals_callbacks(gpu, N, P, L):
    """pc_process (graph replays) gives bit-identical results to pc_run."""
    rng = np.random.default_rng(L + 1)
    h = _ir(rng, L)
    N0 = N[0]
    frames = N0 * 300
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    a = PartConvMulti()
    a.setup_layout(48000, N0, 1, 1, [dict(ir=h, N=N, P=P)])
    ya = _run_callbacks(a, x, N0)
    b = PartConvMulti()
    b.setup_layout(48000, N0, 1, 1, [dict(ir=h, N=N, P=P)])
    yb = np.concatenate([b.process(x[:frames // 3 // N0 * N0]), b.process(x[frames // 3 // N0 * N0:])])
    assert np.array_equal(ya, yb)


@pytest.mark.parametrize("N,P,L", [([64], [0], 40), ([64], [0], 100), ([64], [0], 180), ([64], [0], 250),
                                   ([64, 128], [2, 0], 1500), ([64, 128], [3, 0], 1500), ([128, 256], [4, 0], 3000),
                                   ([512, 1024], [3, 0], 5000)])
def test_few_level0_parts(gpu, N, P, L):
    """Level 0 with one to four parts, alone and under a larger level (the
    one-block fire sums parts 0..2 itself, spread tasks the rest): long calls
    and one call per block match the oracle and each other bit for bit.  A
    long call transforms the two blocks before each block from its own
    input, a one-block call reads them from the input ring."""
    rng = np.random.default_rng(L + 7)
    h = _ir(rng, L)
    N0 = N[0]
    frames = N0 * 60
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    ref = oracle.OracleMulti(N0, 1, 1, [dict(ir=h, N=N, P=P)]).run(x)
    m = PartConvMulti()
    m.setup_layout(48000, N0, 1, 1, [dict(ir=h, N=N, P=P)])
    y = np.concatenate([m.process(x[: 7 * N0]), m.process(x[7 * N0: 8 * N0]), m.process(x[8 * N0:])])
    assert wl.rel_l2(y[:, 0], ref[:, 0]) <= TOL
    m.reset()
    assert np.array_equal(_run_callbacks(m, x, N0), y)


def test_planar_equals_interleaved_and_mixing(gpu):
    rng = np.random.default_rng(21)
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
    m = PartConvMulti()
    m.setup_layout(48000, N0, 3, 4, pcs)
    yi = m.process(x, PC_INTERLEAVED)
    m.reset()
    yp = m.process(np.ascontiguousarray(x.T), PC_PLANAR)
    assert np.array_equal(yi, yp.T)
    for o in (1, 2):
        assert wl.rel_l2(yi[:, o], ref[:, o]) <= TOL
    assert np.all(yi[:, 0] == 0) and np.all(yi[:, 3] == 0)
    m.reset()
    yc = _run_callbacks(m, x, N0)
    assert np.array_equal(yc, yi)


def test_relaxed_variant_matches_oracle(gpu):
    rng = np.random.default_rng(22)
    N, P, L = [128, 512, 2048], [4, 3, 0], 7000
    h = _ir(rng, L)
    frames = 128 * 200
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    ref = oracle.OracleMulti(128, 1, 1, [dict(ir=h, N=N, P=P)], relaxed=True).run(x)
    m = PartConvMultiRelaxed()
    m.setup_layout(48000, 128, 1, 1, [dict(ir=h, N=N, P=P)])
    y1 = _run_callbacks(m, x, 128)
    assert np.all(y1[:128] == 0)
    assert wl.rel_l2(y1[:, 0], ref[:, 0]) <= TOL
    m.reset()
    y2 = np.concatenate([m.process(x[: 128 * 70]), m.process(x[128 * 70:])])
    assert np.array_equal(y1, y2)


def test_reset_reproduces(gpu):
    rng = np.random.default_rng(23)
    h = _ir(rng, 5000)
    x = (0.1 * rng.standard_normal((64 * 150, 1))).astype(np.float32)
    m = PartConvMulti()
    m.setup_layout(48000, 64, 1, 1, [dict(ir=h, N=[64, 256, 1024], P=[4, 3, 0])])
    a = m.process(x)
    m.reset()
    b = m.process(x)
    assert np.array_equal(a, b)


def test_errors_do_not_exit(gpu):
    m = PartConvMulti()
    m.setup_layout(48000, 64, 1, 1, [dict(ir=np.ones(300, np.float32), N=[64, 128], P=[2, 0])])
    buf = np.zeros(64, np.float32)
    with pytest.raises(PartConvError) as ei:
        m.run(buf, np.zeros(32, np.float32), 32)
    assert ei.value.code == nat.PC_ERR_ARG and "frameCount" in str(ei.value)
    with pytest.raises(PartConvError):
        m.setup_layout(48000, 64, 1, 1, [dict(ir=np.ones(300, np.float32), N=[64], P=[0])])
    m.cleanup()
    m.setup_layout(48000, 64, 1, 1, [dict(ir=np.ones(300, np.float32), N=[64], P=[0])])
    with pytest.raises(PartConvError) as ei:
        PartConvMulti().setup_layout(48000, 64, 1, 1, [dict(ir=np.ones(300, np.float32), N=[64, 1024], P=[2, 0])])
    assert ei.value.code == nat.PC_ERR_LAYOUT


def test_config1_full_size(gpu):
    """Config 1 at full size: 2^20 samples + IR flush, vs oracle and FP64."""
    c = wl.cfg1()
    N0 = c["N0"]
    x = np.concatenate([c["x"], np.zeros(len(c["h"]), np.float32)])[:, None]
    m = PartConvMulti()
    m.setup_layout(48000, N0, 1, 1, [dict(ir=c["h"], N=c["N"], P=c["P"])])
    y = m.process(x)[:, 0]
    ref = oracle.OracleMulti(N0, 1, 1, [dict(ir=c["h"], N=c["N"], P=c["P"])]).run(x)[:, 0]
    ref64 = wl.conv_fp64(c["x"], c["h"])
    n = len(ref64)
    e_or = wl.rel_l2(y[:n], ref[:n])
    e_64 = wl.rel_l2(y[:n], ref64)
    assert e_or <= TOL, e_or
    assert e_64 <= TOL, e_64
    # sampled FP64 direct convolution (independent of any FFT)
    idx = np.random.default_rng(0).integers(0, n, 256)
    d = oracle.conv_direct_f64(c["x"], c["h"], idx)
    assert np.abs(y[idx] - d).max() <= 1e-4 * np.abs(ref64).max()


def test_config2_batched_full_size(gpu):
    """32 streams of config 2 in one handle vs the oracle, per stream."""
    c = wl.cfg2()
    S = len(c["irs"])
    N0 = c["N0"]
    tail = max(len(h) for h in c["irs"])
    frames = c["x"].shape[1] + (tail + N0 - 1) // N0 * N0
    x = np.zeros((S, frames), np.float32)
    x[:, : c["x"].shape[1]] = c["x"]
    pcs = [dict(ir=h, N=N, P=P, in_ch=s, out_ch=s) for s, (h, (N, P)) in enumerate(zip(c["irs"], c["layouts"]))]
    m = PartConvMulti()
    m.setup_layout(48000, N0, S, S, pcs)
    y = m.process(x, PC_PLANAR)
    ref, _ = oracle.run_streams(c["layouts"], c["irs"], x, N0)
    for s in range(S):
        assert wl.rel_l2(y[s], ref[s]) <= TOL, s


def test_deferred_and_in_step_levels_mixed(gpu):
    """One handle with PCs whose larger levels fire within their step (slack
    0) and PCs whose larger levels are deferred, summed into shared outputs."""
    rng = np.random.default_rng(77)
    N0 = 128
    specs = [dict(N=[128, 1024], P=[8, 0], L=9000, in_ch=0, out_ch=0),
             dict(N=[128, 1024, 8192], P=[14, 14, 0], L=40000, in_ch=1, out_ch=0),
             dict(N=[128, 512, 2048], P=[6, 6, 0], L=7000, in_ch=0, out_ch=1),
             dict(N=[128, 1024], P=[20, 0], L=12000, in_ch=1, out_ch=1, scale=0.5)]
    pcs = [dict(ir=_ir(rng, s_["L"]), N=s_["N"], P=s_["P"], in_ch=s_["in_ch"], out_ch=s_["out_ch"],
                scale=s_.get("scale", 1.0)) for s_ in specs]
    frames = N0 * 700
    x = (0.1 * rng.standard_normal((frames, 2))).astype(np.float32)
    m = PartConvMulti()
    m.setup_layout(48000, N0, 2, 2, pcs)
    y = m.process(x)
    ref = oracle.OracleMulti(N0, 2, 2, pcs).run(x)
    for o in range(2):
        assert wl.rel_l2(y[:, o], ref[:, o]) <= TOL
    m.reset()
    yc = _run_callbacks(m, x, N0)
    assert np.array_equal(y, yc)


def test_rt_driver_matches_callbacks_and_reports(gpu):
    """Headless real-time driver: same samples as pc_run callbacks, one
    callback per 256-sample period at 48 kHz, latency and misses reported."""
    from partconv_gb300.rtdriver import RealtimeDriver

    rng = np.random.default_rng(5)
    N, P, L = [256, 2048, 16384], [14, 14, 0], 60000
    h = _ir(rng, L)
    frames = 256 * 120
    x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
    m = PartConvMulti()
    m.setup_layout(48000, 256, 1, 1, [dict(ir=h, N=N, P=P)])
    y_cb = _run_callbacks(m, x, 256)
    m.reset()
    y, st = RealtimeDriver(m).run(x, realtime=True)
    assert np.array_equal(y, y_cb)
    assert st["callbacks"] == 120 and abs(st["period_us"] - 1e6 * 256 / 48000) < 1e-6
    assert 0 < st["latency_p50_us"] <= st["latency_p99_us"] <= st["latency_max_us"]
    assert st["wall_s"] >= 120 * 256 / 48000 * 0.99
    print("rt driver:", {k: round(v, 2) for k, v in st.items()})
    m.reset()
    y2, st2 = RealtimeDriver(m).run(x, realtime=False)
    assert np.array_equal(y2, y_cb) and st2["misses"] == 0


@pytest.mark.parametrize("layout", [PC_INTERLEAVED, PC_PLANAR])
def test_long_process_pipeline_equals_device_path(gpu, layout):
    """A long pc_process call runs as chunks whose copies overlap the steps;
    the result equals the unchunked device path bit for bit, for two inputs
    mixed into three outputs."""
    import torch

    rng = np.random.default_rng(41)
    N0 = 64
    pcs = [dict(ir=_ir(rng, 9000), N=[64, 512, 4096], P=[14, 14, 0], in_ch=0, out_ch=0),
           dict(ir=_ir(rng, 3000), N=[64, 256], P=[6, 0], in_ch=1, out_ch=0, scale=0.5),
           dict(ir=_ir(rng, 5000), N=[64, 512], P=[10, 0], in_ch=1, out_ch=2)]
    frames = N0 * 1500   # chunks of 128 blocks (the last one shorter)
    x = (0.1 * rng.standard_normal((frames, 2))).astype(np.float32)
    xin = x if layout == PC_INTERLEAVED else np.ascontiguousarray(x.T)
    a = PartConvMulti()
    a.setup_layout(48000, N0, 2, 3, pcs)
    ya = a.process(xin, layout)
    b = PartConvMulti()
    b.setup_layout(48000, N0, 2, 3, pcs)
    xd = torch.from_numpy(xin).cuda()
    yd = torch.empty(ya.shape, dtype=torch.float32, device="cuda")
    b.process_device(yd, xd, frames, layout)
    torch.cuda.synchronize()
    assert np.array_equal(ya, yd.cpu().numpy())
    yt = ya if layout == PC_INTERLEAVED else ya.T
    ref = oracle.OracleMulti(N0, 2, 3, pcs).run(x)
    for o in (0, 2):
        assert wl.rel_l2(yt[:, o], ref[:, o]) <= TOL
    assert np.all(yt[:, 1] == 0)
