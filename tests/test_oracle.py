"""The CPU oracle against independent truths (FP64 convolution, numpy FFT)
and the reference's layout rules.  No GPU needed."""
import numpy as np
import pytest

import oracle
from partconv_gb300.workloads import conv_fp64, rel_l2


def _case(rng, ir_len, N0, blocks, extra=3):
    h = (rng.standard_normal(ir_len) * np.exp(-np.arange(ir_len) / (ir_len / 4 + 1))).astype(np.float32)
    nx = blocks * N0
    x = (0.1 * rng.standard_normal(nx)).astype(np.float32)
    return x, h


@pytest.mark.parametrize("n", [2, 4, 8, 32, 256, 2048, 32768])
def test_rfft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n).astype(np.float32)
    X = oracle.rfft(x)
    ref = np.fft.rfft(x.astype(np.float64))
    assert np.abs(X - ref).max() <= 2e-6 * np.abs(ref).max() * np.log2(n + 1)
    y = oracle.irfft(X, n) / n
    assert np.abs(y - x).max() < 2e-6 * np.log2(n + 1) * np.abs(x).max()


def test_irfft_ignores_imag_of_dc_and_nyquist():
    # FFTW c2r semantics (the reference's bck plans, partconv.cpp:272-276)
    rng = np.random.default_rng(1)
    X = rng.standard_normal(33) + 1j * rng.standard_normal(33)
    a = oracle.irfft(X, 64)
    X2 = X.copy()
    X2[0] = X2[0].real
    X2[-1] = X2[-1].real
    b = oracle.irfft(X2, 64)
    assert np.array_equal(a, b)
    ref = np.fft.irfft(X2, 64) * 64
    assert np.abs(a - ref).max() < 1e-4


STRICT_LAYOUTS = [
    ([64], [0]),
    ([64, 128], [2, 0]),
    ([64, 256, 1024], [6, 6, 0]),
    ([64, 256, 1024, 4096], [6, 6, 6, 0]),
    ([128, 512, 4096], [14, 14, 0]),
]
RELAXED_LAYOUTS = [
    ([256, 2048, 16384], [8, 7, 7]),   # config 1
    ([128, 2048], [16, 15]),           # config 3
    ([512, 4096], [8, 15]),            # config 4
    ([64, 256, 1024], [4, 3, 0]),
    ([32, 64, 128, 256], [2, 1, 1, 0]),
]


@pytest.mark.parametrize("N,P", STRICT_LAYOUTS)
@pytest.mark.parametrize("schedule", [1, 2])
def test_strict_layouts_match_fp64(N, P, schedule):
    """Both the reference's DelayBuffer schedule (1) and the minimum-latency
    schedule (2) compute y = x * h with zero added latency."""
    rng = np.random.default_rng(sum(N) + schedule)
    st, Pc, _, _ = oracle.layout_check(N, P, 9000)
    assert st == 0
    x, h = _case(rng, 9000, N[0], 60 + 9000 // N[0] * 2)
    m = oracle.OracleMulti(N[0], 1, 1, [dict(ir=h, N=N, P=P)], schedule=schedule)
    y = m.run(x[:, None])[:, 0]
    ref = conv_fp64(x, h, len(x))
    assert rel_l2(y, ref) < 1e-6


@pytest.mark.parametrize("N,P", RELAXED_LAYOUTS)
def test_relaxed_layouts_match_fp64(N, P):
    rng = np.random.default_rng(N[-1] + P[0])
    ir_len = sum(n * p for n, p in zip(N[:-1], P[:-1])) + N[-1] * max(P[-1], 2) - N[-1] // 3
    st, Pc, _, _ = oracle.layout_check(N, P, ir_len, relaxed=True)
    assert st == 0
    blocks = (ir_len * 2) // N[0] + 16
    x, h = _case(rng, ir_len, N[0], blocks)
    x[-(ir_len + N[0]):] = 0.0  # flush tail so the whole response is checked
    m = oracle.OracleMulti(N[0], 1, 1, [dict(ir=h, N=N, P=P)], schedule=0)
    y = m.run(x[:, None])[:, 0]
    ref = conv_fp64(x, h, len(x))
    assert rel_l2(y, ref) < 1e-6


def test_strict_schedule_rejects_relaxed_layout():
    with pytest.raises(ValueError, match="sufficient delay"):
        oracle.OracleMulti(256, 1, 1, [dict(ir=np.ones(131072, np.float32), N=[256, 2048, 16384], P=[8, 7, 7])],
                           schedule=1)


@pytest.mark.parametrize("N,P", [STRICT_LAYOUTS[2], RELAXED_LAYOUTS[3]])
def test_relaxed_variant_is_one_block_late(N, P):
    """PartConvMultiRelaxed emits last call's result (partconvMulti.cpp:1077-1111)."""
    rng = np.random.default_rng(7)
    x, h = _case(rng, 5000, N[0], 200)
    a = oracle.OracleMulti(N[0], 1, 1, [dict(ir=h, N=N, P=P)]).run(x[:, None])[:, 0]
    b = oracle.OracleMulti(N[0], 1, 1, [dict(ir=h, N=N, P=P)], relaxed=True).run(x[:, None])[:, 0]
    assert np.all(b[: N[0]] == 0)
    np.testing.assert_allclose(b[N[0]:], a[: -N[0]], rtol=0, atol=1e-6)


def test_impulse_in_impulse_response_out():
    """Known answer: a unit impulse at t0 returns h starting exactly at t0."""
    N, P = [64, 256, 1024], [4, 3, 0]
    rng = np.random.default_rng(3)
    h = rng.standard_normal(3000).astype(np.float32)
    x = np.zeros(64 * 80, np.float32)
    t0 = 64 * 5 + 17
    x[t0] = 1.0
    y = oracle.OracleMulti(64, 1, 1, [dict(ir=h, N=N, P=P)]).run(x[:, None])[:, 0]
    np.testing.assert_allclose(y[t0:t0 + 3000], h, atol=2e-6)
    assert np.abs(y[:t0]).max() < 1e-6


def test_layout_invariance():
    rng = np.random.default_rng(4)
    x, h = _case(rng, 20000, 64, 700)
    outs = []
    for N, P in [([64], [0]), ([64, 256, 1024], [6, 6, 0]), ([64, 512, 4096], [8, 7, 0])]:
        outs.append(oracle.OracleMulti(64, 1, 1, [dict(ir=h, N=N, P=P)]).run(x[:, None])[:, 0])
    for o in outs[1:]:
        assert rel_l2(o, outs[0]) < 1e-6


def test_linearity():
    rng = np.random.default_rng(5)
    x1, h = _case(rng, 4000, 128, 100)
    x2 = (0.3 * rng.standard_normal(len(x1))).astype(np.float32)
    run = lambda x: oracle.OracleMulti(128, 1, 1, [dict(ir=h, N=[128, 1024], P=[8, 0])]).run(x[:, None])[:, 0]
    y = run(x1 + x2)
    assert rel_l2(y, run(x1) + run(x2)) < 1e-6


@pytest.mark.parametrize("N,P,msg", [
    ([64, 100], [2, 0], "power of 2"),
    ([128, 64], [2, 0], "<="),
    ([64, 1024], [2, 0], "sufficient delay"),
    ([64, 128], [2, 0], None),
])
def test_layout_errors(N, P, msg):
    st, _, _, m = oracle.layout_check(N, P, 5000, relaxed=True)
    if msg is None:
        assert st == 0
    else:
        assert st != 0 and msg in m


def test_last_level_part_count_and_delays():
    # partconv.cpp:148-181: delays (2 N0 + s_L)/N0, P_last = ceil((len - s)/N)
    st, P, d, _ = oracle.layout_check([64, 256, 1024], [6, 6, 99], 5000)
    assert st == 0
    assert list(P) == [6, 6, int(np.ceil((5000 - 64 * 6 - 256 * 6) / 1024))]
    assert list(d) == [2, 2 + 6, 2 + 6 + 24]
    st, _, _, m = oracle.layout_check([64, 256], [100, 0], 5000)
    assert st != 0 and "not required" in m


def test_multi_mixing_scaling_and_mute():
    """Deinterleave * scale, sum unmuted PCs per output in PC order
    (partconvMulti.cpp:839-847, :911-921)."""
    rng = np.random.default_rng(6)
    N0 = 64
    hs = [rng.standard_normal(700 + 300 * i).astype(np.float32) for i in range(4)]
    pcs = [
        dict(ir=hs[0], N=[64, 256], P=[4, 0], in_ch=0, out_ch=1, scale=0.5),
        dict(ir=hs[1], N=[64], P=[0], in_ch=1, out_ch=1, scale=2.0),
        dict(ir=hs[2], N=[64, 128], P=[2, 0], in_ch=1, out_ch=0, scale=1.0, mute=1),
        dict(ir=hs[3], N=[64, 256], P=[4, 0], in_ch=2, out_ch=2, scale=-1.0),
    ]
    frames = N0 * 120
    x = (0.1 * rng.standard_normal((frames, 3))).astype(np.float32)
    y = oracle.OracleMulti(N0, 3, 4, pcs).run(x)
    ref1 = conv_fp64(0.5 * x[:, 0], hs[0], frames) + conv_fp64(2.0 * x[:, 1], hs[1], frames)
    ref2 = conv_fp64(-x[:, 2], hs[3], frames)
    assert rel_l2(y[:, 1], ref1) < 1e-6
    assert rel_l2(y[:, 2], ref2) < 1e-6
    assert np.all(y[:, 0] == 0) and np.all(y[:, 3] == 0)


def test_filter_fine_grained_api_matches_multi():
    """PartConvFilter sync_levels/input/runLevel/output sequence."""
    rng = np.random.default_rng(8)
    N, P = [64, 256, 1024], [6, 6, 0]
    x, h = _case(rng, 6000, 64, 150)
    f = oracle.OracleFilter(N, P, h)
    ys = []
    for b in range(150):
        f.sync_levels()
        f.input(x[b * 64:(b + 1) * 64])
        for L in range(3):
            if b % (N[L] // 64) == 0:
                f.runLevel(L)
        ys.append(f.output())
    y = np.concatenate(ys)
    assert not f.error()
    assert rel_l2(y, conv_fp64(x, h, len(x))) < 1e-6


def test_filter_spectra_are_scaled_rfft_of_shifted_rows():
    # partconv.cpp:185-230: row p = [0_N, h_p], H = rfft(row) / 2N
    h = np.arange(1, 1 + 64 * 3, dtype=np.float32)
    f = oracle.OracleFilter([64], [0], h)
    H = f.spectra(0)
    for p in range(3):
        row = np.zeros(128)
        row[64:] = h[p * 64:(p + 1) * 64]
        np.testing.assert_allclose(H[p], np.fft.rfft(row) / 128, rtol=1e-5, atol=1e-5)


def test_direct_fp64():
    rng = np.random.default_rng(9)
    x = rng.standard_normal(500).astype(np.float32)
    h = rng.standard_normal(77).astype(np.float32)
    np.testing.assert_allclose(oracle.conv_direct_f64(x, h), np.convolve(x.astype(np.float64), h), atol=1e-9)
    idx = np.array([0, 10, 400, 575])
    np.testing.assert_allclose(oracle.conv_direct_f64(x, h, idx), np.convolve(x.astype(np.float64), h)[idx],
                               atol=1e-9)


def test_run_streams_matches_multi():
    rng = np.random.default_rng(10)
    layouts = [([64, 256], [4, 0]), ([64], [0]), ([64, 512, 4096], [8, 7, 0])]
    irs = [rng.standard_normal(L).astype(np.float32) for L in (3000, 500, 9000)]
    x = (0.1 * rng.standard_normal((3, 64 * 200))).astype(np.float32)
    y, t = oracle.run_streams(layouts, irs, x, 64, threads=2)
    assert t >= 0
    for s in range(3):
        assert rel_l2(y[s], conv_fp64(x[s], irs[s], x.shape[1])) < 1e-6


def test_leveled_workers_equal_sequential_restatement():
    """The reference-shaped CPU baseline (one worker thread per level, level
    outputs summed in level order) gives the sequential restatement's bits."""
    from partconv_gb300 import workloads as wl

    rng = np.random.default_rng(3)
    for N, P, L in [([64, 256, 1024], [4, 3, 0], 9000), ([128, 1024, 8192], [14, 14, 0], 40000), ([32], [0], 500)]:
        h = wl.decaying_ir(rng, L, 0.3)
        x = (0.1 * rng.standard_normal(N[0] * 200)).astype(np.float32)
        y1, t = oracle.run_leveled(N, P, h, x)
        yr, _ = oracle.run_streams([(N, P)], [h], x[None, :], N[0])
        assert np.array_equal(y1, yr[0]) and t > 0
