"""The oracle pinned to the reference's own code.

oracle/_ref/libpcref.so is the reference's PartConvFilter compiled from its
own src/partconv.cpp and src/buffers.cpp (FFTW stood in for by the oracle's
float32 transform, oracle/fftw_shim/), driven through PartConvMulti::run's
callback sequence.  With the transform shared, the oracle's strict
restatement must equal it bit for bit; the minimum-latency schedule the GPU
engine follows must agree to float32 rounding.

tests/golden/ref_golden.npz holds outputs the reference's code produced
(tests/golden/make_ref_golden.py), for hosts where it cannot be built.
CPU only."""
import numpy as np
import pytest

import oracle
from golden import make_ref_golden as mrg
from oracle import ref
from partconv_gb300 import workloads as wl

CASES = mrg.load()
needs_ref = pytest.mark.skipif(not ref.available(), reason="reference sources not present (x86_64 host with the "
                                                            "reference checkout needed)")


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_fixture(name):
    """The oracle's strict restatement gives the reference's outputs: the
    same bits where both run the same transform (x86_64 here); within 1e-7
    elsewhere.  Its Relaxed variant gives them one block later."""
    c = CASES[name]
    y = oracle.OracleMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"], schedule=1).run(c["x"])
    yr = oracle.OracleMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"], relaxed=True, schedule=1).run(c["x"])
    for o in range(c["n_out"]):
        if not np.any(c["y"][:, o]):
            assert not np.any(y[:, o])
            continue
        assert _rel(y[:, o], c["y"][:, o]) <= 1e-7, (name, o)
        assert _rel(yr[:, o], c["y_relaxed"][:, o]) <= 1e-7, (name, o)
    if ref.available():
        assert np.array_equal(y, c["y"]) and np.array_equal(yr, c["y_relaxed"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_fixture_matches_fp64_and_min_latency_schedule(name):
    """The reference's outputs against an FP64 convolution (1e-6), and the
    minimum-latency schedule that the GPU engine runs against them (1e-6)."""
    c = CASES[name]
    y2 = oracle.OracleMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"], schedule=2).run(c["x"])
    for o in range(c["n_out"]):
        ref64 = np.zeros(c["frames"])
        for p in c["pcs"]:
            if p["out_ch"] == o and not p["mute"]:
                ref64 += p["scale"] * wl.conv_fp64(c["x"][:, p["in_ch"]], p["ir"], c["frames"])
        if not np.any(ref64):
            continue
        assert _rel(c["y"][:, o], ref64) <= 1e-6, (name, o)
        assert _rel(y2[:, o], c["y"][:, o]) <= 1e-6, (name, o)


@needs_ref
@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_fixture_is_current(name):
    """Re-running the reference's code on the fixture's inputs gives the
    committed outputs, and its Relaxed run is the strict run one block later,
    bit for bit."""
    c = CASES[name]
    y = ref.RefMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"]).run(c["x"])
    yr = ref.RefMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"], relaxed=True).run(c["x"])
    assert np.array_equal(y, c["y"])
    assert np.array_equal(yr, mrg.relaxed_from_strict(y, c["bs"]))


def _random_strict_layout(rng):
    """A layout the reference's setup accepts: powers of two, increasing,
    2 N0 + s_L >= 2 N_L (src/partconv.cpp:148-166)."""
    N0 = int(rng.choice([16, 32, 64, 128, 256]))
    M = int(rng.integers(1, 5))
    N, P = [N0], []
    s = 0
    for L in range(1, M):
        nb = N[-1] * int(rng.choice([2, 4, 8]))
        need = max(1, -(-(2 * nb - 2 * N0 - s) // N[-1]))
        p = need + int(rng.integers(0, 3))
        P.append(p)
        s += N[-1] * p
        N.append(nb)
    L_ir = s + int(rng.integers(1, 3 * N[-1]))
    P.append(1)
    return N, P, L_ir


@needs_ref
def test_oracle_equals_reference_on_random_strict_layouts():
    """40 seeded random strict layouts (1 to 4 levels, block ratios 2/4/8,
    base blocks 16..256), random input scale: oracle == reference bit for bit
    (strict and Relaxed), minimum-latency schedule within 1e-6."""
    rng = np.random.default_rng(2024)
    for trial in range(40):
        N, P, L = _random_strict_layout(rng)
        st, Pr = ref.layout_check(N, P, L)
        assert st == 0, (N, P, L)
        h = wl.decaying_ir(rng, L, float(rng.uniform(0.05, 0.5)))
        pcs = [dict(ir=h, N=N, P=list(Pr), scale=float(rng.uniform(0.5, 2.0)))]
        frames = N[0] * (-(-L // N[0]) + int(rng.integers(4, 40)))
        x = (0.1 * rng.standard_normal((frames, 1))).astype(np.float32)
        yr_ = ref.RefMulti(N[0], 1, 1, pcs).run(x)
        yo = oracle.OracleMulti(N[0], 1, 1, pcs, schedule=1).run(x)
        assert np.array_equal(yr_, yo), (trial, N, list(Pr), L)
        yrr = ref.RefMulti(N[0], 1, 1, pcs, relaxed=True).run(x)
        yor = oracle.OracleMulti(N[0], 1, 1, pcs, relaxed=True, schedule=1).run(x)
        assert np.array_equal(yrr, yor), (trial, N, list(Pr), L)
        ym = oracle.OracleMulti(N[0], 1, 1, pcs, schedule=2).run(x)
        assert _rel(ym, yr_) <= 1e-6, (trial, N, list(Pr), L)


@needs_ref
def test_layout_check_agrees_with_reference():
    """The oracle's strict check accepts and rejects what PartConvFilter::setup
    does, with the same last-level part count.  One documented difference:
    when the earlier levels cover the IR exactly (remainder 0) the reference
    accepts with P[M-1] = 0 (its runLevel would then divide by zero), the
    oracle and the engine refuse."""
    rng = np.random.default_rng(5)
    seen_reject = seen_zero = 0
    for trial in range(300):
        N0 = int(rng.choice([16, 64, 256]))
        M = int(rng.integers(1, 4))
        N = [N0 << int(e) for e in np.concatenate([[0], np.cumsum(rng.integers(1, 4, M - 1))])]
        P = [int(v) for v in rng.integers(1, 16, len(N))]
        s = sum(n * p for n, p in zip(N[:-1], P[:-1]))
        L = int(max(1, s + rng.integers(-N[-1], 3 * N[-1])))
        if trial % 25 == 0:
            L = s   # remainder 0
        st_r, P_r = ref.layout_check(N, P, L)
        st_o, P_o, _, _ = oracle.layout_check(N, P, L, relaxed=False)
        if st_r == 0 and L - s == 0:
            assert st_o != 0 and P_r[-1] == 0
            seen_zero += 1
            continue
        assert (st_r == 0) == (st_o == 0), (N, P, L)
        if st_r == 0:
            assert P_r[-1] == P_o[-1], (N, P, L)
        else:
            seen_reject += 1
    assert seen_reject > 20 and seen_zero > 0


@needs_ref
def test_large_block_layout_of_the_reference_config():
    """The layout of the reference's src/pc.config:2, 64x6 | 256x6 | 1024x6 |
    4096x6 | 16384x6 | 65536x9 (a 131072-point top transform), with a seeded
    decaying IR of 300000 taps: oracle == reference bit for bit."""
    rng = np.random.default_rng(31)
    N = [64, 256, 1024, 4096, 16384, 65536]
    h = wl.decaying_ir(rng, 300000, 2.0)
    st, P = ref.layout_check(N, [6, 6, 6, 6, 6, 9], len(h))
    assert st == 0 and P[-1] == 3
    pcs = [dict(ir=h, N=N, P=list(P))]
    frames = 64 * (-(-len(h) // 64) + 64)
    x = np.zeros((frames, 1), np.float32)
    x[:8192, 0] = 0.1 * rng.standard_normal(8192)
    yr_ = ref.RefMulti(64, 1, 1, pcs).run(x)
    yo = oracle.OracleMulti(64, 1, 1, pcs, schedule=1).run(x)
    assert np.array_equal(yr_, yo)
    assert _rel(yr_[:, 0], wl.conv_fp64(x[:, 0], h, frames)) <= 1e-6


@needs_ref
def test_reference_reset_clears_only_part_of_its_delay_buffers():
    """A documented difference: DelayBuffer::reset (src/partconv.cpp:1459-1465)
    clears bufferSize floats of the bufferSize * frameSize it holds, so after
    PartConvMulti::reset the reference replays stale input for a while.  The
    oracle and the engine clear all state: a run after reset repeats the
    first run exactly."""
    rng = np.random.default_rng(8)
    N, L = [64, 256, 1024], 9000
    h = wl.decaying_ir(rng, L, 0.3)
    st, P = ref.layout_check(N, [6, 6, 1], L)
    pcs = [dict(ir=h, N=N, P=list(P))]
    x = (0.1 * rng.standard_normal((64 * 400, 1))).astype(np.float32)
    r = ref.RefMulti(64, 1, 1, pcs)
    y1 = r.run(x)
    r.reset()
    y2 = r.run(x)
    assert not np.array_equal(y1, y2)
    o = oracle.OracleMulti(64, 1, 1, pcs, schedule=1)
    z1 = o.run(x)
    o.reset()
    z2 = o.run(x)
    assert np.array_equal(z1, z2) and np.array_equal(z1, y1)


@pytest.mark.gpu
@pytest.mark.parametrize("relaxed", [False, True])
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_outputs(gpu, name, relaxed):
    """The CUDA path through the C ABI against the outputs of the reference's
    own code (tests/golden/ref_golden.npz): PartConvMulti and
    PartConvMultiRelaxed, block by block (pc_run) and in one pc_process call
    (same bits), relative L2 <= 1e-5 per output channel."""
    from partconv_gb300.multi import PartConvMulti, PartConvMultiRelaxed

    c = CASES[name]
    want = c["y_relaxed"] if relaxed else c["y"]
    m = PartConvMultiRelaxed() if relaxed else PartConvMulti()
    m.setup_layout(48000, c["bs"], c["n_in"], c["n_out"], c["pcs"])
    bs = c["bs"]
    yb = np.zeros((c["frames"], c["n_out"]), np.float32)
    out = np.zeros(bs * c["n_out"], np.float32)
    for b in range(c["frames"] // bs):
        m.run(out, np.ascontiguousarray(c["x"][b * bs:(b + 1) * bs]), bs)
        yb[b * bs:(b + 1) * bs] = out.reshape(bs, c["n_out"])
    m.reset()
    yp = m.process(c["x"])
    m.cleanup()
    assert np.array_equal(yb, yp)
    for o in range(c["n_out"]):
        if not np.any(want[:, o]):
            assert not np.any(yp[:, o])
            continue
        err = _rel(yp[:, o], want[:, o])
        print(f"{name} relaxed={relaxed} out {o}: rel L2 vs reference {err:.2e}")
        assert err <= 1e-5, (name, relaxed, o)
