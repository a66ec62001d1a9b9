"""Committed golden fixtures (tests/golden/golden.npz, made by
tests/golden/make_golden.py from seeded inputs).

CPU: the oracle still reproduces the fixtures, the fixtures agree with an
FP64 FFT convolution (the independent truth that pins the oracle), and the
Relaxed variant is the strict output one block later.
GPU: the CUDA path through the C ABI reproduces the fixtures, strict and
Relaxed, block by block (pc_run) and in one pc_process call."""
import numpy as np
import pytest

from golden.make_golden import load

TOL_GPU = 1e-5      # relative L2 per output channel, GPU vs oracle fixture
TOL_F64 = 1e-6      # relative L2 per output channel, fixture vs FP64
CASES = load()


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _fp64(case):
    """sum over unmuted PCs of scale * (x_in * h) in float64, per output."""
    frames = case["frames"]
    y = np.zeros((frames, case["n_out"]))
    for p in case["pcs"]:
        if p["mute"]:
            continue
        x = case["x"][:, p["in_ch"]].astype(np.float64)
        h = p["ir"].astype(np.float64)
        n = 1 << int(np.ceil(np.log2(frames + len(h))))
        full = np.fft.irfft(np.fft.rfft(x, n) * np.fft.rfft(h, n), n)[:frames]
        y[:, p["out_ch"]] += p["scale"] * full
    return y


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_fixture(name):
    import oracle

    c = CASES[name]
    y = oracle.OracleMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"]).run(c["x"])
    yr = oracle.OracleMulti(c["bs"], c["n_in"], c["n_out"], c["pcs"], relaxed=True).run(c["x"])
    for o in range(c["n_out"]):
        assert _rel(y[:, o], c["y"][:, o]) <= 1e-7 or not np.any(c["y"][:, o])
        assert _rel(yr[:, o], c["y_relaxed"][:, o]) <= 1e-7 or not np.any(c["y_relaxed"][:, o])


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_matches_fp64(name):
    c = CASES[name]
    ref = _fp64(c)
    for o in range(c["n_out"]):
        if not np.any(ref[:, o]):
            assert not np.any(c["y"][:, o])
            continue
        assert _rel(c["y"][:, o], ref[:, o]) <= TOL_F64, (name, o)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_relaxed_is_one_block_later(name):
    c = CASES[name]
    bs = c["bs"]
    assert np.all(c["y_relaxed"][:bs] == 0)
    assert np.array_equal(c["y_relaxed"][bs:], c["y"][:-bs])


@pytest.mark.gpu
@pytest.mark.parametrize("relaxed", [False, True])
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_fixture(gpu, name, relaxed):
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
        assert _rel(yp[:, o], want[:, o]) <= TOL_GPU, (name, relaxed, o)
