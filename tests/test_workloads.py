"""The seeded synthetic workloads behind every benchmark configuration:
shapes, value ranges and determinism (the same seed gives the same arrays),
and the layouts they name are valid.  CPU only."""
import numpy as np
import pytest

from partconv_gb300 import workloads as wl
from partconv_gb300.multi import check_layout
from partconv_gb300.serving import serving_layout


def test_decaying_ir_is_unit_norm_and_decays():
    h = wl.decaying_ir(np.random.default_rng(0), 48000, 0.5)
    assert h.dtype == np.float32 and h.shape == (48000,)
    assert abs(float(np.linalg.norm(h.astype(np.float64))) - 1.0) < 1e-5
    # 60 dB over T60: the second half-second is far quieter than the first
    e1 = float(np.sum(h[:24000].astype(np.float64) ** 2))
    e2 = float(np.sum(h[24000:].astype(np.float64) ** 2))
    assert e2 < 1e-3 * e1


def test_cfg1_shapes_layout_and_determinism():
    a, b = wl.cfg1(), wl.cfg1()
    assert a["x"].shape == (1 << 20,) and a["h"].shape == (1 << 17,)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["h"], b["h"])
    assert (a["N"], a["P"], a["N0"]) == ([256, 2048, 16384], [8, 7, 7], 256)
    assert abs(float(np.std(a["x"])) - 0.1) < 1e-3
    assert check_layout(a["N"], a["P"], len(a["h"]))[0] == 0


def test_cfg2_draws_and_layouts():
    c = wl.cfg2(n_samples=4096)
    assert c["x"].shape == (32, 4096) and len(c["irs"]) == 32
    lens = np.array([len(h) for h in c["irs"]])
    assert lens.min() >= 1 << 14 and lens.max() <= 1 << 19
    assert np.all((c["t60"] >= 0.3) & (c["t60"] <= 4.0))
    for h, (N, P) in zip(c["irs"], c["layouts"]):
        assert N[0] == 256
        assert check_layout(N, P, len(h))[0] == 0
    d = wl.cfg2(n_samples=4096)
    assert np.array_equal(c["x"], d["x"]) and all(np.array_equal(p, q) for p, q in zip(c["irs"], d["irs"]))


def test_cfg3_and_cfg4_shapes():
    c3 = wl.cfg3(n_in=2, n_out=3, n_samples=1024, ir_len=4096)
    assert c3["irs"].shape == (2, 3, 4096) and c3["x"].shape == (2, 1024)
    # every path is a unit-norm IR scaled by 1 / n_in
    norms = np.linalg.norm(c3["irs"].astype(np.float64), axis=2)
    assert np.allclose(norms, 0.5, rtol=1e-5)
    c4 = wl.cfg4(batch=2, n_samples=2048, ir_len=8192)
    assert c4["x"].shape == (2, 2048) and c4["h_target"].shape == (8192,) and c4["h_init"].shape == (8192,)
    assert (c4["N"], c4["P"], c4["N0"]) == ([512, 4096], [8, 15], 512)


def test_cfg5_request_mix():
    reqs = wl.cfg5_requests(n_streams=400)
    assert reqs == wl.cfg5_requests(n_streams=400)
    arr = np.array([r["arrival"] for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert 170.0 < len(reqs) / arr[-1] < 230.0   # Poisson arrivals at about 200/s
    assert {r["channels"] for r in reqs} <= {1, 2, 8}
    assert {r["N0"] for r in reqs} <= {64, 128, 256, 1024}
    for r in reqs:
        assert (1 << 12) <= r["ir_len"] <= (1 << 20)
        assert 0.2 <= r["t60"] <= 5.0
        assert r["frames"] % r["N0"] == 0 and r["frames"] >= 10 * wl.FS
    irs, x = wl.make_request(reqs[0])
    assert len(irs) == reqs[0]["channels"] and x.shape == (reqs[0]["channels"], reqs[0]["frames"])


def test_serving_layouts_are_valid():
    for L in (100, 4096, 5000, 1 << 16, 1 << 20):
        for n0 in (64, 128, 256, 1024):
            N, P = serving_layout(L, n0)
            assert N[0] == n0 and len(N) <= 5 and N[-1] <= 16384
            assert check_layout(N, P, L)[0] == 0, (L, n0, N, P)


def test_fd_grads_fp64_match_analytic_gradients():
    """The FP64 central differences that check the adjoint equal the exact
    gradients of the quadratic loss: dL/dh_j = 2/M sum r_b[n] x_b[n-j] and
    dL/dx_(b,i) = 2/M sum_n r_b[n] h[n-i]."""
    rng = np.random.default_rng(3)
    B, T, L = 2, 300, 50
    x = (0.1 * rng.standard_normal((B, T))).astype(np.float32)
    h = (0.01 * rng.standard_normal(L)).astype(np.float32)
    t = rng.standard_normal((B, T)) * 0.1
    r = np.stack([np.convolve(x[b].astype(np.float64), h.astype(np.float64))[:T] for b in range(B)]) - t
    M = r.size
    ch = [0, 7, 49]
    cx = [(0, 0), (1, 120), (1, 299)]
    gh, gx = wl.fd_grads_fp64(x, h, t, ch, cx, 1e-3)
    ref_h = [2 / M * sum(np.dot(r[b, j:], x[b, : T - j].astype(np.float64)) for b in range(B)) for j in ch]
    ref_x = [2 / M * np.dot(r[b, i:i + L][: T - i], h[: T - i].astype(np.float64)) for b, i in cx]
    assert np.allclose(gh, ref_h, rtol=1e-9, atol=0)
    assert np.allclose(gx, ref_x, rtol=1e-9, atol=0)


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("ratio", [4, 8])
def test_chain_layout_is_valid_and_minimal(strict, ratio):
    """chain_layout: block sizes grow by `ratio`, every level but the last
    holds just enough parts for the next level's offset (minimum slack, or
    the reference's strict slack), the last covers the IR, and the layout
    passes the matching check."""
    from partconv_gb300.multi import check_layout

    for L in (5000, 70000, 300000):
        N, P = wl.chain_layout(L, 256, ratio=ratio, max_block=65536, strict=strict)
        assert N[0] == 256 and all(b == a * ratio or b == 65536 for a, b in zip(N, N[1:]))
        s = 0
        for i in range(len(N) - 1):
            s += N[i] * P[i]
            need = 2 * N[i + 1] - 2 * 256 if strict else N[i + 1]
            assert s >= need and s - N[i] < need, (L, N, P)   # just enough parts
        assert sum(n * p for n, p in zip(N, P)) >= L
        st, _, _, msg = check_layout(N, P, L, relaxed=not strict)
        assert st == 0, msg


def test_algorithmic_bytes_per_sample():
    """sum_L (8 (N_L + 1)(2 P_L + 1) + 12 N_L) / N_L: H and X ring read, new X
    slot written, 2N window read, N outputs written per level block."""
    N, P = [256, 2048], [14, 15]
    want = (8 * 257 * 29 + 12 * 256) / 256 + (8 * 2049 * 31 + 12 * 2048) / 2048
    assert wl.algorithmic_bytes_per_sample(N, P) == pytest.approx(want, rel=1e-12)
