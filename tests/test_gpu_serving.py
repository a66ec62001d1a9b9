"""Serving (config 5): continuous batching over pools, HBM-budget admission,
per-block latency.  Each request's output equals the oracle's (relative L2
<= 1e-5 per channel) and equals its output when served alone."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import workloads as wl
from partconv_gb300.serving import Server, serving_layout

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _requests(n, seed, rate=400.0, seconds=0.15, lens=(10, 14), n0s=(64, 128, 256)):
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        n0 = int(rng.choice(n0s))
        out.append(dict(arrival=t, channels=int(rng.choice([1, 2], p=[0.6, 0.4])),
                        ir_len=int(round(2 ** rng.uniform(*lens))), t60=float(rng.uniform(0.1, 0.5)), N0=n0,
                        frames=int(np.ceil(seconds * 48000 / n0) * n0), seed=int(rng.integers(0, 2**62))))
    return out


def _check_against_oracle(spec, y):
    irs, x = wl.make_request(spec)
    N, P = serving_layout(spec["ir_len"], spec["N0"])
    ref, _ = oracle.run_streams([(N, P)] * len(irs), irs, x, spec["N0"])
    for ch in range(len(irs)):
        assert wl.rel_l2(y[ch], ref[ch]) <= TOL


def test_serving_layouts_are_valid():
    from partconv_gb300.multi import check_layout

    for L in (100, 4096, 5000, 2**16, 2**20):
        for n0 in (64, 128, 256, 1024):
            N, P = serving_layout(L, n0)
            assert len(N) <= 5 and N[-1] <= 16384
            st, Pc, _, msg = check_layout(N, P, L)
            assert st == 0, (L, n0, N, P, msg)


def test_mix_matches_oracle_and_solo_runs(gpu):
    reqs = _requests(14, 5)
    srv = Server(hbm_budget_bytes=1 << 30, max_pcs_per_pool=64)
    stats, outs = srv.run(reqs, realtime=False)
    assert stats["finished"] == len(reqs)
    specs = sorted(reqs, key=lambda s: s["arrival"])
    for rid, spec in enumerate(specs):
        _check_against_oracle(spec, outs[rid])
    # the same request alone gives the same samples
    for rid in (0, 5, 9):
        solo = Server(hbm_budget_bytes=1 << 28, max_pcs_per_pool=8)
        _, o2 = solo.run([dict(specs[rid], arrival=0.0)], realtime=False)
        assert np.array_equal(o2[0], outs[rid])


def test_admission_by_hbm_budget_queues(gpu):
    # each pool gets 1/4 of 24 MiB: long IRs cannot all be resident at once
    reqs = _requests(10, 7, rate=5000.0, lens=(14.5, 15), n0s=(64,))
    srv = Server(hbm_budget_bytes=24 << 20, block_sizes=(64, 128, 256, 1024), max_pcs_per_pool=64)
    stats, outs = srv.run(reqs, realtime=False)
    assert stats["finished"] == len(reqs)
    assert stats["peak_concurrent"] < len(reqs)
    specs = sorted(reqs, key=lambda s: s["arrival"])
    for rid in (0, len(reqs) - 1):
        _check_against_oracle(specs[rid], outs[rid])


def test_realtime_latency_accounting(gpu):
    reqs = _requests(8, 9, rate=200.0, seconds=0.3)
    srv = Server(hbm_budget_bytes=1 << 29, max_pcs_per_pool=32)
    stats, _ = srv.run(reqs, realtime=True, keep_outputs=False)
    assert stats["finished"] == len(reqs)
    assert stats["latency_us_p50"] > 0 and stats["latency_us_p99"] >= stats["latency_us_p50"]
    assert 0.0 <= stats["deadline_miss_rate"] <= 1.0
    print("serving latency:", {k: round(v, 1) for k, v in stats.items() if "latency" in k})


def test_async_admission_equals_blocking(gpu):
    """pcs_admit_async + pcs_poll: the PC goes live once its spectra are
    built and then produces the same samples as a blocking admission; a
    pending PC can be released and its space returns to the budget."""
    import time

    from partconv_gb300.serving import ServingPool

    rng = np.random.default_rng(11)
    N0 = 128
    ir = wl.decaying_ir(rng, 40000, 0.5)
    N, P = serving_layout(len(ir), N0)
    a = ServingPool(N0, 1 << 28, 4)
    b = ServingPool(N0, 1 << 28, 4)
    pa = a.admit(ir, N, P)
    pb = b.admit(ir, N, P, wait=False)
    for _ in range(20000):
        b.poll()
        if b.is_live(pb):
            break
        time.sleep(1e-4)
    assert a.is_live(pa) and b.is_live(pb) and pa == pb == 0
    x = (0.1 * rng.standard_normal((60, N0))).astype(np.float32)
    ya, yb = np.zeros_like(x), np.zeros_like(x)
    bi = np.zeros((1, N0), np.float32)
    bo = np.zeros((1, N0), np.float32)
    for pool, y in ((a, ya), (b, yb)):
        for t in range(len(x)):
            bi[0] = x[t]
            pool.step(bi.ctypes.data, bo.ctypes.data, 1)
            pool.sync()
            y[t] = bo[0]
    assert np.array_equal(ya, yb)
    used = b.bytes_in_use()
    pc2 = b.admit(ir, N, P, wait=False)
    assert not b.is_live(pc2) and b.bytes_in_use() > used
    b.release(pc2)
    b.poll()
    assert not b.is_live(pc2) and b.bytes_in_use() == used


def test_load_run_with_async_admission(gpu):
    """The real-time load loop admits without blocking and still serves
    every request to completion."""
    reqs = _requests(12, 13, rate=300.0, seconds=0.2)
    irs = []
    for r in reqs:
        g = np.random.Generator(np.random.PCG64(r["seed"]))
        irs.append([wl.decaying_ir(g, r["ir_len"], r["t60"]) for _ in range(r["channels"])])
    noise = (0.1 * np.random.default_rng(3).standard_normal(1 << 18)).astype(np.float32)
    srv = Server(hbm_budget_bytes=1 << 29, max_pcs_per_pool=64)
    stats = srv.run_load(reqs, irs, noise, max_concurrent=100, max_seconds=30.0)
    assert stats["finished"] == len(reqs)
    assert stats["blocks"] > 0 and stats["latency_us_p99"] >= stats["latency_us_p50"] > 0
