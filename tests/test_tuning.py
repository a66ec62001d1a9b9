"""Layout search: the tune.py-compatible API (GPU-timed PartConvFilter.bench)
and the measured-GPU autotuner with its cache."""
import json

import numpy as np
import pytest

from partconv_gb300 import autotune
from partconv_gb300.multi import check_layout


def test_candidates_are_valid_layouts():
    for L in (3000, 1 << 14, 1 << 16, 1 << 19):
        for n0 in (64, 256, 1024):
            cands = autotune.candidate_layouts(L, n0)
            assert cands
            for N, P in cands:
                st, _, _, msg = check_layout(N, P, L)
                assert st == 0, (L, n0, N, P, msg)


@pytest.mark.gpu
def test_tune_py_interface(gpu):
    from partconv_gb300 import tune

    tune.init(64, 6000)
    tune.time([], 0)
    assert tune.total and tune.num_benched > 0
    ranked = tune.best(2)
    assert len(ranked) >= 1
    t, parts, loads = ranked[0]
    assert len(parts) % 2 == 0 and parts[0] == 64
    assert len(loads) == len(parts) // 2 + 1 and loads[-1] > 0


@pytest.mark.gpu
def test_autotuner_measures_and_caches(gpu, tmp_path):
    cache = str(tmp_path / "cache.json")
    N, P = autotune.choose_layout(20000, 256, batch=8, cache=cache)
    st, Pc, _, _ = check_layout(N, P, 20000)
    assert st == 0 and list(Pc) == list(P)
    db = json.load(open(cache))
    (key, rec), = db.items()
    assert "N0=256" in key and len(rec["candidates"]) >= 2
    assert rec["best"]["us_per_step"] == min(c["us_per_step"] for c in rec["candidates"])
    # a second call is served from the cache
    assert autotune.choose_layout(20000, 256, batch=8, cache=cache) == (N, P)


def _brute_chain(L, N0, strict, cost):
    sizes = [N0 << j for j in range(6)]
    U = -(-L // N0)
    best = [None]

    def rec(N, P, cov, c):
        if cov >= U:
            if best[0] is None or c < best[0][0]:
                best[0] = (c, list(N), list(P))
            return
        for Nj in sizes:
            if (N and Nj <= N[-1]) or (not N and Nj != N0):
                continue
            if N and ((2 * N0 + cov * N0 < 2 * Nj) if strict else (cov * N0 < Nj)):
                continue
            b = Nj // N0
            for p in range(1, -(-(U - cov) // b) + 1):
                rec(N + [Nj], P + [p], min(U, cov + p * b), c + cost(Nj, p, N0))

    rec([], [], 0, 0.0)
    return best[0]


@pytest.mark.parametrize("L,N0,strict", [(3000, 64, False), (5000, 64, True), (1200, 32, False), (9000, 128, False),
                                         (700, 16, True)])
def test_optimal_part_dp_matches_exhaustive_search(L, N0, strict):
    """The level DP (matlab/optimal_part.m's search, over levels) finds the
    cheapest valid chain under the reference's cost model."""
    from partconv_gb300 import autotune as at
    from partconv_gb300.multi import check_layout

    N, P = at.optimal_part(L, N0, strict=strict)
    c = sum(at.model_level_cost(n, p, N0) for n, p in zip(N, P))
    want = _brute_chain(L, N0, strict, at.model_level_cost)
    assert c == pytest.approx(want[0], rel=1e-12)
    st, _, _, msg = check_layout(N, P, L, relaxed=not strict)
    assert st == 0, msg


@pytest.mark.gpu
def test_optimal_part_on_measured_costs(gpu):
    from partconv_gb300 import autotune as at
    from partconv_gb300.multi import check_layout

    cost = at.measured_level_costs(256, sizes=[256, 512, 1024, 2048, 4096], trials=50)
    N, P = at.optimal_part(40000, 256, cost, max_block=4096)
    st, _, _, msg = check_layout(N, P, 40000)
    assert st == 0, msg
    assert all(cost(n, p) > 0 for n, p in zip(N, P))


def test_cached_layout_lookup_and_fit(tmp_path):
    """Cache entries are keyed by GPU, base block, IR length class and batch
    class; a lookup without a matching GPU takes the same-shape entry of
    another, and the chosen structure is refitted to the exact length."""
    import json

    from partconv_gb300 import autotune as at
    from partconv_gb300.multi import check_layout

    path = tmp_path / "cache.json"
    key = "Some GPU|N0=256|len=131072|batch=32"
    path.write_text(json.dumps({key: {"best": {"N": [256, 2048, 16384], "P": [14, 14, 7], "us_per_step": 3.7},
                                      "candidates": []}}))
    for L in (70000, 100000, 131072):
        N, P = at.cached_layout(L, 256, 32, cache=str(path))
        assert N == [256, 2048, 16384] and P[:2] == [14, 14]
        assert check_layout(N, P, L)[0] == 0
        assert sum(n * p for n, p in zip(N, P)) >= L
    assert at.cached_layout(5000, 256, 32, cache=str(path)) is None
    assert at.cached_layout(100000, 128, 32, cache=str(path)) is None


def test_shipped_cache_is_consistent():
    """The cache shipped with the package.  Layout entries: every key names a
    GPU, base block, length class and batch class; the best layout is the
    fastest measured candidate, every stored layout is valid for its length
    class, and the entry carries the tile shape measured for it (the fastest
    tile candidate).  Workload tile entries: the best shape is the fastest
    candidate and every candidate is a shape the engine accepts."""
    import re

    with open(autotune.DEFAULT_CACHE) as f:
        db = json.load(f)
    assert db
    n_layout = n_tiles = 0
    for key, rec in db.items():
        t = re.fullmatch(r"(.+)\|tiles\|(.+)\|N0=(\d+)\|pcs=(\d+)", key)
        if t:
            n_tiles += 1
            cands = rec["candidates"]
            assert rec["best"]["us_per_step"] == min(c["us_per_step"] for c in cands)
            for c in cands:
                b, p = c["tiles"]
                assert b in (64, 128, 256, 512) and 1 <= p <= 64 and c["us_per_step"] > 0
            continue
        m = re.fullmatch(r"(.+)\|N0=(\d+)\|len=(\d+)\|batch=(\d+)", key)
        assert m, key
        n_layout += 1
        n0, lc = int(m.group(2)), int(m.group(3))
        assert lc & (lc - 1) == 0
        best = rec["best"]
        cands = rec["candidates"]
        assert {k: best[k] for k in ("N", "P", "us_per_step")} in cands
        assert best["us_per_step"] == min(c["us_per_step"] for c in cands)
        for c in cands:
            assert c["N"][0] == n0 and c["us_per_step"] > 0
            st, _, _, msg = check_layout(c["N"], c["P"], lc)
            assert st == 0, (key, c, msg)
        tc = rec["tile_candidates"]
        assert list(best["tiles"]) == min(tc, key=lambda r: r["us_per_step"])["tiles"]
        assert {tuple(r["tiles"]) for r in tc} == set(autotune.TILE_CANDIDATES)
    assert n_layout >= 5 and n_tiles >= 1


def test_cached_tile_shapes(tmp_path):
    """Tile shapes from the cache without measuring: the one stored with a
    length class's layout, and the one measured for a whole workload handle
    (keyed by workload name, base block and PC count); misses give None."""
    from partconv_gb300 import autotune as at

    path = tmp_path / "cache.json"
    path.write_text(json.dumps({
        "Some GPU|N0=256|len=131072|batch=32": {
            "best": {"N": [256, 2048, 16384], "P": [14, 14, 7], "us_per_step": 3.2, "tiles": [128, 32]},
            "candidates": []},
        "Some GPU|tiles|cfg2|N0=256|pcs=32": {
            "best": {"tiles": [128, 16], "us_per_step": 2.9},
            "candidates": [{"tiles": [128, 16], "us_per_step": 2.9}, {"tiles": [256, 16], "us_per_step": 3.4}]},
    }))
    assert at.cached_tiles(100000, 256, 32, cache=str(path)) == (128, 32)
    assert at.cached_tiles(5000, 256, 32, cache=str(path)) is None
    pcs = [dict(N=[256], P=[1])] * 32
    assert at.choose_tiles(pcs, 256, "cfg2", cache=str(path), measure=False) == (128, 16)
    assert at.choose_tiles(pcs[:8], 256, "cfg2", cache=str(path), measure=False) is None
    assert at.choose_tiles(pcs, 128, "cfg2", cache=str(path), measure=False) is None
    assert at.choose_tiles(pcs, 256, "cfg3", cache=str(path), measure=False) is None
