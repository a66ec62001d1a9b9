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
