"""Partition-layout autotuner from measured GPU timings.

The reference picks layouts offline: src/tune.py:91-154 benches candidate
layouts through PartConvFilter.bench on the CPU, and matlab/optimal_part.m
searches a cost model (4k log2(2N) + 4 per block).  Here candidates are
timed on the GPU engine itself: each candidate layout runs a batch of
identical streams (the way the batched engine will run it) for a few
hyperperiods of base steps, and the layout with the lowest time per
stream-step wins.  Results are cached per (IR length class, base block,
batch class, GPU) in a JSON file, the analogue of the reference's FFTW
wisdom file (src/partconvMulti.cpp:250-254).
"""
from __future__ import annotations

import json
import os
import threading

import numpy as np

from . import workloads as wl

DEFAULT_CACHE = os.environ.get("PARTCONV_AUTOTUNE_CACHE") or os.path.join(
    os.path.dirname(os.path.abspath(__file__)), "autotune_cache.json")
_lock = threading.Lock()


def candidate_layouts(ir_len: int, N0: int, max_block: int = 16384):
    """Level chains with ratios 2, 4, 8 and 16 and largest blocks up to
    max_block, each with minimum slack (every level fires within its step)
    and with the reference's strict slack (larger levels' fires run beside
    later steps), plus the one-level uniform layout for short IRs."""
    seen, out = set(), []
    for strict in (False, True):
        for ratio in (2, 4, 8, 16):
            mb = N0
            while mb * ratio <= max_block:
                mb *= ratio
            tops = []
            while mb >= N0 * ratio:
                tops.append(mb)
                mb //= ratio
            for top in tops[:3]:
                N, P = wl.chain_layout(ir_len, N0, ratio=ratio, max_block=top, strict=strict)
                key = (tuple(N), tuple(P))
                if key not in seen and len(N) <= 16:
                    seen.add(key)
                    out.append((list(N), list(P)))
    if ir_len <= 64 * N0:
        N, P = [N0], [-(-ir_len // N0)]
        if (tuple(N), tuple(P)) not in seen:
            out.append((N, P))
    return out


def _gpu_name():
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "unknown"


def _len_class(ir_len: int) -> int:
    return 1 << int(np.ceil(np.log2(max(ir_len, 2))))


def measure_layout(N, P, ir_len: int, batch: int = 32, steps: int = 0, seed: int = 0, step_blocks: int = 1) -> float:
    """Device time (µs) per base step of `batch` streams of this layout
    (step_blocks: base blocks per launch, pc_set_step_blocks)."""
    import torch

    from .multi import PartConvMulti
    from . import PC_PLANAR

    rng = np.random.default_rng(seed)
    N0 = N[0]
    pcs = [dict(ir=wl.decaying_ir(rng, ir_len, 1.0), N=N, P=P, in_ch=s, out_ch=s) for s in range(batch)]
    m = PartConvMulti(step_blocks=step_blocks)
    m.setup_layout(48000, N0, batch, batch, pcs)
    H = max(m.info().hyperperiod, m.info().step_blocks)
    nsteps = steps or max(2 * H, 128)
    nsteps = (nsteps + H - 1) // H * H
    x = torch.randn(batch, nsteps * N0, device="cuda") * 0.1
    y = torch.empty_like(x)
    m.process_device(y, x, nsteps * N0, PC_PLANAR)   # warm
    torch.cuda.synchronize()
    m.reset()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    m.process_device(y, x, nsteps * N0, PC_PLANAR)
    e1.record()
    torch.cuda.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / nsteps
    m.cleanup()
    return us


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _fit(N, P, ir_len):
    """Fit a level structure chosen for a length class to the exact length."""
    N, P = list(N), list(P)
    s = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    while len(N) > 1 and s >= ir_len:
        N.pop()
        P.pop()
        s = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    P[-1] = max(1, -(-(ir_len - s) // N[-1]))
    return N, P


def _key(ir_len, N0, batch, gpu=None):
    lc = _len_class(ir_len)
    bc = 1 << int(np.ceil(np.log2(max(batch, 1))))
    return f"{gpu or _gpu_name()}|N0={N0}|len={lc}|batch={bc}", lc, bc


def cached_layout(ir_len: int, N0: int, batch: int = 32, cache: str | None = DEFAULT_CACHE):
    """The cached choice for this key without measuring (None on a miss).
    Without a GPU (or with no entry for this one) an entry of the same
    length, block and batch class measured on another GPU is taken."""
    if not cache:
        return None
    db = _load(cache)
    key, _, _ = _key(ir_len, N0, batch)
    rec = db.get(key)
    if rec is None:
        tail = key[key.index("|"):]
        rec = next((v for k, v in sorted(db.items()) if k.endswith(tail)), None)
    return _fit(rec["best"]["N"], rec["best"]["P"], ir_len) if rec else None


def choose_layout(ir_len: int, N0: int, batch: int = 32, cache: str | None = DEFAULT_CACHE, verbose: bool = False):
    """Layout (N, P) with the lowest measured time per step for IRs of this
    length class; P[-1] is recomputed for the exact ir_len."""
    key, lc, bc = _key(ir_len, N0, batch)
    with _lock:
        db = _load(cache) if cache else {}
    if key not in db:
        results = []
        for N, P in candidate_layouts(lc, N0):
            us = measure_layout(N, P, lc, batch=bc)
            results.append({"N": N, "P": P, "us_per_step": us})
            if verbose:
                print(f"  {N} {P}: {us:.2f} us/step")
        best = min(results, key=lambda r: r["us_per_step"])
        db[key] = {"best": best, "candidates": results}
        if cache:
            with _lock:
                cur = _load(cache)
                cur[key] = db[key]
                tmp = cache + ".tmp"
                with open(tmp, "w") as f:
                    json.dump(cur, f, indent=1, sort_keys=True)
                os.replace(tmp, cache)
    return _fit(db[key]["best"]["N"], db[key]["best"]["P"], ir_len)


# ---------------------------------------------------------------------------
# Dynamic program over level costs (matlab/optimal_part.m's Viterbi search,
# restated over levels instead of block positions).
# ---------------------------------------------------------------------------
def model_level_cost(N: int, P: int, N0: int, k: float = 1.5) -> float:
    """Cost per base step of a level of block N with P parts under the
    reference's model (matlab/optimal_part.m: 4 k log2(2N) + 4 per new block
    size, 4 per part), amortised over the N / N0 base steps of one block."""
    return (4.0 * k * np.log2(2 * N) + 4.0 * P) * N0 / N


def optimal_part(ir_len: int, N0: int, level_cost=None, max_block: int = 16384, strict: bool = False):
    """Layout (N, P) minimising the sum of level_cost(N, P, N0) over levels.

    Levels have power-of-two blocks growing from N0 (any factor), and each
    level L >= 1 must satisfy the delay rule for its offset s_L (relaxed:
    s_L >= N_L; strict: 2 N0 + s_L >= 2 N_L).  States are (block size,
    taps covered) in units of N0; the last level's part count covers the
    rest of the IR.  level_cost defaults to model_level_cost; pass
    measured_level_costs(...) for GPU timings."""
    cost = level_cost or model_level_cost
    U = -(-int(ir_len) // N0)                      # IR length in base blocks
    sizes = []
    n = N0
    while n <= max_block:
        sizes.append(n)
        n *= 2
    best = {}                                      # (size index, covered) -> (cost, parent, parts)

    def ok(Ni, covered):                           # delay rule for a new level of block Ni at offset covered
        s = covered * N0
        return (2 * N0 + s >= 2 * Ni) if strict else (s >= Ni)

    # level 0: P parts of N0
    for P in range(1, U + 1):
        best[(0, P)] = (cost(N0, P, N0), None, P)
    result = None
    for i in range(len(sizes)):
        for cov in sorted(c for (j, c) in list(best) if j == i):
            cst, _, _ = best[(i, cov)]
            if cov >= U:
                if result is None or cst < result[0]:
                    result = (cst, (i, cov))
                continue
            for j in range(i + 1, len(sizes)):
                Nj = sizes[j]
                if not ok(Nj, cov):
                    continue
                b = Nj // N0
                maxP = -(-(U - cov) // b)
                for P in range(1, maxP + 1):
                    key = (j, cov + P * b) if P < maxP else (j, U)
                    v = cst + cost(Nj, P, N0)
                    if key not in best or v < best[key][0]:
                        best[key] = (v, (i, cov), P)
    if result is None:
        raise ValueError("no valid layout")
    N, P = [], []
    key = result[1]
    while key is not None:
        _, parent, parts = best[key]
        N.append(sizes[key[0]])
        P.append(parts)
        key = parent
    return N[::-1], P[::-1]


def measured_level_costs(N0: int, sizes=None, parts=(2, 8), trials: int = 200):
    """level_cost(N, P, N0) from GPU timings: PartConvFilter.bench of one
    level (device time per block, CUDA events) at two part counts, fitted
    as a + b P per block and amortised over the N / N0 base steps."""
    from . import partconv

    sizes = sizes or [N0 << j for j in range(8) if (N0 << j) <= 16384]
    fit = {}
    for N in sizes:
        ts = []
        for P in parts:
            f = partconv.PartConvFilter()
            Na, Pa = partconv.intArray(1), partconv.intArray(1)
            Na[0], Pa[0] = N, P
            if f.setup(1, Na, Pa, None) != 0:
                raise RuntimeError(f.last_error)
            ts.append(f.bench(0, trials, 0, 0.1))
            f.cleanup()
        b = max((ts[1] - ts[0]) / (parts[1] - parts[0]), 1e-12)   # timing noise must not make parts free
        fit[N] = (max(ts[0] - b * parts[0], 0.0), b)

    def cost(N, P, n0=N0):
        a, b = fit[N]
        return (a + b * P) * n0 / N
    return cost
