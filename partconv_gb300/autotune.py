"""Partition-layout autotuner from measured GPU timings.

The reference picks layouts offline: src/tune.py:91-154 benches candidate
layouts through PartConvFilter.bench on the CPU, and matlab/optimal_part.m
searches a cost model (4k log2(2N) + 4 per block).  Here candidates are
timed on the GPU engine itself: each candidate layout runs a batch of
identical streams (the way the batched engine will run it) for a few
hyperperiods of base steps, and the layout with the lowest time per
stream-step wins.  The kernel tile shape (bins and parts per spread task,
pc_set_tiles) is then measured the same way for the winning layout, and for
a whole mixed workload by choose_tiles.  Results are cached per (IR length
class, base block, batch class, GPU) in a JSON file, the analogue of the
reference's FFTW wisdom file (src/partconvMulti.cpp:250-254).
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


MAX_BLOCK = 65536   # the engine's PC_MAX_BLOCK (blocks above 16384 run on 8-CTA clusters)

# (bins, parts) per spread task tried for a layout or a workload
TILE_CANDIDATES = [(64, 16), (128, 8), (128, 16), (128, 32), (256, 16), (256, 32), (512, 32)]
DEFAULT_TILES = (128, 16)


def candidate_layouts(ir_len: int, N0: int, max_block: int = MAX_BLOCK):
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


def measure_layout(N, P, ir_len: int, batch: int = 32, steps: int = 0, seed: int = 0, step_blocks: int = 1,
                   tiles=None) -> float:
    """Device time (µs) per base step of `batch` streams of this layout
    (step_blocks: base blocks per launch, pc_set_step_blocks; tiles: (bins,
    parts) per spread task, pc_set_tiles)."""
    rng = np.random.default_rng(seed)
    N0 = N[0]
    pcs = [dict(ir=wl.decaying_ir(rng, ir_len, 1.0), N=N, P=P, in_ch=s, out_ch=s) for s in range(batch)]
    return measure_pcs(pcs, N0, steps=steps, step_blocks=step_blocks, tiles=tiles)


def measure_pcs(pcs, N0: int, steps: int = 0, step_blocks: int = 1, tiles=None) -> float:
    """Device time (µs) per base step of one handle holding these PCs (one
    stream each), over at least two hyperperiods."""
    import torch

    from .multi import PartConvMulti
    from . import PC_PLANAR

    batch = len(pcs)
    m = PartConvMulti(step_blocks=step_blocks, tiles=tiles)
    m.setup_layout(48000, N0, batch, batch, [p | dict(in_ch=s, out_ch=s) for s, p in enumerate(pcs)])
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


def _save(cache, key, rec):
    with _lock:
        cur = _load(cache)
        cur[key] = rec
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cur, f, indent=1, sort_keys=True)
        os.replace(tmp, cache)


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
    if key not in db or "tiles" not in db[key]["best"]:
        results = []
        for N, P in candidate_layouts(lc, N0):
            us = measure_layout(N, P, lc, batch=bc)
            results.append({"N": N, "P": P, "us_per_step": us})
            if verbose:
                print(f"  {N} {P}: {us:.2f} us/step")
        best = dict(min(results, key=lambda r: r["us_per_step"]))
        # the kernel tile shape, measured on the winning layout
        tiles = []
        for tb, tp in TILE_CANDIDATES:
            us = measure_layout(best["N"], best["P"], lc, batch=bc, tiles=(tb, tp))
            tiles.append({"tiles": [tb, tp], "us_per_step": us})
            if verbose:
                print(f"  tiles {tb}x{tp}: {us:.2f} us/step")
        bt = min(tiles, key=lambda r: r["us_per_step"])
        best["tiles"] = bt["tiles"]
        best["us_per_step_tiled"] = bt["us_per_step"]
        db[key] = {"best": best, "candidates": results, "tile_candidates": tiles}
        if cache:
            _save(cache, key, db[key])
    return _fit(db[key]["best"]["N"], db[key]["best"]["P"], ir_len)


def cached_tiles(ir_len: int, N0: int, batch: int = 32, cache: str | None = DEFAULT_CACHE):
    """The tile shape cached with this length class's layout (None: none)."""
    if not cache:
        return None
    db = _load(cache)
    key, _, _ = _key(ir_len, N0, batch)
    rec = db.get(key)
    if rec is None:
        tail = key[key.index("|"):]
        rec = next((v for k, v in sorted(db.items()) if k.endswith(tail)), None)
    t = rec["best"].get("tiles") if rec else None
    return tuple(t) if t else None


def choose_tiles(pcs, N0: int, name: str, cache: str | None = DEFAULT_CACHE, measure: bool = True,
                 verbose: bool = False):
    """Tile shape (bins, parts per spread task) for one handle holding these
    PCs, measured on the handle itself for every TILE_CANDIDATES entry and
    cached under `name` (a workload with layouts of several length classes
    takes one shape per handle).  Without measuring, a miss gives None."""
    key = f"{_gpu_name()}|tiles|{name}|N0={N0}|pcs={len(pcs)}"
    with _lock:
        db = _load(cache) if cache else {}
    rec = db.get(key)
    if rec is None and not measure:
        tail = key[key.index("|"):]
        rec = next((v for k, v in sorted(db.items()) if k.endswith(tail)), None)
    if rec is None:
        if not measure:
            return None
        res = []
        for tb, tp in TILE_CANDIDATES:
            us = measure_pcs(pcs, N0, tiles=(tb, tp))
            res.append({"tiles": [tb, tp], "us_per_step": us})
            if verbose:
                print(f"  tiles {tb}x{tp}: {us:.2f} us/step")
        rec = {"best": dict(min(res, key=lambda r: r["us_per_step"])), "candidates": res}
        if cache:
            _save(cache, key, rec)
    return tuple(rec["best"]["tiles"])


# ---------------------------------------------------------------------------
# Dynamic program over level costs (matlab/optimal_part.m's Viterbi search,
# restated over levels instead of block positions).
# ---------------------------------------------------------------------------
def model_level_cost(N: int, P: int, N0: int, k: float = 1.5) -> float:
    """Cost per base step of a level of block N with P parts under the
    reference's model (matlab/optimal_part.m: 4 k log2(2N) + 4 per new block
    size, 4 per part), amortised over the N / N0 base steps of one block."""
    return (4.0 * k * np.log2(2 * N) + 4.0 * P) * N0 / N


def optimal_part(ir_len: int, N0: int, level_cost=None, max_block: int = MAX_BLOCK, strict: bool = False):
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


def retune_batched_workload(streams: int = 32, samples: int = 1 << 19, cache: str | None = DEFAULT_CACHE,
                            verbose: bool = True):
    """Measure and cache the batched 32-stream workload's choices: a layout
    (and tile shape) per IR length class, then one tile shape for the handle
    holding all streams.  Existing entries for this GPU are measured again."""
    if cache:
        db = _load(cache)
        gpu = _gpu_name()
        for k in [k for k in db if k.startswith(gpu + "|")]:
            del db[k]
        with _lock:
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(db, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)

    def pick(L, n0):
        if verbose:
            print(f"IR length {L} (class {_len_class(L)}):")
        return choose_layout(L, n0, batch=streams, cache=cache, verbose=verbose)

    c = wl.cfg2(n_streams=streams, n_samples=1024, layout_fn=pick)
    pcs = [dict(ir=h, N=N, P=P) for h, (N, P) in zip(c["irs"], c["layouts"])]
    if verbose:
        print("tile shape of the whole handle:")
    return choose_tiles(pcs, c["N0"], "cfg2", cache=cache, verbose=verbose)


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="measure and cache layouts and tile shapes on this GPU")
    ap.add_argument("--cache", default=DEFAULT_CACHE)
    ap.add_argument("--streams", type=int, default=32)
    a = ap.parse_args()
    print("tiles:", retune_batched_workload(a.streams, cache=a.cache))
