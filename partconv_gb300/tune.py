"""Partition search with the interface of the reference's src/tune.py
(ebattenberg/partconv), timed on the GPU.

Same entry points and meaning: ``init(N, L)`` sets the base block and IR
length; ``bench(parts, level='total', fs=44100.)`` sets up a PartConvFilter
with layout ``parts = [N0, P0, N1, P1, ...]`` (no IR: an all-ones one of the
layout's length) and returns the total load in percent of real time, or the
per-level loads plus the total with ``level='all'``; ``time(prev, ptr)``
recursively enumerates layouts (next block size ``ptr/2 + N``, part counts
2, 6, 14, ...) recording totals in ``total`` and partial timings in
``partial``; ``best(num)`` re-benches the fastest ones.  Timings come from
``PartConvFilter.bench`` (CUDA events around runLevel) instead of FFTW.
Written for Python 3 from the reference's behaviour, not translated.
"""
from __future__ import annotations

import math

from . import partconv

L = 0
N = 0
total: dict = {}
partial: dict = {}
num_benched = 0
type = "mean"
pc = None


def init(inN, inL):
    global L, N, total, partial, pc, num_benched
    L = int(inL)
    N = int(inN)
    total = {}
    partial = {}
    num_benched = 0
    pc = partconv.PartConvFilter()
    pc.FS = 44100


def bench(parts, level="total", fs=44100.0):
    """Load of layout ``parts`` in percent of real time (tune.py:21-55)."""
    global num_benched
    M = len(parts) // 2
    blocksize = partconv.intArray(M)
    numblocks = partconv.intArray(M)
    for i in range(M):
        blocksize[i] = int(parts[2 * i])
        numblocks[i] = int(parts[2 * i + 1])
    if pc.setup(M, blocksize, numblocks, None, 2, "wisdom.wis") != 0:
        return None
    loads = []
    for lv in range(M):
        t = pc.bench(lv, 1000, 3, 0.1)
        loads.append(t * 100.0 * fs / blocksize[lv])
    pc.cleanup()
    num_benched += 1
    if level == "all":
        return loads + [sum(loads)]
    if level == "total":
        return sum(loads)
    return None


def _key(parts):
    return " ".join(str(int(v)) for v in parts) + " "


def time(prev, ptr):
    """Recursive layout enumeration (tune.py:91-154): the next block size is
    ptr/2 + N; the current level first takes the whole remainder, then
    2, 6, 14, ... parts with the rest handed to a larger level."""
    rem = L - ptr
    B = N if ptr == 0 else ptr // 2 + N
    numB = math.ceil(rem / B)
    curr = [int(B), int(numB)]
    parts = list(prev) + curr
    prev_time = 0.0
    if prev:
        k = _key(prev)
        if k not in partial:
            partial[k] = bench(prev)
        prev_time = partial[k]
    k = _key(curr)
    if k not in partial:
        partial[k] = bench(curr)
    curr_time = partial[k]
    if prev_time is not None and curr_time is not None:
        total[prev_time + curr_time] = parts
    numB = 2
    while numB * B < rem / 4:
        curr = [int(B), int(numB)]
        k = _key(curr)
        if k not in partial:
            partial[k] = bench(curr)
        time(list(prev) + curr, ptr + numB * B)
        numB = numB * 2 + 2


def best(num=3):
    """Re-bench the `num` fastest layouts (tune.py:58-75); returns
    [(total load, parts, per-level loads)]."""
    out = []
    for t in sorted(total)[:num]:
        out.append((t, total[t], bench(total[t], "all")))
    return out
