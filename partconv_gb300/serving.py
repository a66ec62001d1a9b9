"""Serving: a continuous-batching request loop over partitioned-convolution
pools.

Requests (streams of 1..n channels, each channel with its own impulse
response, a base block size and an input of fixed length) arrive over time.
Each channel is one partitioned convolver (PC) in the pool of its block size
(pcs_* C ABI, include/partconv_gb300.h).  A request is admitted when every
one of its channels fits the pool's HBM budget; otherwise it waits in a
queue until finished requests release memory.  Each pool ticks once per
base block period; a tick gathers the next block of every active channel,
runs one batched GPU step for all of them on the pool's own CUDA stream (so
pools overlap on the device) and scatters the outputs when the step
completes.  Per-block latency is the time from the tick (block due) to the
step's completion; a block misses its deadline when that exceeds one block
period.  No reference counterpart: the reference drives one fixed
PartConvMulti from an audio callback (src/pcRTMulti.cpp:138-185).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat
from ._native import PartConvError
from . import workloads as wl


def serving_layout(ir_len: int, N0: int, ratio: int = 4, max_levels: int = 5, max_block: int = 16384):
    """Block-size chain for a pooled PC: ratio-4 levels (at most five, blocks
    up to 16384) with minimum slack (s_{L+1} = N_{L+1})."""
    N = [N0]
    P = [ratio]
    while sum(n * p for n, p in zip(N, P)) < ir_len and len(N) < max_levels and N[-1] * ratio <= max_block:
        N.append(N[-1] * ratio)
        P.append(ratio - 1)
    s_last = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    if s_last >= ir_len and len(N) > 1:   # last level not needed
        N.pop()
        P.pop()
        s_last = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    P[-1] = max(1, -(-(ir_len - s_last) // N[-1]))
    return N, P


class ServingPool:
    """PCs of one base block size sharing one HBM-budget arena."""

    def __init__(self, block_size: int, hbm_budget_bytes: int, max_pcs: int):
        self._lib = nat.lib()
        self._h = self._lib.pcs_create(int(block_size), int(hbm_budget_bytes), int(max_pcs))
        if not self._h:
            raise PartConvError(nat.PC_ERR_CUDA, "pcs_create failed (CUDA device, budget >= 1 MiB, block size)")
        self.block_size = int(block_size)
        self.max_pcs = int(max_pcs)

    def _check(self, code):
        if code != nat.PC_OK:
            raise PartConvError(code, self._lib.pcs_last_error(self._h).decode())

    def admit(self, ir, N, P, wait: bool = True) -> int:
        """Admit one channel.  wait=False returns at once with the PC pending:
        poll() makes it live when its spectra are built (is_live tells)."""
        ir = np.ascontiguousarray(ir, dtype=np.float32)
        Nv = np.ascontiguousarray(N, dtype=np.int32)
        Pv = np.ascontiguousarray(P, dtype=np.int32).copy()
        pid = C.c_int(-1)
        fn = self._lib.pcs_admit if wait else self._lib.pcs_admit_async
        self._check(fn(self._h, ir.ctypes.data_as(nat._f32p), len(ir), len(Nv),
                       Nv.ctypes.data_as(nat._i32p), Pv.ctypes.data_as(nat._i32p), C.byref(pid)))
        return pid.value

    def poll(self) -> int:
        """Make live the pending PCs whose admission work has completed."""
        n = C.c_int(0)
        self._check(self._lib.pcs_poll(self._h, C.byref(n)))
        return n.value

    def is_live(self, pc_id: int) -> bool:
        return self._lib.pcs_is_live(self._h, int(pc_id)) == 1

    def release(self, pc_id: int):
        self._check(self._lib.pcs_release(self._h, int(pc_id)))

    def step(self, in_ptr: int, out_ptr: int, n_channels: int):
        self._check(self._lib.pcs_step(self._h, C.c_void_p(in_ptr), C.c_void_p(out_ptr), int(n_channels)))

    def done(self) -> bool:
        return self._lib.pcs_query(self._h) == 1

    def sync(self):
        self._check(self._lib.pcs_sync(self._h))

    def bytes_in_use(self) -> int:
        return int(self._lib.pcs_bytes_in_use(self._h))

    def live(self) -> int:
        return int(self._lib.pcs_live(self._h))

    def kernel_launches(self) -> int:
        return int(self._lib.pcs_kernel_launches(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.pcs_destroy(h)
            except Exception:
                pass
            self._h = None


@dataclass
class _Req:
    rid: int
    spec: dict
    irs: list = None
    x: np.ndarray = None
    y: np.ndarray = None
    pcs: list = field(default_factory=list)
    pos: int = 0          # next block to feed
    done_blocks: int = 0  # blocks whose output has arrived
    admitted_at: float = -1.0
    finished_at: float = -1.0


class Server:
    """Continuous batching over pools keyed by base block size."""

    def __init__(self, hbm_budget_bytes: int, block_sizes=(64, 128, 256, 1024), max_pcs_per_pool: int = 1024,
                 fs: int = 48000):
        import torch

        self.fs = fs
        share = int(hbm_budget_bytes) // len(block_sizes)
        self.pools = {b: ServingPool(b, share, max_pcs_per_pool) for b in block_sizes}
        self.max_pcs = max_pcs_per_pool
        self._in = {b: torch.zeros((max_pcs_per_pool, b), dtype=torch.float32).pin_memory() for b in block_sizes}
        self._out = {b: torch.zeros((max_pcs_per_pool, b), dtype=torch.float32).pin_memory() for b in block_sizes}

    # ------------------------------------------------------------------------
    def _try_admit(self, r: _Req) -> bool:
        pool = self.pools[r.spec["N0"]]
        if r.irs is None:
            r.irs, r.x = wl.make_request(r.spec)
            r.y = np.zeros_like(r.x)
        N, P = serving_layout(r.spec["ir_len"], r.spec["N0"])
        got = []
        try:
            for ch in range(r.spec["channels"]):
                got.append(pool.admit(r.irs[ch], N, P))
        except PartConvError as e:
            for pid in got:
                pool.release(pid)
            if e.code in (nat.PC_ERR_NOMEM, nat.PC_ERR_LIMIT):
                return False
            raise
        r.pcs = got
        return True

    def run(self, requests, realtime: bool = True, max_concurrent: int = 1000, max_seconds: float = 600.0,
            keep_outputs: bool = True):
        """Serve `requests` (dicts from workloads.cfg5_requests or the same
        fields).  realtime=False runs as fast as the GPU allows (ticks when
        the previous step completed; arrivals in tick time).  Returns stats
        and, with keep_outputs, each request's output [channels, frames]."""
        reqs = [_Req(i, s) for i, s in enumerate(sorted(requests, key=lambda s: s["arrival"]))]
        pending = list(reqs)
        queue: list[_Req] = []
        active = {b: [] for b in self.pools}
        period = {b: b / self.fs for b in self.pools}
        next_tick = {b: 0.0 for b in self.pools}
        inflight = {b: None for b in self.pools}   # (tick_time, [(req, chan_offset)], n_ch)
        lat_us, miss, steps_done, blocks_done = [], 0, 0, 0
        vt = 0.0                                   # virtual clock for realtime=False
        t0 = time.perf_counter()
        now = lambda: (time.perf_counter() - t0) if realtime else vt  # noqa: E731
        concurrent = 0
        peak_concurrent = 0
        finished = []
        while len(finished) < len(reqs):
            t = now()
            if t > max_seconds:
                break
            # arrivals and admissions (FIFO: a waiting request blocks later ones)
            while pending and pending[0].spec["arrival"] <= t:
                queue.append(pending.pop(0))
            while queue and concurrent < max_concurrent:
                r = queue[0]
                if not self._try_admit(r):
                    break
                queue.pop(0)
                r.admitted_at = t
                active[r.spec["N0"]].append(r)
                concurrent += 1
                peak_concurrent = max(peak_concurrent, concurrent)
            progressed = False
            for b, pool in self.pools.items():
                # completion of the step in flight
                if inflight[b] is not None and pool.done():
                    tick_t, members, _ = inflight[b]
                    tdone = time.perf_counter() - t0 if realtime else vt
                    out = self._out[b].numpy()
                    for r, start_block in members:
                        for ch, pid in enumerate(r.pcs):
                            r.y[ch, start_block * b:(start_block + 1) * b] = out[pid]
                        r.done_blocks += 1
                        if r.done_blocks * b >= r.x.shape[1]:
                            for pid in r.pcs:
                                pool.release(pid)
                            r.finished_at = tdone
                            active[b].remove(r)
                            finished.append(r)
                            concurrent -= 1
                    lat = (tdone - tick_t) * 1e6 if realtime else None
                    if lat is not None:
                        lat_us.extend([lat] * len(members))
                        if lat > period[b] * 1e6:
                            miss += len(members)
                    blocks_done += sum(len(r.pcs) for r, _ in members)
                    steps_done += 1
                    inflight[b] = None
                    progressed = True
                # a tick is due: one batched step for every active channel
                if inflight[b] is None and active[b] and (not realtime or next_tick[b] <= t):
                    feeders = [r for r in active[b] if r.pos * b < r.x.shape[1]]
                    if not feeders:
                        continue
                    inp = self._in[b].numpy()
                    n_ch = 0
                    members = []
                    for r in feeders:
                        blk = r.x[:, r.pos * b:(r.pos + 1) * b]
                        for ch, pid in enumerate(r.pcs):
                            inp[pid] = blk[ch]
                            n_ch = max(n_ch, pid + 1)
                        members.append((r, r.pos))
                        r.pos += 1
                    tick_t = (time.perf_counter() - t0) if realtime else vt
                    if realtime and next_tick[b] < tick_t - period[b]:
                        next_tick[b] = tick_t          # fell behind: restart the cadence
                    next_tick[b] += period[b]
                    pool.step(self._in[b].data_ptr(), self._out[b].data_ptr(), n_ch)
                    inflight[b] = (tick_t, members, n_ch)
                    progressed = True
            if not realtime:
                if not progressed:
                    # advance virtual time to the next arrival when idle
                    busy = any(v is not None for v in inflight.values())
                    if busy:
                        time.sleep(0)
                    elif pending:
                        vt = max(vt, pending[0].spec["arrival"])
                    else:
                        vt += min(period.values())
                else:
                    vt += min(period.values()) / 4
            elif not progressed:
                time.sleep(50e-6)
        wall = time.perf_counter() - t0
        audio_s = sum(r.x.shape[0] * r.x.shape[1] for r in finished) / self.fs
        stats = {
            "requests": len(reqs), "finished": len(finished), "peak_concurrent": peak_concurrent,
            "steps": steps_done, "blocks": blocks_done, "wall_s": wall, "audio_s": audio_s,
            "audio_s_per_s": audio_s / wall if wall > 0 else 0.0,
        }
        if lat_us:
            stats.update(latency_us_p50=float(np.percentile(lat_us, 50)),
                         latency_us_p99=float(np.percentile(lat_us, 99)),
                         latency_us_max=float(np.max(lat_us)),
                         deadline_miss_rate=miss / len(lat_us))
        outputs = {r.rid: r.y for r in finished} if keep_outputs else None
        return stats, outputs

    def run_load(self, requests, irs, noise: np.ndarray, max_concurrent: int = 1000, max_seconds: float = 120.0,
                 seed: int = 4321):
        """Real-time load run for throughput and latency, in native code
        (pcs_run_load: admission, per-tick gathers, steps and latency
        accounting run on this thread without the Python interpreter): every
        channel reads its input from ``noise`` (a shared float32 buffer,
        channel c of request r starting at a seeded offset) and outputs are
        discarded.  irs[r] holds request r's IRs (one per channel)."""
        blocks = sorted(self.pools)
        idx = {b: i for i, b in enumerate(blocks)}
        n = len(requests)
        keep = []   # arrays the native loop reads
        arrival = np.array([r["arrival"] for r in requests], np.float64)
        pool_of = np.array([idx[r["N0"]] for r in requests], np.int32)
        chans = np.array([r["channels"] for r in requests], np.int32)
        frames = np.array([r["frames"] for r in requests], np.int64)
        ir_len = np.array([r["ir_len"] for r in requests], np.int32)
        M, Nf, Pf, ptrs = [], [], [], []
        for ri, r in enumerate(requests):
            N, P = serving_layout(r["ir_len"], r["N0"])
            M.append(len(N))
            Nf += list(N)
            Pf += list(P)
            for ch in range(r["channels"]):
                a = np.ascontiguousarray(irs[ri][ch], np.float32)
                assert len(a) == r["ir_len"]
                keep.append(a)
                ptrs.append(a.ctypes.data_as(nat._f32p))
        M = np.array(M, np.int32)
        Nf = np.array(Nf, np.int32)
        Pf = np.array(Pf, np.int32)
        noise = np.ascontiguousarray(noise, np.float32)
        handles = (C.c_void_p * len(blocks))(*[self.pools[b]._h for b in blocks])
        pblock = np.array(blocks, np.int32)
        ip = lambda a: a.ctypes.data_as(nat._i32p)  # noqa: E731
        st = nat.PCSLoadStats()
        lib = nat.lib()
        rc = lib.pcs_run_load(handles, ip(pblock), len(blocks), n, arrival.ctypes.data_as(C.POINTER(C.c_double)),
                              ip(pool_of), ip(chans), frames.ctypes.data_as(C.POINTER(C.c_longlong)),
                              (nat._f32p * max(1, len(ptrs)))(*ptrs), ip(ir_len), ip(M), ip(Nf), ip(Pf),
                              noise.ctypes.data_as(nat._f32p), len(noise), int(seed), int(max_concurrent),
                              float(max_seconds), float(self.fs), C.byref(st))
        if rc != nat.PC_OK:
            raise PartConvError(rc, "pcs_run_load failed: " + "; ".join(
                self.pools[b]._lib.pcs_last_error(self.pools[b]._h).decode() for b in blocks))
        return {"requests": int(st.requests), "finished": int(st.finished), "peak_concurrent": int(st.peak_concurrent),
                "wall_s": st.wall_s, "audio_s": st.audio_s,
                "audio_s_per_s": st.audio_s / st.wall_s if st.wall_s > 0 else 0.0, "blocks": int(st.blocks),
                "steps": int(st.steps),
                "latency_us_p50": st.latency_p50_us, "latency_us_p99": st.latency_p99_us,
                "latency_us_max": st.latency_max_us, "deadline_miss_rate": st.miss_rate,
                "per_block_size": {str(blocks[i]): {"period_us": blocks[i] / self.fs * 1e6,
                                                    "steps": int(st.pool_steps[i]), "blocks": int(st.pool_blocks[i]),
                                                    "step_latency_us_p50": st.pool_p50_us[i],
                                                    "step_latency_us_p99": st.pool_p99_us[i],
                                                    "deadline_miss_rate": st.pool_miss_rate[i]}
                                   for i in range(len(blocks))},
                "launches": sum(p.kernel_launches() for p in self.pools.values()),
                "loop": "native (pcs_run_load)"}
