#!/usr/bin/env python
"""Benchmark of the batched partitioned-convolution path.

Workload (one "step"): 32 independent mono float32 streams, each 2^19
samples of N(0, 0.1^2) input followed by zeros to flush its IR (IR lengths
log-uniform in [2^14, 2^19] taps, T60 U(0.3, 4) s, seeded), base block 256,
layouts chosen by the measured-GPU autotuner (partconv_gb300/autotune.py,
cached in partconv_gb300/autotune_cache.json), all streams in one handle: every
256-sample base block is one launch per kernel class, replayed from CUDA
graphs.  A step starts from reset state and processes the whole workload.

Metric: audio-seconds processed per second (48 kHz).  ``value`` runs on
device-resident inputs; ``e2e`` goes through the C ABI (pc_process) with
pinned host buffers, host<->device copies inside the timed region.  The
per-stream drop-in path (one handle and one pc_run call per stream per
block) is timed on a bounded sample as ``plain_gpu``.  ``cpu_baseline`` is
the oracle restatement of the reference CPU path on all host cores.

--impl reference times that CPU restatement alone on a bounded sample per
step.  The reference's own PartConvFilter code (built against an FFTW
stand-in as the oracle's pin) uses SSE3 intrinsics and compiles on x86_64
hosts only; on other hosts the restatement (bit for bit the reference's
code on the strict schedule; timed here on the minimum-latency schedule,
the same transforms and MACs per block) stands in.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FS = 48000


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--streams", type=int, default=32)
    ap.add_argument("--samples", type=int, default=None,
                    help="input samples per stream/channel (default: the workload's, 2^19 cfg2, 2^18 cfg3)")
    ap.add_argument("--plain-blocks", type=int, default=96, help="pc_run calls per stream in the plain sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=0, help="base steps for the per-kernel profile (0: 4*H)")
    ap.add_argument("--step-blocks", type=int, default=1,
                    help="cfg2: base blocks per step (pc_set_step_blocks); 1 = one launch per 256-sample block "
                         "(the headline). The other mode (4, or 1) is measured beside it")
    ap.add_argument("--no-alt", action="store_true", help="cfg2: skip the other blocks-per-step mode")
    ap.add_argument("--no-legs", action="store_true",
                    help="cfg2: skip the other workloads' legs (cfg3 MIMO, cfg4 adjoint, cfg5 serving) that the "
                         "default run records beside the headline")
    ap.add_argument("--serve-seconds", type=float, default=40.0, help="cfg5 leg: real-time limit of the load run")
    ap.add_argument("--max-block", type=int, default=16384,
                    help="cfg2 with --layouts chain: largest block of the chains (up to 65536)")
    ap.add_argument("--chain-ratio", type=int, default=8, help="cfg2 with --layouts chain: block ratio between levels")
    ap.add_argument("--layouts", default="auto", choices=["auto", "chain"],
                    help="cfg2 layouts: measured-GPU autotuner (cached) or the minimum-slack chain")
    ap.add_argument("--workload", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5"],
                    help="cfg2: batched streams (the headline); cfg1: plain mono drop-in; cfg3: 64x64 MIMO; "
                         "cfg4: forward + adjoint; cfg5: serving")
    return ap.parse_args()


# --------------------------------------------------------------------------
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, device=None):
    """Element-wise maximum over ranks of per-rank timings: a replicated job
    takes as long as its slowest rank.  Identity without a process group."""
    import torch
    import torch.distributed as dist

    vals = [float(v) for v in values]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vals
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_rate(world_size: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput of independent replicas: all ranks' units over
    the slowest rank's time."""
    return world_size * units_per_rank / seconds


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.idx)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.strip().split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = max(smax, float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


# --------------------------------------------------------------------------
def workload(streams: int, samples: int, layouts: str = "auto", measure: bool = True, align: int = 1,
             max_block: int = 16384, ratio: int = 8):
    """Config 2 inputs.  layouts: "auto" = the measured-GPU autotuner's
    choice per IR length class (its cache, measuring on a miss when allowed;
    the minimum-slack chain when not), "chain" = the minimum-slack chain.
    align: base blocks the frame count is rounded up to (zeros appended)."""
    from partconv_gb300 import autotune
    from partconv_gb300 import workloads as wl

    def pick(L, n0):
        if layouts == "auto":
            got = autotune.choose_layout(L, n0, batch=streams) if measure else autotune.cached_layout(L, n0, streams)
            if got:
                return got
        return wl.chain_layout(L, n0, ratio=ratio, max_block=max_block)

    c = wl.cfg2(n_streams=streams, n_samples=samples, layout_fn=pick)
    N0 = c["N0"]
    tail = max(len(h) for h in c["irs"])
    frames = samples + (tail + N0 - 1) // N0 * N0
    frames = (frames + align * N0 - 1) // (align * N0) * (align * N0)
    x = np.zeros((streams, frames), np.float32)
    x[:, :samples] = c["x"]
    return c, x, frames


def workload_name(streams: int, samples: int, frames1: int, N0: int) -> str:
    """The cfg2 workload as both arms name it in ``config.workload``."""
    return (f"cfg2: {streams} streams x {samples} samples + IR flush ({frames1} per stream), "
            f"IR 2^14..2^19 taps, N0={N0}")


def bytes_per_sample(layouts):
    from partconv_gb300 import workloads as wl

    return float(np.mean([wl.algorithmic_bytes_per_sample(N, P) for N, P in layouts]))


def cpu_baseline(c, x, frames, max_seconds=20.0, threads=None):
    """Oracle restatement on host threads over a bounded prefix of every
    stream; returns (audio-s/s, cores, sample description, elapsed)."""
    import oracle

    threads = threads or os.cpu_count() or 1
    S = x.shape[0]
    N0 = c["N0"]
    # probe 1/16 of the workload, then size the sample to ~max_seconds
    probe = max(N0 * 64, (frames // 16) // N0 * N0)
    _, t = oracle.run_streams(c["layouts"], c["irs"], x[:, :probe], N0, threads)
    rate = S * probe / max(t, 1e-9)
    n = int(min(frames, max(probe, rate * max_seconds / S)) // N0 * N0)
    _, t = oracle.run_streams(c["layouts"], c["irs"], x[:, :n], N0, threads)
    return S * n / FS / t, threads, f"first {n} of {frames} samples of all {S} streams", t


# --------------------------------------------------------------------------
def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    c, x, frames = workload(args.streams, args.samples, args.layouts, measure=False)
    import oracle

    threads = os.cpu_count() or 1
    N0 = c["N0"]
    S = x.shape[0]
    # bounded sample per step: sized from a probe to ~8 s per step
    probe = (frames // 32) // N0 * N0
    _, t = oracle.run_streams(c["layouts"], c["irs"], x[:, :probe], N0, threads)
    n = int(min(frames, max(probe, probe * 8.0 / max(t, 1e-9))) // N0 * N0)
    for _ in range(args.warmup):
        oracle.run_streams(c["layouts"], c["irs"], x[:, :n], N0, threads)
    times = []
    for _ in range(args.steps):
        _, t = oracle.run_streams(c["layouts"], c["irs"], x[:, :n], N0, threads)
        times.append(t)
    sec = float(np.mean(times))
    v = S * n / FS / sec
    sample = f"first {n} of {frames} samples of all {S} streams per step"
    line = {
        "impl": "reference", "metric": "audio-s/s (batched partitioned convolution, 32 streams, N0=256)",
        "value": v, "unit": "audio-s/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": workload_name(S, args.samples, frames, N0), "sample": sample},
        "cpu_baseline": {"value": v, "unit": "audio-s/s", "cores": threads, "kind": "port",
                         "sample": sample + "; CPU restatement of the reference path on the minimum-latency schedule (the same transforms and MACs per block as the reference's own code, which the restatement matches bit for bit on its strict schedule; that code needs SSE3, x86_64 only)"},
        "e2e": {"value": v, "unit": "audio-s/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
def run_ours(args):
    import torch

    from partconv_gb300 import PC_PLANAR, PartConvMulti

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    K = max(1, args.step_blocks)
    ALT = 4 if K == 1 else 1   # the other mode, measured beside the headline
    c, x_pad, frames_pad = workload(args.streams, args.samples, args.layouts, align=max(K, ALT),
                                    max_block=args.max_block, ratio=args.chain_ratio)
    S, N0 = x_pad.shape[0], c["N0"]
    # the workload's own length (input + IR flush); a step with K blocks pads
    # it to a multiple of K base blocks, and only the unpadded audio counts
    frames1 = args.samples + (max(len(h) for h in c["irs"]) + N0 - 1) // N0 * N0
    frames = frames1 if K == 1 else frames_pad
    x_host = np.ascontiguousarray(x_pad[:, :frames])
    pcs = [dict(ir=h, N=N, P=P, in_ch=s, out_ch=s) for s, (h, (N, P)) in enumerate(zip(c["irs"], c["layouts"]))]
    # kernel tile shape for this handle: the autotuner's measured choice (cached)
    tiles = None
    if args.layouts == "auto":
        from partconv_gb300 import autotune

        tiles = autotune.choose_tiles(pcs, N0, "cfg2", measure=True)
    m = PartConvMulti(step_blocks=K, tiles=tiles)
    m.setup_layout(FS, N0, S, S, pcs)
    info = m.info()
    K = info.step_blocks
    audio_s = S * frames1 / FS

    x = torch.from_numpy(x_host).to(dev)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)   # 256 MB > L2

    def one_step(h=m, n=frames, xd=x, yd=y):
        h.reset()
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.process_device(yd, xd, n, PC_PLANAR, stream)
        e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()

    # ---- parity of the benchmarked output (last warm-up) vs the oracle -----
    parity = None
    if not args.no_parity and rank == 0:
        import oracle
        from partconv_gb300 import workloads as wl

        y_np = y.cpu().numpy()
        t0 = time.time()
        ref, t_or = oracle.run_streams(c["layouts"], c["irs"], x_host, N0)
        errs = [wl.rel_l2(y_np[s], ref[s]) for s in range(S)]
        parity = {"rel_l2_max_vs_oracle": max(errs), "tol": 1e-5, "oracle_seconds": time.time() - t0}

    # ---- timed region -----------------------------------------------------------
    clocks = ClockSampler(local)
    launches0 = m.kernel_launches()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    w0 = time.perf_counter()
    evs = [one_step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    launches = m.kernel_launches() - launches0
    ms = max_over_ranks([np.mean([a.elapsed_time(b) for a, b in evs])], dev)[0]
    value = job_rate(ws, audio_s, ms / 1e3)

    # ---- the same workload in the other mode (K = 4 base blocks per launch,
    #      or one launch per block when the headline uses K > 1) ---------------
    alt = None
    if not args.no_alt:
        m1 = PartConvMulti(step_blocks=ALT, tiles=tiles)
        m1.setup_layout(FS, N0, S, S, pcs)
        alt_k = m1.info().step_blocks
        n_alt = frames_pad if alt_k > 1 else frames1
        x1 = torch.from_numpy(np.ascontiguousarray(x_pad[:, :n_alt])).to(dev)
        y1 = torch.empty_like(x1)
        for _ in range(args.warmup):
            one_step(m1, n_alt, x1, y1)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        l1 = m1.kernel_launches()
        ev1 = [one_step(m1, n_alt, x1, y1) for _ in range(args.steps)]
        torch.cuda.synchronize()
        ms1 = max_over_ranks([np.mean([a.elapsed_time(b) for a, b in ev1])], dev)[0]
        alt = {"step_blocks": alt_k, "value": job_rate(ws, audio_s, ms1 / 1e3), "unit": "audio-s/s", "ms_per_step": ms1,
               "gpu_launches": int(m1.kernel_launches() - l1),
               "rel_l2_max_vs_headline": max(
                   float(torch.linalg.vector_norm(y1[s_, :frames1] - y[s_, :frames1]) /
                         torch.linalg.vector_norm(y[s_, :frames1]).clamp_min(1e-30)) for s_ in range(S)),
               "how": f"same layouts, {alt_k} base block{'s' if alt_k > 1 else ''} per level-0 launch "
                      "(pc_set_step_blocks), same audio counted"}
        del m1, x1, y1

    # ---- e2e: host buffers through the C ABI (pinned), copies timed -------------
    xp = torch.from_numpy(x_host).pin_memory()
    yp = torch.empty_like(xp).pin_memory()
    m.reset()
    m.process_into(yp.data_ptr(), xp.data_ptr(), frames, PC_PLANAR)   # grows device buffers once
    e2e_times = []
    for _ in range(max(1, args.steps)):
        m.reset()
        t0 = time.perf_counter()
        m.process_into(yp.data_ptr(), xp.data_ptr(), frames, PC_PLANAR)
        e2e_times.append(time.perf_counter() - t0)
    if ws > 1:
        torch.distributed.barrier()
    e2e_v = job_rate(ws, audio_s, max_over_ranks([np.mean(e2e_times)], dev)[0])
    nbytes = x_host.nbytes

    # ---- per-kernel profile for the roofline --------------------------------------
    m.reset()
    prof_steps = args.profile_steps or max(4 * info.hyperperiod, 256)
    m.process_device(y, x, frames, PC_PLANAR, stream)   # fill state (steady-state FDL)
    torch.cuda.synchronize()
    prof = m.profile_kernels(prof_steps)
    dom = max(prof, key=lambda r: r["launches"])   # the level-0 kernel: one launch per base step
    per_launch_s = dom["total_ms"] / 1e3 / dom["launches"]   # isolated launches (profile pass)
    per_launch_b = dom["alg_bytes"] / dom["launches"]
    peak, peak_kind = measured_peak_gbs()
    # Inside the timed region the level-0 kernel runs once per base step and
    # consecutive launches overlap (programmatic dependent launch), so its
    # live average duration per launch is the timed time over its launches.
    live_launch_s = (ms / 1e3) / (frames // (N0 * K))
    achieved = per_launch_b / live_launch_s / 1e9
    # captured per kernel kind and blocks per step (the K-block kernel is another instance)
    traffic = ncu_traffic().get(dom["name"] if K == 1 else f"{dom['name']}@K{K}")
    kernels = {r["name"]: {"launches": r["launches"], "avg_us": r["total_ms"] * 1e3 / r["launches"],
                           "share": r["total_ms"] / sum(q["total_ms"] for q in prof),
                           "alg_bytes_per_launch": r["alg_bytes"] / r["launches"],
                           "achieved_gbs": r["alg_bytes"] / (r["total_ms"] / 1e3) / 1e9} for r in prof}

    # ---- plain per-stream drop-in path (bounded sample) -----------------------------
    plain = None
    if rank == 0 and args.plain_blocks > 0:
        hs = []
        for s in range(S):
            ms_ = PartConvMulti()
            ms_.setup_layout(FS, N0, 1, 1, [pcs[s] | dict(in_ch=0, out_ch=0)])
            hs.append(ms_)
        buf = np.zeros(N0, np.float32)
        lat = []
        R = args.plain_blocks
        for b in range(8):   # warm
            for s in range(S):
                hs[s].run(buf, x_host[s, b * N0:(b + 1) * N0], N0)
        t0 = time.perf_counter()
        for b in range(R):
            for s in range(S):
                a = time.perf_counter()
                hs[s].run(buf, x_host[s, b * N0:(b + 1) * N0], N0)
                lat.append(time.perf_counter() - a)
        tp = time.perf_counter() - t0
        plain_v = S * R * N0 / FS / tp
        plain = {"value": plain_v, "unit": "audio-s/s",
                 "sample": f"{R} pc_run calls per stream x {S} streams (one handle per stream)",
                 "pc_run_latency_us": {"p50": float(np.percentile(lat, 50) * 1e6),
                                       "p99": float(np.percentile(lat, 99) * 1e6)}}
        del hs

    # ---- batched per-block latency: one base step of all streams, device time ------
    # (one block of all streams is contiguous in the interleaved layout)
    m.reset()
    B = N0 * K   # samples of one step
    nlat = min(frames // B, max(2 * info.hyperperiod // K, 256))
    step_ms = []
    xi = torch.from_numpy(np.ascontiguousarray(x_host[:, : nlat * B].T)).to(dev)
    yi = torch.empty_like(xi)
    for b in range(nlat):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.process_device(yi[b * B:(b + 1) * B], xi[b * B:(b + 1) * B], B, 0, stream)
        e1.record(stream)
        step_ms.append((e0, e1))
    torch.cuda.synchronize()
    lat_us = [a.elapsed_time(b) * 1e3 for a, b in step_ms]

    # ---- CPU baseline (oracle port, all host threads, bounded sample) ------------------
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, sample, _ = cpu_baseline(c, x_host, frames)
        cpu = {"value": v, "unit": "audio-s/s", "cores": cores, "kind": "port",
               "sample": sample + "; CPU restatement of the reference path on the minimum-latency schedule (the same transforms and MACs per block as the reference's own code, which the restatement matches bit for bit on its strict schedule; that code needs SSE3, x86_64 only)"}

    if rank == 0:
        bps = bytes_per_sample(c["layouts"])
        line = {
            "metric": "audio-s/s (batched partitioned convolution, 32 streams, N0=256)",
            "value": value, "unit": "audio-s/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded numpy PCG64, cfg seed 1002)",
            "config": {"workload": workload_name(S, args.samples, frames1, N0),
                       "execution": f"one handle, graph-replayed steps of {K} base block{'s' if K > 1 else ''}",
                       "step_blocks": K,
                       "tiles": {"spread_bins": info.spread_bins, "spread_parts": info.spread_parts,
                                 "how": "bins and parts per spread task, measured by the autotuner on this handle"
                                        if tiles else "default"},
                       "frames_processed_per_stream": frames,
                       "layouts": ("autotuned from measured GPU timings (partconv_gb300/autotune_cache.json)"
                                   if args.layouts == "auto"
                                   else f"minimum-slack level chain (ratio {args.chain_ratio}, max {args.max_block})"),
                       "max_block": max(max(N) for N, _ in c["layouts"]),
                       "layout_set": sorted({f"{N}x{P}" for N, P in c["layouts"]})[:8],
                       "streams": S, "frames_per_stream": frames, "N0": N0,
                       "hyperperiod_steps": info.hyperperiod,
                       "l2": "256 MB buffer written between timed steps (outside the events); "
                             "FDL state (%.0f MB) stays L2-resident within a step" % (info.device_bytes / 1e6),
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": e2e_v, "unit": "audio-s/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "how": "pc_process on pinned host buffers (planar), copies inside the timed region"},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "limited_by": "latency: the level-0 step chain (one dependent launch per base block); the "
                                       "FDL state is L2-resident and DRAM moves a few % of the algorithmic bytes "
                                       "(traffic below)",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": per_launch_b, "avg_launch_us": live_launch_s * 1e6,
                         "isolated_launch_us": per_launch_s * 1e6,
                         "how": "avg_launch_us: timed region / level-0 launches in it (one per base step, "
                                "overlapping); isolated_launch_us: CUDA events around single launches"},
            "kernels": kernels,
            "path_alg_bytes_per_sample": bps,
            "path_roofline_frac": (bps * S * frames1 / (ms / 1e3)) / 1e9 / peak,
            "block_latency_us": {"p50": float(np.percentile(lat_us, 50)), "p99": float(np.percentile(lat_us, 99)),
                                 "max": float(np.max(lat_us)), "deadline_us": B / FS * 1e6,
                                 "how": f"device time of one step ({K} base block{'s' if K > 1 else ''}, all "
                                        "streams), single launches"},
            "wall_s_timed_region": wall,
        }
        if alt:
            line["alt_step_blocks"] = alt
        if plain:
            line["plain_gpu"] = plain
            line["batched_over_plain"] = value / plain["value"]
        if cpu:
            line["cpu_baseline"] = cpu
        if parity:
            line["parity"] = parity
        if clk:
            line["clocks"] = clk
        if not args.no_legs and ws == 1:
            # the other workloads, each its own measurement on this GPU, so one
            # default run records them beside the headline
            import argparse as _ap

            legs = {}
            for name, fn, steps in (("cfg3_mimo", run_mimo, 5), ("cfg4_adjoint", run_adjoint, 20),
                                    ("cfg5_serving", run_serving, 0)):
                sub = _ap.Namespace(**vars(args))
                sub.steps, sub.warmup, sub.samples, sub.streams = max(steps, 1), 3, None, 32
                try:
                    legs[name] = fn(sub)
                except Exception as e:   # a leg that fails is reported, the headline stands
                    legs[name] = {"error": f"{type(e).__name__}: {e}"}
            line["legs"] = legs
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_mimo(args):
    """Config 3: 64 x 64 MIMO paths of 2^15 taps, 2^18 frames + IR flush,
    layout 128x16 | 2048x15, per-bin channel sums.  audio-s/s counts
    multichannel frames (one 64-channel frame = 1/48000 audio-s)."""
    import torch

    from partconv_gb300 import workloads as wl
    from partconv_gb300.mimo import PartConvMIMO

    torch.cuda.set_device(0)
    c = wl.cfg3(n_samples=args.samples or (1 << 18))
    irs, N, P = c["irs"], c["N"], c["P"]
    n_in, n_out, L = irs.shape
    frames = c["x"].shape[1] + L
    x = np.zeros((n_in, frames), np.float32)
    x[:, : c["x"].shape[1]] = c["x"]
    m = PartConvMIMO()
    m.setup(irs, N, P)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty((n_out, frames), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")   # 256 MB > L2

    def step():
        m.reset()
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.process_device(yd, xd, frames, 1, stream)
        e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = m.kernel_launches()
    clocks = ClockSampler(0)
    clocks.start()
    evs = [step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    launches = m.kernel_launches() - launches0
    value = frames / FS / (ms / 1e3)
    m.reset()
    prof = m.profile_kernels(64)
    mac = [r for r in prof if r["name"] == "mimo_mac"][0]
    peak, peak_kind = measured_peak_gbs()
    ach = mac["alg_bytes"] / (mac["total_ms"] / 1e3) / 1e9
    line = {
        "metric": "audio-s/s (MIMO 64x64 per-bin channel sum)", "value": value, "unit": "audio-s/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "dtype": "f32", "data": "synthetic (seeded numpy PCG64, cfg seed 1003)",
        "config": {"workload": f"cfg3: {n_in}x{n_out} paths of {L} taps, {frames} frames, layout 128x16|2048x15",
                   "device_bytes": m.device_bytes(),
                   "l2": "256 MB buffer written between timed steps (outside the events); the level-0 filter "
                         "spectra (68 MB, read every base step) are loaded with an L2 evict-last policy, the "
                         "level-1 spectra evict-first (the spectra, 1.07 GB, exceed L2)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "mimo_mac", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "peak_kind": peak_kind,
                     "alg_bytes_per_launch": mac["alg_bytes"] / mac["launches"],
                     "avg_launch_us": mac["total_ms"] * 1e3 / mac["launches"]},
        "kernels": {r["name"]: {"launches": r["launches"], "avg_us": r["total_ms"] * 1e3 / r["launches"],
                                "share": r["total_ms"] / sum(q["total_ms"] for q in prof)} for r in prof},
    }
    if clk:
        line["clocks"] = clk
    return line


def run_adjoint(args):
    """Config 4: batch 8 x 2^18, learnable 2^16-tap IR, MSE loss; a step is
    forward + hand-written backward (dL/dx and dL/dh)."""
    import torch

    from partconv_gb300 import workloads as wl
    from partconv_gb300.adjoint import PartitionedConv

    torch.cuda.set_device(0)
    c = wl.cfg4()
    x = torch.from_numpy(c["x"]).cuda().requires_grad_(True)
    B, T = c["x"].shape
    t64 = np.stack([wl.conv_fp64(c["x"][b], c["h_target"], T) for b in range(B)])
    target = torch.from_numpy(t64.astype(np.float32)).cuda()
    mod = PartitionedConv(c["h_init"], c["N"], c["P"], B, T).cuda()
    stream = torch.cuda.current_stream()

    def step():
        mod.h.grad = None
        x.grad = None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        loss = torch.mean((mod(x) - target) ** 2)
        loss.backward()
        e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = mod.plan.kernel_launches()
    evs = [step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    launches = int(mod.plan.kernel_launches() - l0)
    audio = B * T / FS
    gx_ours, gh_ours = x.grad.detach().double(), mod.h.grad.detach().double()

    # the same loss through a dense FFT convolution with torch autograd: in
    # float64 as the gradient reference, in float32 as the timing comparison
    def dense(dtype):
        xd = x.detach().to(dtype).requires_grad_(True)
        hd = mod.h.detach().to(dtype).requires_grad_(True)
        n = 1 << int(np.ceil(np.log2(T + hd.shape[0])))
        y = torch.fft.irfft(torch.fft.rfft(xd, n) * torch.fft.rfft(hd, n), n)[:, :T]
        loss = torch.mean((y - target.to(dtype)) ** 2)
        loss.backward()
        return xd.grad, hd.grad

    gx64, gh64 = dense(torch.float64)
    rel = lambda a, b: float(torch.linalg.norm(a - b) / torch.linalg.norm(b))  # noqa: E731
    # FP64 central differences (step 1e-3) at 64 random IR taps and 64 random
    # input samples; the last timed step's gradients (same IR, same inputs)
    frng = np.random.default_rng(77)
    ch = np.sort(frng.choice(len(c["h_init"]), 64, replace=False))
    cx = [(int(b), int(i)) for b, i in zip(frng.integers(0, B, 64), frng.choice(T, 64, replace=False))]
    fd_h, fd_x = wl.fd_grads_fp64(c["x"], c["h_init"], t64, ch, cx, 1e-3)
    gh_np, gx_np = gh_ours.cpu().numpy(), gx_ours.cpu().numpy()
    fd_err_h = wl.rel_l2(gh_np[ch], fd_h)
    fd_err_x = wl.rel_l2(np.array([gx_np[b, i] for b, i in cx]), fd_x)
    for _ in range(2):
        dense(torch.float32)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        dense(torch.float32)
    e1.record(stream)
    torch.cuda.synchronize()
    dense_ms = e0.elapsed_time(e1) / args.steps
    return ({"metric": "audio-s/s (differentiable conv, forward + backward)", "value": audio / (ms / 1e3),
                      "unit": "audio-s/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
                      "data": "synthetic (seeded numpy PCG64, cfg seed 1004)",
                      "config": {"workload": "cfg4: batch 8 x 2^18, IR 2^16 taps, layout 512x8|4096x15, MSE"},
                      "gpu_launches": launches,
                      "parity": {"dL_dh_rel_l2_vs_dense_fp64": rel(gh_ours, gh64),
                                 "dL_dx_rel_l2_vs_dense_fp64": rel(gx_ours, gx64),
                                 "dL_dh_rel_l2_vs_fd64": fd_err_h, "dL_dx_rel_l2_vs_fd64": fd_err_x,
                                 "tol": 1e-6,
                                 "how": "dense: same inputs, IR and loss through torch.fft convolution autograd in "
                                        "float64; fd64: FP64 central differences, step 1e-3, 64 random IR taps "
                                        "and 64 random input samples"},
                      "dense_torch_fft_fp32": {"ms_per_step": dense_ms, "value": audio / (dense_ms / 1e3),
                                               "unit": "audio-s/s"}})


def run_plain_mono(args):
    """Config 1: the plain drop-in on one mono stream, 2^20 samples + IR
    flush, IR 2^17 taps, layout 256x8 | 2048x7 | 16384x7 (relaxed slack).
    Reports pc_run per-block latency (host buffers, one call per 256-sample
    block, as an audio callback makes it), pc_process throughput, the CPU
    oracle on one core, and the error against the oracle and FP64."""
    import torch

    import oracle
    from partconv_gb300 import PartConvMulti
    from partconv_gb300 import workloads as wl

    torch.cuda.set_device(0)
    c = wl.cfg1()
    N0 = c["N0"]
    x = np.concatenate([c["x"], np.zeros(len(c["h"]), np.float32)])
    frames = (len(x) + N0 - 1) // N0 * N0
    x = np.concatenate([x, np.zeros(frames - len(x), np.float32)])[:, None]
    pcs = [dict(ir=c["h"], N=c["N"], P=c["P"])]
    m = PartConvMulti()
    m.setup_layout(FS, N0, 1, 1, pcs)
    audio_s = frames / FS
    # pc_process over the whole signal (host buffers, copies included)
    for _ in range(args.warmup):
        m.reset()
        y = m.process(x)
    times = []
    for _ in range(args.steps):
        m.reset()
        t0 = time.perf_counter()
        y = m.process(x)
        times.append(time.perf_counter() - t0)
    proc = audio_s / float(np.mean(times))
    # pc_run: one call per block, wall time per call
    m.reset()
    out = np.zeros(N0, np.float32)
    nb = min(frames // N0, 4096)
    lat = np.zeros(nb)
    for b in range(nb):
        t0 = time.perf_counter()
        m.run(out, x[b * N0:(b + 1) * N0], N0)
        lat[b] = time.perf_counter() - t0
    plain = nb * N0 / FS / float(lat.sum())
    # the CPU restatement over the same signal: one core, and reference-shaped
    # (one worker thread per level, as the reference's level threads)
    t0 = time.perf_counter()
    ref = oracle.OracleMulti(N0, 1, 1, pcs).run(x)[:, 0]
    cpu_s = time.perf_counter() - t0
    _, lvl_s = oracle.run_leveled(c["N"], c["P"], c["h"], x[:, 0])
    ref64 = wl.conv_fp64(c["x"], c["h"])
    n = len(ref64)
    line = {"metric": "audio-s/s (plain mono drop-in, cfg1)", "value": proc, "unit": "audio-s/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded numpy PCG64, cfg seed 1001)",
            "config": {"workload": f"cfg1: 1 stream x {frames} frames (2^20 + IR flush), IR 2^17 taps, "
                                   "256x8|2048x7|16384x7", "how": "pc_process on host buffers, copies timed"},
            "e2e": {"value": proc, "unit": "audio-s/s", "h2d_bytes_per_step": int(x.nbytes),
                    "d2h_bytes_per_step": int(x.nbytes)},
            "plain_pc_run": {"value": plain, "unit": "audio-s/s", "blocks": int(nb),
                             "latency_us": {"p50": float(np.percentile(lat, 50) * 1e6),
                                            "p99": float(np.percentile(lat, 99) * 1e6),
                                            "max": float(lat.max() * 1e6)},
                             "deadline_us": N0 / FS * 1e6},
            "cpu_baseline": {"value": audio_s / lvl_s, "unit": "audio-s/s", "cores": len(c["N"]), "kind": "port",
                             "sample": "whole signal, one worker thread per level (reference-shaped); restated "
                                       "CPU path (own FFT); reference FFTW build unavailable"},
            "cpu_single_core": {"value": audio_s / cpu_s, "unit": "audio-s/s", "cores": 1},
            "parity": {"rel_l2_vs_oracle": wl.rel_l2(y[:n, 0], ref[:n]), "rel_l2_vs_fp64": wl.rel_l2(y[:n, 0], ref64),
                       "oracle_rel_l2_vs_fp64": wl.rel_l2(ref[:n], ref64), "tol": 1e-5}}
    print(json.dumps(line))
    return 0


def run_serving(args):
    """Config 5: Poisson arrivals at 200/s up to 1000 concurrent streams of
    1/2/8 channels, IRs 2^12..2^20 taps, base blocks 64..1024, 10 s of audio
    each, real time; per-block latency and deadline misses."""
    import torch

    from partconv_gb300 import workloads as wl
    from partconv_gb300.serving import Server

    torch.cuda.set_device(0)
    reqs = wl.cfg5_requests(n_streams=args.streams if args.streams != 32 else 1000)
    t0 = time.time()
    irs = []
    for r in reqs:
        g = np.random.Generator(np.random.PCG64(r["seed"]))
        irs.append([wl.decaying_ir(g, r["ir_len"], r["t60"]) for _ in range(r["channels"])])
    noise = (0.1 * np.random.default_rng(5).standard_normal(1 << 22)).astype(np.float32)
    gen_s = time.time() - t0
    srv = Server(hbm_budget_bytes=160 << 30, max_pcs_per_pool=4096)
    stats = srv.run_load(reqs, irs, noise, max_concurrent=1000, max_seconds=args.serve_seconds)
    return ({"metric": "serving: per-block latency and audio-s/s (cfg5 mix, real time)",
                      "value": stats["audio_s_per_s"], "unit": "audio-s/s", "n_gpus": 1, "higher_is_better": True,
                      "dtype": "f32", "data": "synthetic (seeded; inputs are slices of one noise buffer)",
                      "config": {"workload": "cfg5: 1000 streams, Poisson 200/s, 1/2/8 ch, IR 2^12..2^20, "
                                             "N0 64..1024, 10 s each", "request_gen_s": gen_s},
                      "serving": stats})


def main():
    args = parse_args()
    if args.samples is None and args.workload == "cfg2":
        args.samples = 1 << 19
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "cfg1":
        return run_plain_mono(args)
    if args.workload in ("cfg3", "cfg4", "cfg5"):
        line = {"cfg3": run_mimo, "cfg4": run_adjoint, "cfg5": run_serving}[args.workload](args)
        print(json.dumps(line))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
