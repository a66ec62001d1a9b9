"""Seeded synthetic workloads for the five benchmark configurations.

All draws use numpy ``Generator(PCG64(seed))`` in float64, cast to float32;
configuration k uses seed 1000 + k; draw order is IR parameters, IRs, inputs.
IRs are Gaussian noise times exp(-6.91 n / (T60 * 48000)) (a 60 dB decay over
T60 seconds), normalised to unit L2 norm, then scaled where stated.  There is
no dataset: these stand in for the reference's WAV reverbs.
"""
from __future__ import annotations

import math

import numpy as np

FS = 48000


def rng_for(cfg: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(1000 + cfg))


def decaying_ir(rng: np.random.Generator, length: int, t60: float, fs: int = FS) -> np.ndarray:
    n = np.arange(length, dtype=np.float64)
    h = rng.standard_normal(length) * np.exp(-6.91 * n / (t60 * fs))
    h /= np.linalg.norm(h)
    return h.astype(np.float32)


def chain_layout(ir_len: int, N0: int, ratio: int = 8, max_block: int = 16384, first_parts: int | None = None,
                 strict: bool = False):
    """Level chain: block sizes grow by ``ratio`` per level and every level
    but the last holds just enough parts for the next level's offset.  Default
    ("minimum slack", Gardner): s_{L+1} = N_{L+1}, the relaxed condition of
    matlab/MFDL_part_conv.m:25-31.  strict=True: s_{L+1} = 2 N_{L+1} - 2 N0,
    the reference's setup condition (src/partconv.cpp:148-170), which leaves
    each larger level N_{L+1}/N0 - 2 base steps between the completion of a
    block and its first output sample.  The last level (<= max_block) takes
    the rest.  Returns (N, P) with P[-1] recomputed from ir_len."""
    P0 = first_parts if first_parts is not None else (2 * ratio - 2 if strict else ratio)
    N = [N0]
    P = [P0]
    covered = N0 * P0
    while covered < ir_len:
        nb = N[-1] * ratio
        if nb > max_block:
            break
        # parts of the current level so that s_{L+1} reaches its target
        target = 2 * nb - 2 * N0 if strict else nb
        need = target - (covered - N[-1] * P[-1])
        P[-1] = max(P[-1], -(-need // N[-1]))
        covered = sum(n * p for n, p in zip(N, P))
        if covered >= ir_len:
            break
        N.append(nb)
        P.append(2 * ratio - 2 if strict else ratio - 1)
        covered += nb * P[-1]
    s_last = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    P[-1] = max(1, -(-(ir_len - s_last) // N[-1]))
    return N, P


def cfg1():
    """Plain mono: x 2^20 samples N(0, 0.1^2); IR 2^17 taps, T60 2.5 s
    (decay exp(-6.91 n / 120000)); layout 256x8 | 2048x7 | 16384x7."""
    rng = rng_for(1)
    h = decaying_ir(rng, 1 << 17, 2.5)
    x = (0.1 * rng.standard_normal(1 << 20)).astype(np.float32)
    return dict(x=x, h=h, N=[256, 2048, 16384], P=[8, 7, 7], N0=256)


def cfg2(n_streams: int = 32, n_samples: int = 1 << 19, N0: int = 256, layout_fn=None):
    """Batched streams: IR lengths round(2^U(14,19)), T60 ~ U(0.3, 4) s,
    inputs N(0, 0.1^2) of n_samples.  layout_fn(ir_len, N0) -> (N, P)
    (default: chain_layout)."""
    rng = rng_for(2)
    lens = np.round(2.0 ** rng.uniform(14, 19, n_streams)).astype(np.int64)
    t60 = rng.uniform(0.3, 4.0, n_streams)
    irs = [decaying_ir(rng, int(L), float(t)) for L, t in zip(lens, t60)]
    x = (0.1 * rng.standard_normal((n_streams, n_samples))).astype(np.float32)
    layout_fn = layout_fn or (lambda L, n0: chain_layout(L, n0))
    layouts = [layout_fn(len(h), N0) for h in irs]
    return dict(x=x, irs=irs, layouts=layouts, N0=N0, t60=t60)


def cfg3(n_in: int = 64, n_out: int = 64, n_samples: int = 1 << 18, ir_len: int = 1 << 15):
    """MIMO: n_in x n_out paths of ir_len taps (T60 0.5 s) scaled by 1/n_in;
    layout 128x16 | 2048x15."""
    rng = rng_for(3)
    irs = np.stack([decaying_ir(rng, ir_len, 0.5) for _ in range(n_in * n_out)]).reshape(n_in, n_out, ir_len)
    irs *= np.float32(1.0 / n_in)
    x = (0.1 * rng.standard_normal((n_in, n_samples))).astype(np.float32)
    return dict(x=x, irs=irs, N=[128, 2048], P=[16, 15], N0=128)


def cfg4(batch: int = 8, n_samples: int = 1 << 18, ir_len: int = 1 << 16):
    """Differentiable: target IR (T60 1 s), initial IR N(0, 0.01^2), inputs
    N(0, 0.1^2); layout 512x8 | 4096x15."""
    rng = rng_for(4)
    h_target = decaying_ir(rng, ir_len, 1.0)
    h_init = (0.01 * rng.standard_normal(ir_len)).astype(np.float32)
    x = (0.1 * rng.standard_normal((batch, n_samples))).astype(np.float32)
    return dict(x=x, h_target=h_target, h_init=h_init, N=[512, 4096], P=[8, 15], N0=512)


def cfg5_requests(n_streams: int = 1000, rate: float = 200.0, seconds: float = 10.0, seed_offset: int = 0):
    """Serving mix: Poisson arrivals at ``rate``/s; channels {1,2,8} with
    p = (.5,.3,.2); IR length round(2^U(12,20)); T60 ~ U(0.2, 5) s; N0 in
    {64,128,256,1024}; each stream carries ``seconds`` of audio.  Returns a
    list of request parameter dicts (IRs drawn lazily by ``make_request``)."""
    rng = np.random.Generator(np.random.PCG64(1005 + seed_offset))
    gaps = rng.exponential(1.0 / rate, n_streams)
    arrivals = np.cumsum(gaps)
    chans = rng.choice([1, 2, 8], size=n_streams, p=[0.5, 0.3, 0.2])
    lens = np.round(2.0 ** rng.uniform(12, 20, n_streams)).astype(np.int64)
    t60 = rng.uniform(0.2, 5.0, n_streams)
    n0 = rng.choice([64, 128, 256, 1024], size=n_streams)
    seeds = rng.integers(0, 2**62, n_streams)
    return [dict(arrival=float(a), channels=int(c), ir_len=int(L), t60=float(t), N0=int(b),
                 frames=int(math.ceil(seconds * FS / b) * b), seed=int(s))
            for a, c, L, t, b, s in zip(arrivals, chans, lens, t60, n0, seeds)]


def make_request(req: dict):
    """Draw one serving request's IRs (one per channel) and input."""
    rng = np.random.Generator(np.random.PCG64(req["seed"]))
    irs = [decaying_ir(rng, req["ir_len"], req["t60"]) for _ in range(req["channels"])]
    x = (0.1 * rng.standard_normal((req["channels"], req["frames"]))).astype(np.float32)
    return irs, x


def conv_fp64(x: np.ndarray, h: np.ndarray, n: int | None = None) -> np.ndarray:
    """Full linear convolution in float64 via FFT (first n samples)."""
    L = len(x) + len(h) - 1
    nf = 1 << (L - 1).bit_length()
    y = np.fft.irfft(np.fft.rfft(np.asarray(x, np.float64), nf) * np.fft.rfft(np.asarray(h, np.float64), nf), nf)
    return y[: (n if n is not None else L)]


def rel_l2(y: np.ndarray, ref: np.ndarray) -> float:
    d = np.linalg.norm(np.asarray(y, np.float64) - np.asarray(ref, np.float64))
    r = np.linalg.norm(np.asarray(ref, np.float64))
    return float(d / r) if r > 0 else float(d)


def algorithmic_bytes_per_sample(N, P) -> float:
    """Streaming bytes per audio sample for one convolver:
    sum_L B_L / N_L with B_L = 8 (N_L + 1)(2 P_L + 1) + 12 N_L (read H and
    the X ring, write the new X slot, read 2N inputs, write N outputs)."""
    return sum((8.0 * (n + 1) * (2 * p + 1) + 12.0 * n) / n for n, p in zip(N, P))


def fd_grads_fp64(x: np.ndarray, h: np.ndarray, target: np.ndarray, coords_h, coords_x, step: float = 1e-3):
    """FP64 central differences of L = mean((conv(x_b, h)[:T] - target_b)^2)
    over a batch x [B, T], at the IR taps ``coords_h`` and the input samples
    ``coords_x`` (pairs (b, i)), step ``step``.

    y is linear in h and in x, so L(h +- d e_j) only moves the residual by
    +- d x_b shifted by j, and L(x +- d e_(b,i)) moves row b by +- d h
    shifted by i; each difference (L+ - L-) / 2d is evaluated from those two
    loss values in float64.  Returns (dL/dh at coords_h, dL/dx at coords_x)."""
    x64 = np.asarray(x, np.float64)
    h64 = np.asarray(h, np.float64)
    B, T = x64.shape
    r = np.stack([conv_fp64(x64[b], h64, T) for b in range(B)]) - np.asarray(target, np.float64)
    M = r.size
    gh = np.empty(len(coords_h))
    for n, j in enumerate(coords_h):
        xs = np.zeros_like(x64)
        xs[:, j:] = x64[:, : T - j]
        lp = np.sum((r + step * xs) ** 2) / M
        lm = np.sum((r - step * xs) ** 2) / M
        gh[n] = (lp - lm) / (2 * step)
    gx = np.empty(len(coords_x))
    L = len(h64)
    for n, (b, i) in enumerate(coords_x):
        hs = np.zeros(T)
        m = min(L, T - i)
        hs[i:i + m] = h64[:m]
        # rows other than b are unchanged and cancel exactly in L+ - L-
        lp = np.sum((r[b] + step * hs) ** 2) / M
        lm = np.sum((r[b] - step * hs) ** 2) / M
        gx[n] = (lp - lm) / (2 * step)
    return gh, gx
