// step_kernels.cu -- the per-base-block kernel of the partitioned
// convolution engine (sm_103a).
//
// One base step c (one run() callback of N0 frames) is a set of tasks, one
// CTA each:
//   * fire: level L of one PC computes its block b when its input completes
//     ((c + 1) N0 + s_L == (b + 1) N_L): load the newest 2 N_L input samples,
//     real FFT (shared-memory Stockham), store the spectrum in ring slot
//     b mod P_L, Y = X_b H_0 + (partial sum of the older parts), inverse FFT,
//     keep the first N_L samples (overlap-save with the block at offset N_L,
//     matlab/FDL_part_conv.m:18-20 of ebattenberg/partconv).  The MAC is the
//     one of PartConvFilter::runLevel (src/partconv.cpp:354-490) split in
//     time: level 0 adds X_{b-1} H_1 itself and reads the sum over p >= 2
//     that spread tasks built during the previous step; other levels read the
//     sum over p >= 1 built during the N_L/N0 - 1 steps since their last block.
//     Level 0's CTA then emits the step's output: its block plus the due
//     N0-slice of every other level's output ring, in level order
//     (PartConvFilter::output, src/partconv.cpp:616-631), mixed into the
//     output channel (src/partconvMulti.cpp:911-921).
//   * spread: the streaming FDL MAC over a slice of bins,
//     Yp[k] = sum_p X[(b'-p) mod P][k] H[p][k] for the level's next block b'.
//     This is where the reference's per-level worker threads spread a large
//     block's work over the base periods (src/partconvMulti.cpp:930-1013).
// Tasks of one step touch disjoint data (level 0's partial sums are double
// buffered by block parity), so every CTA of a step runs independently; the
// next step depends on this one.
//
// Latency: a small fire is a chain of dependent steps, so every phase that
// touches global memory first issues all of its loads into registers and
// only then uses them (one memory round trip per phase).
#include <cuda_runtime.h>

#include <algorithm>

#include "engine_types.h"
#include "fft_smem.cuh"
#include "kernels.h"

namespace pcg {

__device__ __forceinline__ long long imod(long long a, long long m) {
    long long r = a % m;
    return r < 0 ? r + m : r;
}

__device__ __forceinline__ float4 f4mac(float4 acc, float4 x, float4 h) {
    // two complex multiply-adds: (x.x + i x.y)(h.x + i h.y), (x.z + i x.w)(h.z + i h.w)
    acc.x += x.x * h.x - x.y * h.y;
    acc.y += x.x * h.y + x.y * h.x;
    acc.z += x.z * h.z - x.w * h.w;
    acc.w += x.z * h.w + x.w * h.z;
    return acc;
}
__device__ __forceinline__ float4 f4mul(float4 x, float4 h) { return f4mac(make_float4(0.f, 0.f, 0.f, 0.f), x, h); }
__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// Kernel class: threads per CTA, largest block size, operand prefetch.
template <int NT_, int MAXN_, bool PREFETCH_>
struct Cls {
    static constexpr int NT = NT_;
    static constexpr int MAXN = MAXN_;
    static constexpr bool PREFETCH = PREFETCH_;
    static constexpr int MAXB = MAXN / 4 / NT;                   // radix-4 butterflies per thread
    static constexpr int MAXQ = (MAXN / 2 + NT - 1) / NT;        // window quads (4 samples) per thread
    static constexpr int MAXT = (MAXN / 2 + NT - 1) / NT;        // twiddles per thread
    static constexpr int MAXK = (MAXN / 2 + 1 + NT - 1) / NT;    // bin pairs per thread (prefetch)
    static constexpr int MAXE = (MAXN / 4 + NT - 1) / NT;        // output quads per thread
    static constexpr int SPLIT_CH = 4;                           // post-FFT pairs loaded per batch
    static_assert(MAXB >= 1, "class too small");
};
// dynamic shared memory that leaves no room for a level-0 CTA beside it on
// an SM (228 KB per SM, 1 KB reserved per CTA, 227 KB per CTA at most)
constexpr size_t kWholeSmSmem = 220 * 1024;
using Cls0 = Cls<256, 1024, true>;
using Cls1 = Cls<512, 4096, false>;
// 1024 threads: four radix-4 butterflies per thread per stage at N = 16384
// (64 registers); the fire of one 16384-sample block takes 54 instead of
// 60 us with 512 threads
using Cls2 = Cls<1024, 16384, false>;

// dynamic shared memory bytes of a fire for block size N
__host__ __device__ constexpr size_t fire_smem_bytes(int N, bool prefetch) {
    // data N + quarter twiddles N/2 complex (+ yacc N+2, h0 N+2 complex, emit N
    // floats, FFT scratch N complex)
    return prefetch ? (size_t)8 * N + 4 * N + 16 * ((size_t)N + 2) + 4 * (size_t)N + 8 * (size_t)N
                    : (size_t)8 * N + 4 * (size_t)N;
}

// ---------------------------------------------------------------------------
// Spread: the streaming FDL MAC over the task's bins [k0, k1) and parts
// [p_lo, p_hi).  NT threads form G = NT / LANES part-groups of LANES
// threads; thread t owns bins k0 + 2 (t mod LANES), +1 (one float4) and sums
// parts p_lo + g, + G, ... (g = t / LANES); the groups are added in order
// through shared memory.  Bins per task (2 LANES; a tile shape the autotuner
// picks per handle) travel in the task's M field, 0 meaning kSpreadBins;
// each width is its own instantiation (constant strides): the step kernel
// is instantiated per width and launched for the handle's width.  Parts per task
// set how many partial-sum rows a level keeps.
//
// Measured and rejected: the G threads of one bin pair as adjacent lanes of
// a warp, summed by warp shuffles instead of shared memory (no barrier) --
// 33 % slower per step on 32 streams (3.48 -> 4.65 us for 256x14 | 2048x14 |
// 16384x15): each warp load then spans G rows instead of one.  A runtime
// group width in the same loop cost 4 % (3.48 -> 3.63 us).
// ---------------------------------------------------------------------------
constexpr int kSpreadBins = 128;   // default bins per task
constexpr int kSpreadParts = 16;   // default parts per task (one round of loads per thread)
constexpr int kSpreadLanes = 64;   // K-block level-0 spreads (spread_multi): threads per part-group

// kb: base blocks per step (level 0 keeps 2 kb partial-sum buffers per row).
template <int NT, int LANES>
__device__ __forceinline__ void spread_lanes(const Task& tk, long long c, float4* red, int kb) {
    constexpr int G = NT / LANES;
    const int lane = threadIdx.x % LANES;
    const int g = threadIdx.x / LANES;
    const int k = tk.k0 + 2 * lane;
    const bool active = k < tk.k1;
    long long bt;      // block whose partial sum this step builds
    float2* dst;
    c -= tk.origin;    // the PC's own step count
    if (tk.T == 1) {   // level 0: parts p >= 2 kb of block c + 1, [row][block mod 2 kb][cs]
        const int nbuf = 2 * kb;
        bt = c + 1;
        dst = tk.Yp + ((size_t)tk.out_ch * nbuf + (size_t)(bt & (nbuf - 1))) * tk.cs;   // kb: a power of two
    } else {           // the block after the newest fired one: parts p >= 1, or
                       // p >= 2 (double-buffered) for a deferred level
        const size_t row = (size_t)tk.out_ch * 2;   // [row][parity][cs]
        bt = (c + 1 + tk.s_blocks) / tk.T;
        dst = tk.Yp + (row + (tk.dfer ? (size_t)(bt & 1) : 0)) * tk.cs;
    }
    const int P = tk.P;
    const int p_hi = tk.in_ch > 0 ? tk.in_ch : P;
    const size_t rs4 = (size_t)(tk.cs >> 1);   // row stride in float4
    const float4* X4 = reinterpret_cast<const float4*>(tk.X + k);
    const float4* H4 = reinterpret_cast<const float4*>(tk.H + k);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        constexpr int U = 4;   // parts whose loads are in flight together
        const int Gm = G % P;  // slot step between a group's consecutive parts
        int sl0 = (int)imod(bt - (tk.p_lo + g), P);   // slot of part p0
        for (int p0 = tk.p_lo + g; p0 < p_hi; p0 += U * G) {
            float4 xv[U], hv[U];
            int sl = sl0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int p = p0 + u * G;
                if (p < p_hi) {
                    xv[u] = __ldcg(X4 + (size_t)sl * rs4);
                    hv[u] = __ldg(H4 + (size_t)p * rs4);
                }
                sl -= Gm;
                if (sl < 0) sl += P;
            }
            sl0 = sl;
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (p0 + u * G < p_hi) acc = f4mac(acc, xv[u], hv[u]);
        }
    }
    if (G > 1) {
        if (g > 0) red[(g - 1) * LANES + lane] = acc;
        __syncthreads();
        if (g == 0 && active) {
#pragma unroll
            for (int j = 1; j < G; ++j) acc = f4add(acc, red[(j - 1) * LANES + lane]);
            *reinterpret_cast<float4*>(dst + k) = acc;
        }
    } else if (active) {
        *reinterpret_cast<float4*>(dst + k) = acc;
    }
}

// red: NT - 32 float4 of shared memory at least
template <int NT>
__device__ __forceinline__ void spread_body(const Task& tk, long long c, float4* red, int kb) {
    switch (tk.M > 0 ? tk.M : kSpreadBins) {
        case 64: spread_lanes<NT, 32>(tk, c, red, kb); break;
        case 256: spread_lanes<NT, (NT >= 128 ? 128 : NT)>(tk, c, red, kb); break;
        case 512: spread_lanes<NT, (NT >= 256 ? 256 : NT)>(tk, c, red, kb); break;
        default: spread_lanes<NT, 64>(tk, c, red, kb); break;
    }
}

// Level 0 with K base blocks per step: parts [p_lo, p_hi) of the next
// step's K blocks bt_j = c + 1 + j (the task's c is the step's last base
// step) over one slice of bins: each filter row is loaded once for the K
// blocks.  Group g sums parts p_lo + g, p_lo + g + G, ...; groups are added
// in order, per block.
template <int NT, int KM>
__device__ __forceinline__ void spread_multi(const Task& tk, long long c, float4* red) {
    constexpr int G = NT / kSpreadLanes;
    constexpr int U = 2;   // parts whose loads are in flight together
    const int lane = threadIdx.x % kSpreadLanes;
    const int g = threadIdx.x / kSpreadLanes;
    const int k = tk.k0 + 2 * lane;
    const bool active = k < tk.k1;
    c -= tk.origin;
    const long long bt0 = c + 1;
    const int nbuf = 2 * KM;
    const int P = tk.P;
    const int p_hi = tk.in_ch > 0 ? tk.in_ch : P;
    const size_t rs4 = (size_t)(tk.cs >> 1);
    const float4* X4 = reinterpret_cast<const float4*>(tk.X + k);
    const float4* H4 = reinterpret_cast<const float4*>(tk.H + k);
    float4 acc[KM];
#pragma unroll
    for (int j = 0; j < KM; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        const int Gm = G % P;
        int sl0 = (int)imod(bt0 - (tk.p_lo + g), P);   // slot of block bt0 - p for the group's part p
        for (int p0 = tk.p_lo + g; p0 < p_hi; p0 += U * G) {
            float4 xv[U][KM], hv[U];
            int sl = sl0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (p0 + u * G < p_hi) {
                    hv[u] = __ldg(H4 + (size_t)(p0 + u * G) * rs4);
                    int sj = sl;
#pragma unroll
                    for (int j = 0; j < KM; ++j) {   // blocks bt0 + j - p: consecutive slots
                        xv[u][j] = __ldcg(X4 + (size_t)sj * rs4);
                        sj = (sj + 1 == P) ? 0 : sj + 1;
                    }
                }
                sl -= Gm;
                if (sl < 0) sl += P;
            }
            sl0 = sl;
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (p0 + u * G < p_hi) {
#pragma unroll
                    for (int j = 0; j < KM; ++j) acc[j] = f4mac(acc[j], xv[u][j], hv[u]);
                }
        }
    }
#pragma unroll
    for (int j = 0; j < KM; ++j) {
        float2* dst = tk.Yp + ((size_t)tk.out_ch * nbuf + (size_t)((bt0 + j) & (nbuf - 1))) * tk.cs;
        if (G > 1) {
            if (g > 0) red[(g - 1) * kSpreadLanes + lane] = acc[j];
            __syncthreads();
            if (g == 0 && active) {
                float4 a = acc[j];
#pragma unroll
                for (int q = 1; q < G; ++q) a = f4add(a, red[(q - 1) * kSpreadLanes + lane]);
                *reinterpret_cast<float4*>(dst + k) = a;
            }
            __syncthreads();   // red is reused for the next block
        } else if (active) {
            *reinterpret_cast<float4*>(dst + k) = acc[j];
        }
    }
}

// ---------------------------------------------------------------------------
// EARLY (step kernels): a level-0 fire whose whole window lies in this
// call's input runs its forward transform and forms X_b H_0 before waiting
// for the previous step, keeping X_b in registers; only the global writes
// (X_b, the input-ring append), X_{b-1} H_1 + Yp, the inverse transform and
// the output follow the wait.  Before the wait a step kernel reads only data
// no kernel writes (input, twiddles, filter spectra) and writes only shared
// memory, so it may overlap any number of earlier step kernels: it signals
// its dependents at entry.
// Output samples 4 i4 .. 4 i4 + 3 of a transform buffer (complex elements
// 2 i4 and 2 i4 + 1, which sidx keeps in one aligned pair, possibly swapped).
template <bool SW>
__device__ __forceinline__ float4 ld_out4(const float2* s, int i4) {
    const int p = sidx<SW>(2 * i4);
    const float4 v = *reinterpret_cast<const float4*>(s + (p & ~1));
    return (p & 1) ? make_float4(v.z, v.w, v.x, v.y) : v;
}

template <class C, bool EARLY>
__device__ __forceinline__ void fire_body(const Bank& bank, const Task& tk, const RunState& rs, long long c,
                                          float2* smem, int* s_last) {
    constexpr int NT = C::NT;
    const int tid = threadIdx.x;
    const int N = tk.N, logN = tk.logN, P = tk.P, cs = tk.cs;
    const int N0 = bank.N0;
    const bool l0 = (tk.T == 1);
    // a deferred fire runs after the step that completed its block (its whole
    // window is in the input ring) and sums X_b H_0 + X_{b-1} H_1 + Yp[b & 1]
    // like level 0, with parts >= 2 spread over the level's phases
    const bool dfer = tk.dfer != 0;
    const bool two = l0 || dfer;
    float2* s = smem;                 // N complex
    float2* twt = s + N;              // N/2 quarter-wave twiddles
    float2* yacc = twt + N / 2;       // N + 2 (PREFETCH)
    float2* h0s = yacc + (N + 2);     // N + 2 (PREFETCH)
    float* emit = reinterpret_cast<float*>(h0s + (N + 2));   // N0 floats (PREFETCH, level 0)
    float2* ftmp = reinterpret_cast<float2*>(emit + N);       // N complex FFT scratch (PREFETCH)
    const Twiddles tw{twt, logN};
    // the large classes keep the transform buffer in the conflict-free
    // placement (element i at s[sidx<SW>(i)])
    constexpr bool SW = !C::PREFETCH;
    // prefetch classes transform through the scratch buffer (fewer barriers)
    auto fft = [&](bool inv) {
        if constexpr (C::PREFETCH) {
            switch (logN) {   // unrolled for the common base blocks; same results
                case 7: fft_smem_pp_c<NT, C::MAXB, 7>(s, ftmp, twt, inv); break;
                case 8: fft_smem_pp_c<NT, C::MAXB, 8>(s, ftmp, twt, inv); break;
                case 9: fft_smem_pp_c<NT, C::MAXB, 9>(s, ftmp, twt, inv); break;
                default: fft_smem_pp<NT, C::MAXB>(s, ftmp, N, logN, tw, inv);
            }
        } else {
            fft_smem<NT, C::MAXB, SW>(s, N, logN, tw, inv);
        }
    };

    const long long io_step = c - rs.io.step0;   // I/O is addressed by the global step
    c -= tk.origin;                              // schedule and rings by the PC's own steps
    const long long q = c + 1 + tk.s_blocks;
    const long long b = q / tk.T - 1;
    const int slot = (int)imod(b, P);
    const long long t_new = c * (long long)N0;
    const long long t_end = t_new + N0;
    const float* in = rs.io.in + io_step * rs.io.in_step + (long long)tk.in_ch * rs.io.in_ch;
    const long long isamp = rs.io.in_sample;
    const float scale = tk.scale;
    const float2* X1 = tk.X + (size_t)imod(b - 1, P) * cs;   // block b-1 (level 0, p = 1)
    const float2* Ypb = tk.Yp + (two ? (size_t)(b & 1) * cs : 0);   // row 0; row q at + 2 q cs
    const int npart = tk.k0 > 0 ? tk.k0 : 1;
    const size_t rstride = 2 * (size_t)cs;

    const int nq = N >> 1;                       // window quads: samples t_end - 2N + 4q .. + 3
    const int nq_old = dfer ? nq : nq - (N0 >> 2);   // quads before this step's input
    const int npair = (N + 2) >> 1;              // bin pairs (float4 of two bins)
    const bool use_x1 = two && P >= 2;
    const bool use_yp = (two && P >= 3) || (!two && P >= 2);
    const bool early = EARLY && C::PREFETCH && l0 && io_step >= 1;
    const int Le = tk.M - 1 < kEmitLevels ? tk.M - 1 : kEmitLevels;
    // the other levels' due output slices, summed in level order into `emit`
    // (their fires completed before this launch: full graph/stream edges)
    auto gather_emit = [&]() {
        if constexpr (C::PREFETCH) {
            float4 ev[C::PREFETCH ? C::MAXE : 1][kEmitLevels];
#pragma unroll
            for (int i = 0; i < C::MAXE; ++i) {
                const int e4 = tid + i * NT;
#pragma unroll
                for (int L = 0; L < kEmitLevels; ++L)
                    if (L < Le && 4 * e4 < N0)
                        ev[i][L] = __ldcg(reinterpret_cast<const float4*>(tk.eyring[L] + ((t_new + 4 * e4) & tk.emask[L])));
            }
#pragma unroll
            for (int i = 0; i < C::MAXE; ++i) {
                const int e4 = tid + i * NT;
                if (4 * e4 >= N0) continue;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int L = 0; L < kEmitLevels; ++L)
                    if (L < Le) v = f4add(v, ev[i][L]);
                for (int L = kEmitLevels + 1; L < tk.M; ++L) {   // rare: more than 5 levels
                    const DevLevel& l2 = bank.lv[tk.lv_index + L];
                    v = f4add(v, __ldcg(reinterpret_cast<const float4*>(l2.yring + ((t_new + 4 * e4) & l2.rmask))));
                }
                *reinterpret_cast<float4*>(emit + 4 * e4) = v;
            }
        }
    };

    // ---- static prologue: data no running kernel writes (twiddles, filter
    //      rows, this call's input), so it overlaps the previous step's tail.
    //      The input-ring append and the other levels' output slices wait for
    //      the dependency (a larger level of the same kernel class may still
    //      be reading the ring and writing its output in the previous step).
    float4 wv[C::MAXQ];   // this step's input quads (kept for the EARLY ring append)
    {
#pragma unroll
        for (int i = 0; i < C::MAXQ; ++i) {
            const int qd = tid + i * NT;
            if (qd >= nq_old && qd < nq) {
                const long long j = 4LL * (qd - nq_old);
                wv[i] = make_float4(in[j * isamp] * scale, in[(j + 1) * isamp] * scale, in[(j + 2) * isamp] * scale,
                                    in[(j + 3) * isamp] * scale);
            } else if (early && qd < nq_old) {   // previous block, from the call's input
                const float* pin = in - rs.io.in_step;
                const long long j = 4LL * qd;
                wv[i] = make_float4(pin[j * isamp] * scale, pin[(j + 1) * isamp] * scale,
                                    pin[(j + 2) * isamp] * scale, pin[(j + 3) * isamp] * scale);
            }
        }
        const int ntw = N >> 1;
        const int sh = bank.wlog - (logN + 1);
        float2 tv[C::MAXT];
#pragma unroll
        for (int i = 0; i < C::MAXT; ++i) {
            const int m = tid + i * NT;
            if (m < ntw) tv[i] = __ldg(&bank.W[m << sh]);
        }
        float4 ha[C::PREFETCH ? C::MAXK : 1], h0a[C::PREFETCH ? C::MAXK : 1];
        if (C::PREFETCH) {
#pragma unroll
            for (int i = 0; i < C::MAXK; ++i) {
                const int kk = 2 * (tid + i * NT);
                if (kk < 2 * npair) {
                    h0a[i] = __ldg(reinterpret_cast<const float4*>(tk.H + kk));
                    if (use_x1) ha[i] = __ldg(reinterpret_cast<const float4*>(tk.H + cs + kk));
                }
            }
        }
#pragma unroll
        for (int i = 0; i < C::MAXQ; ++i) {
            const int qd = tid + i * NT;
            if ((qd >= nq_old || early) && qd < nq) {
                s[sidx<SW>(2 * qd)] = make_float2(wv[i].x, wv[i].y);
                s[sidx<SW>(2 * qd + 1)] = make_float2(wv[i].z, wv[i].w);
            }
        }
#pragma unroll
        for (int i = 0; i < C::MAXT; ++i) {
            const int m = tid + i * NT;
            if (m < ntw) twt[SW ? twsw(m) : m] = tv[i];
        }
        if (C::PREFETCH) {
#pragma unroll
            for (int i = 0; i < C::MAXK; ++i) {
                const int kk = 2 * (tid + i * NT);
                if (kk < 2 * npair) {
                    *reinterpret_cast<float4*>(h0s + kk) = h0a[i];
                    if (use_x1) *reinterpret_cast<float4*>(yacc + kk) = ha[i];   // H_1 until X_{b-1} arrives
                }
            }
        }
    }

    float2* __restrict__ Xs = tk.X + (size_t)slot * cs;
    const int half = N >> 1;

    // Prefetch classes run the split/MAC/merge in two passes with X_b H_0
    // parked in shared memory, whether or not the forward transform ran
    // before the dependency wait: one sequence of float operations, so the
    // EARLY and the in-order paths give identical bits.
    constexpr int kXr = C::PREFETCH ? C::MAXK : 1;
    float2 xr[kXr][2];   // EARLY: this thread's X_b pairs until after the wait
    auto forward_pass = [&]() {   // forward FFT, X_b, X_b H_0 -> h0s (k = half: N - k product in slot N + 1)
        __syncthreads();
        fft(false);
        int j = 0;
        for (int k = tid; k <= half; k += NT, ++j) {
            const int nk = (k == 0) ? 0 : N - k;
            float2 xk, xnk;
            rfft_split(s[k], s[nk], k, logN, tw, xk, xnk);
            const int bnk = N - k;
            if (early) {
                if (j < kXr) {
                    xr[j][0] = xk;
                    xr[j][1] = xnk;
                }
            } else {
                Xs[k] = xk;
                if (bnk != k) Xs[bnk] = xnk;
            }
            const float2 pk = cmul(xk, h0s[k]);
            const float2 pnk = cmul(xnk, h0s[bnk]);
            h0s[k] = pk;
            h0s[bnk != k ? bnk : N + 1] = pnk;
        }
    };
    // Y = X_b H_0 + (X_{b-1} H_1 + Yp[b & 1]) and the inverse merge into s, by
    // bin pair (k, N - k) -- the pairs the forward split gave this thread, so
    // it reads only its own h0s entries; H_1 waits in yacc since the prologue.
    // xp, yp: this thread's X_{b-1} and partial sums of its pairs.
    auto merge_pass = [&](const float2 (*xp)[2], const float2 (*yp)[2]) {
#pragma unroll
        for (int j = 0; j < kXr; ++j) {
            const int k = tid + j * NT;
            if (k > half) continue;
            const int bnk = N - k;
            float2 ak = make_float2(0.f, 0.f), ank = ak;
            if (use_x1) {
                ak = cmul(xp[j][0], yacc[k]);
                ank = cmul(xp[j][1], yacc[bnk]);
            }
            if (use_yp) {
                ak = cadd(ak, yp[j][0]);
                ank = cadd(ank, yp[j][1]);
            }
            const float2 yk = cadd(h0s[k], ak);
            const float2 ynk = cadd(h0s[bnk != k ? bnk : N + 1], ank);
            float2 zk, znk;
            irfft_merge(yk, ynk, k, logN, tw, zk, znk);
            s[k] = zk;
            if (k != 0 && k != half) s[N - k] = znk;
        }
        __syncthreads();
    };

    // several PCs feed this output: the last one to arrive sums them in PC
    // order (deterministic, no atomics on samples, no waiting)
    auto mix_last = [&](float* out, long long osamp, long long och) {
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const int o = tk.out_ch;
            const int cnt = bank.out_off[o + 1] - bank.out_off[o];
            *s_last = (atomicAdd(&bank.mix_cnt[o], 1) == cnt - 1);
        }
        __syncthreads();
        if (!*s_last) return;
        __threadfence();
        const int o = tk.out_ch;
        const int j0 = bank.out_off[o], j1 = bank.out_off[o + 1];
        for (int i = tid; i < N0; i += NT) {
            float v = 0.0f;
            for (int j = j0; j < j1; ++j) v += __ldcg(&bank.pcs[bank.out_pcs[j]].pcout[i]);
            out[i * osamp + (long long)o * och] = v;
        }
        if (tid == 0) bank.mix_cnt[o] = 0;
    };

    if (early) forward_pass();

    // earlier steps' kernels have completed and their writes are visible
    cudaGridDependencySynchronize();
    if (early) {   // X_b, held in registers since the forward pass
        for (int k = tid, j = 0; k <= half; k += NT, ++j) {
            const int bnk = N - k;
            Xs[k] = xr[j][0];
            if (bnk != k) Xs[bnk] = xr[j][1];
        }
    }

    if constexpr (C::PREFETCH) {
        // ---- dependent inputs: input-ring history (unless EARLY), previous
        //      spectrum, partial sums, the other levels' due output slices ----
        float4 wo[C::MAXQ];
        float2 xp[kXr][2], yp[kXr][2];
        if (!early) {
#pragma unroll
            for (int i = 0; i < C::MAXQ; ++i) {
                const int qd = tid + i * NT;
                if (qd < nq_old) {
                    const long long ta = t_end - 2LL * N + 4LL * qd;
                    wo[i] = __ldcg(reinterpret_cast<const float4*>(tk.xring + (ta & tk.rin_mask)));
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kXr; ++j) {
            const int k = tid + j * NT;
            if (k <= half) {
                const int bnk = N - k;
                if (use_x1) {
                    xp[j][0] = __ldcg(&X1[k]);
                    xp[j][1] = __ldcg(&X1[bnk]);
                }
                if (use_yp) {
                    yp[j][0] = __ldcg(&Ypb[k]);
                    yp[j][1] = __ldcg(&Ypb[bnk]);
                    for (int q = 1; q < npart; ++q) {
                        yp[j][0] = cadd(yp[j][0], __ldcg(&Ypb[q * rstride + k]));
                        yp[j][1] = cadd(yp[j][1], __ldcg(&Ypb[q * rstride + bnk]));
                    }
                }
            }
        }
        if (l0) gather_emit();
#pragma unroll
        for (int i = 0; i < C::MAXQ; ++i) {
            const int qd = tid + i * NT;
            if (qd < nq_old) {
                if (!early) {
                    s[2 * qd] = make_float2(wo[i].x, wo[i].y);
                    s[2 * qd + 1] = make_float2(wo[i].z, wo[i].w);
                }
            } else if (l0 && qd < nq) {   // level 0 appends this step's input to the PC's ring
                const long long ta = t_end - 2LL * N + 4LL * qd;
                *reinterpret_cast<float4*>(tk.xring + (ta & tk.rin_mask)) = wv[i];
            }
        }
        if (!early) forward_pass();
        merge_pass(xp, yp);
    } else {
        // ---- dependent inputs (no prefetch): input-ring history ----------------
        {
            float4 wo[C::MAXQ];
#pragma unroll
            for (int i = 0; i < C::MAXQ; ++i) {
                const int qd = tid + i * NT;
                if (qd < nq_old) {
                    const long long ta = t_end - 2LL * N + 4LL * qd;
                    wo[i] = __ldcg(reinterpret_cast<const float4*>(tk.xring + (ta & tk.rin_mask)));
                }
            }
#pragma unroll
            for (int i = 0; i < C::MAXQ; ++i) {
                const int qd = tid + i * NT;
                if (qd < nq_old) {
                    s[sidx<SW>(2 * qd)] = make_float2(wo[i].x, wo[i].y);
                    s[sidx<SW>(2 * qd + 1)] = make_float2(wo[i].z, wo[i].w);
                } else if (l0 && qd < nq) {   // append, read back from this thread's own writes
                    const long long ta = t_end - 2LL * N + 4LL * qd;
                    const float2 a = s[sidx<SW>(2 * qd)], bb = s[sidx<SW>(2 * qd + 1)];
                    *reinterpret_cast<float4*>(tk.xring + (ta & tk.rin_mask)) = make_float4(a.x, a.y, bb.x, bb.y);
                }
            }
        }
        __syncthreads();
        fft_smem<NT, C::MAXB, SW>(s, N, logN, tw, false);

        // ---- split, FDL MAC, inverse merge, operands streamed from L2 ----------
        auto finish_pair = [&](int k, float2 h0k, float2 h0nk, float2 ak, float2 ank) {
            const int nk = (k == 0) ? 0 : N - k;
            float2 xk, xnk;
            rfft_split<SW>(s[sidx<SW>(k)], s[sidx<SW>(nk)], k, logN, tw, xk, xnk);
            const int bk = k, bnk = N - k;   // k == 0 pairs bin 0 with bin N
            Xs[bk] = xk;
            if (bnk != bk) Xs[bnk] = xnk;
            const float2 yk = cadd(cmul(xk, h0k), ak);
            const float2 ynk = cadd(cmul(xnk, h0nk), ank);
            float2 zk, znk;
            irfft_merge<SW>(yk, ynk, k, logN, tw, zk, znk);
            s[sidx<SW>(k)] = zk;
            if (k != 0 && k != half) s[sidx<SW>(N - k)] = znk;
        };
        constexpr int CH = C::SPLIT_CH;
        for (int k0 = tid; k0 <= half; k0 += CH * NT) {
            float2 h0v[CH][2], av[CH][2];
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                const int k = k0 + u * NT;
                if (k <= half) {
                    const int bnk = N - k;
                    h0v[u][0] = __ldg(&tk.H[k]);
                    h0v[u][1] = __ldg(&tk.H[bnk]);
                    av[u][0] = make_float2(0.f, 0.f);
                    av[u][1] = av[u][0];
                    if (use_yp) {
                        av[u][0] = __ldcg(&Ypb[k]);
                        av[u][1] = __ldcg(&Ypb[bnk]);
                        for (int q = 1; q < npart; ++q) {
                            av[u][0] = cadd(av[u][0], __ldcg(&Ypb[q * rstride + k]));
                            av[u][1] = cadd(av[u][1], __ldcg(&Ypb[q * rstride + bnk]));
                        }
                    }
                    if (use_x1) {
                        av[u][0] = cadd(av[u][0], cmul(__ldcg(&X1[k]), __ldg(&tk.H[cs + k])));
                        av[u][1] = cadd(av[u][1], cmul(__ldcg(&X1[bnk]), __ldg(&tk.H[cs + bnk])));
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                const int k = k0 + u * NT;
                if (k <= half) finish_pair(k, h0v[u][0], h0v[u][1], av[u][0], av[u][1]);
            }
        }
        __syncthreads();
    }

    fft(true);

    const float* sf = reinterpret_cast<const float*>(s);   // y[i] = sf[i], i < 2N
    if (!l0) {
        // level block b covers output samples [b N, (b+1) N)
        const long long t0 = b * (long long)N;
        for (int i4 = tid; 4 * i4 < N; i4 += NT)
            *reinterpret_cast<float4*>(tk.yring + ((t0 + 4 * i4) & tk.rmask)) = ld_out4<SW>(s, i4);
        return;
    }

    // ---- level 0: emit this step's output ----------------------------------------
    float* out = rs.io.out + io_step * rs.io.out_step;
    const long long osamp = rs.io.out_sample, och = rs.io.out_ch;
    for (int i = tid; i < N0; i += NT) {
        float v = SW ? reinterpret_cast<const float*>(s + sidx<SW>(i >> 1))[i & 1] : sf[i];
        if (C::PREFETCH) {
            if (tk.M > 1) v += emit[i];
        } else {
            for (int L = 1; L < tk.M; ++L) {
                const float* yr = L <= kEmitLevels ? tk.eyring[L - 1] : bank.lv[tk.lv_index + L].yring;
                const int mk = L <= kEmitLevels ? tk.emask[L - 1] : bank.lv[tk.lv_index + L].rmask;
                v += __ldcg(&yr[(t_new + i) & mk]);
            }
        }
        if (tk.mix_mode == 1) out[i * osamp + (long long)tk.out_ch * och] = v;
        else if (tk.mix_mode == 2) tk.pcout[i] = v;
        for (int z = 0; z < tk.zero_outs; ++z) out[i * osamp + (long long)bank.zero_list[tk.zero_off + z] * och] = 0.0f;
    }
    if (tk.mix_mode == 2) mix_last(out, osamp, och);
}

// 16-byte global -> shared copies that bypass the registers (L2-cached)
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// Level 0 over K base blocks per step (bank.kb = K > 1; offline processing
// of many blocks per call): the CTA of one PC computes its blocks
// b = c .. c + K - 1.  Block b + t sums X_{b+t-p} H_p over the parts
// p < Q here (Q = min(P, the shared-memory cap) >= min(P, 2K), in the task's
// p_lo) -- p <= t from this CTA's own forward transforms, the others from
// the spectra ring -- and adds the partial-sum rows of the parts p >= Q that
// spread tasks built during the previous step (those read only spectra of
// blocks <= b - 1 since Q >= 2K).  Order: p ascending, then the rows in
// order.  The K forward and K inverse transforms run as one batched
// shared-memory FFT: a 256-point transform has 64 radix-4 butterflies per
// stage, so four of them fill a 256-thread CTA for the cost of one.
// Before the dependency wait the CTA reads only the call's input, twiddles
// and filter rows and writes only shared memory, like the one-block fire.
// ---------------------------------------------------------------------------
constexpr int kMaxStepSamples = 1024;   // K N0 at most
constexpr int kMaxStepBlocks = 4;       // K at most

// shared memory of fire_multi summing Q parts itself
__host__ __device__ constexpr size_t multi_smem_bytes(int N, int K, int Q) {
    // transform buffers 2 K N, twiddles N/2 (complex); filter rows Q, spectra
    // rows Q - 1 + K, sums K (rows of N + 2 complex); due output slices K N floats
    return (size_t)8 * (2 * (size_t)K * N + (size_t)N / 2 + (size_t)(2 * Q + 2 * K - 1) * (N + 2)) +
           (size_t)4 * K * N;
}
// shared memory that still lets two such CTAs share an SM
constexpr size_t kMultiSmemCap = 112 * 1024;
constexpr int kMaxMultiParts = 32;

template <class C>
__device__ __forceinline__ void fire_multi(const Bank& bank, const Task& tk, const RunState& rs, long long c,
                                           float2* smem, int* s_last) {
    constexpr int NT = C::NT;
    constexpr int MAXBB = (kMaxStepSamples / 4 + NT - 1) / NT;        // batched radix-4 butterflies per thread
    constexpr int MAXI = (kMaxStepSamples / 2 + 8 + NT - 1) / NT;     // (block, bin pair) items per thread
    constexpr int MAXW = (kMaxStepSamples / 4 + 128 + NT - 1) / NT;   // window quads per thread (K + 1 blocks)
    constexpr int MAXE = (kMaxStepSamples / 4 + NT - 1) / NT;         // output quads per thread
    const int tid = threadIdx.x;
    const int K = bank.kb;
    const int N = tk.N, logN = tk.logN, P = tk.P, cs = tk.cs;   // N = N0
    const int half = N >> 1, ncol = cs >> 1;                     // ncol = half + 1 bin pairs (float4) per row
    // item it < K half: block it >> (logN - 1), pair it & (half - 1); the
    // K items after that: pair `half` (bins N, N + 1; the split's k = N/2)
    const int nitem = K * half + K;
    auto item = [&](int it, int& t, int& col) {
        if (it < K * half) {
            t = it >> (logN - 1);
            col = it & (half - 1);
        } else {
            t = it - K * half;
            col = half;
        }
    };
    const int Q = tk.p_lo;                        // parts summed here: min(P, cap), >= min(P, 2K)
    const int nrows = P > Q ? tk.k0 : 0;          // partial-sum rows (parts >= Q)
    const int nbuf = 2 * K;                       // partial-sum buffers per row
    const long long io_step = c - rs.io.step0;
    c -= tk.origin;
    const long long b = c;                        // level-0 block of the first base block
    const int sold0 = (int)imod(b - (Q - 1), P);  // ring slot of the oldest spectrum read
    const int snew0 = (int)imod(b, P);            // ring slot of block b
    const float scale = tk.scale;
    float2* sb = smem;                                   // K N: transform data
    float2* sc = sb + (size_t)K * N;                     // K N: transform scratch
    float2* twt = sc + (size_t)K * N;                    // N/2 quarter-wave twiddles
    float2* hs = twt + half;                             // Q rows: H_0 .. H_{Q-1}
    float2* xs = hs + (size_t)Q * cs;                    // Q - 1 + K rows: row i holds block b - (Q - 1) + i
    float2* ys = xs + (size_t)(Q - 1 + K) * cs;          // K rows: Y of blocks b .. b + K - 1
    float* emit = reinterpret_cast<float*>(ys + (size_t)K * cs);   // K N0: other levels' due slices
    const Twiddles tw{twt, logN};
    // the K transforms, unrolled for the common base blocks
    auto fftb = [&](bool inv) -> float2* {
        switch (logN) {
            case 6: return fft_smem_batch_c<NT, MAXBB, 6>(sb, sc, K, twt, inv);
            case 7: return fft_smem_batch_c<NT, MAXBB, 7>(sb, sc, K, twt, inv);
            case 8: return fft_smem_batch_c<NT, MAXBB, 8>(sb, sc, K, twt, inv);
            case 9: return fft_smem_batch_c<NT, MAXBB, 9>(sb, sc, K, twt, inv);
            default: return fft_smem_batch<NT, MAXBB>(sb, sc, K, N, logN, tw, inv);
        }
    };
    const bool early = io_step >= 1;   // block c - 1 lies in this call's input too
    const int qpb = N >> 2;            // quads per base block
    const int nqw = (K + 1) * qpb;     // window: blocks c - 1 .. c + K - 1
    const long long isamp = rs.io.in_sample;
    const float* in0 = rs.io.in + (long long)tk.in_ch * rs.io.in_ch;
    auto X4 = [&](int row, int col) { return *reinterpret_cast<const float4*>(xs + (size_t)row * cs + 2 * col); };
    auto H4 = [&](int p, int col) { return *reinterpret_cast<const float4*>(hs + (size_t)p * cs + 2 * col); };
    // quad qd of window block bi (block c + bi - 1): second half of sub-block
    // bi - 1's window, first half of sub-block bi's
    auto place = [&](int qd, float4 v) {
        const int bi = qd >> (logN - 2), w = qd & (qpb - 1);
        if (bi < K) {
            sb[bi * N + 2 * w] = make_float2(v.x, v.y);
            sb[bi * N + 2 * w + 1] = make_float2(v.z, v.w);
        }
        if (bi >= 1) {
            sb[(bi - 1) * N + half + 2 * w] = make_float2(v.x, v.y);
            sb[(bi - 1) * N + half + 2 * w + 1] = make_float2(v.z, v.w);
        }
    };
    // rows [r0, r0 + n) of a ring starting at slot s0 (wrapping at P): two
    // contiguous runs; f(ring_row, first_local_row, rows)
    auto ring_runs = [&](int s0, int n, auto&& f) {
        const int n1 = min(n, P - s0);
        f(s0, 0, n1);
        if (n > n1) f(0, n1, n - n1);
    };

    // ---- static prologue: the call's input, twiddles, filter rows -----------------
    float4 wv[MAXW];
#pragma unroll
    for (int i = 0; i < MAXW; ++i) {
        const int qd = tid + i * NT;
        const int bi = qd >> (logN - 2);
        if (qd < nqw && (bi >= 1 || early)) {
            const float* src = in0 + (io_step + bi - 1) * rs.io.in_step + 4LL * (qd & (qpb - 1)) * isamp;
            wv[i] = make_float4(src[0] * scale, src[isamp] * scale, src[2 * isamp] * scale, src[3 * isamp] * scale);
        }
    }
    {
        const int sh = bank.wlog - (logN + 1);
        for (int m = tid; m < half; m += NT) {
            const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(twt + m));
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(bank.W + ((size_t)m << sh))
                         : "memory");
        }
        const float4* H4g = reinterpret_cast<const float4*>(tk.H);
        float4* hs4 = reinterpret_cast<float4*>(hs);
        for (int i = tid; i < Q * ncol; i += NT) cp_async16(hs4 + i, H4g + i);   // rows 0 .. Q-1 are contiguous
    }
#pragma unroll
    for (int i = 0; i < MAXW; ++i) {
        const int qd = tid + i * NT;
        if (qd < nqw && (qd >= qpb || early)) place(qd, wv[i]);
    }
    if (!early) {   // the call's first step: block c - 1 from the input ring
        cudaGridDependencySynchronize();
        if (tid < qpb) {
            const long long ta = (c - 1) * (long long)N + 4LL * tid;
            place(tid, __ldcg(reinterpret_cast<const float4*>(tk.xring + (ta & tk.rin_mask))));
        }
    }
    cp_async_wait_all();

    // ---- K forward transforms, X_{b+t} -> xs, X_{b+t} H_0 + ... + X_b H_t -> acc ------
    float4 acc[MAXI];
    {
        __syncthreads();
        const float2* r = fftb(false);
        for (int it = tid; it < nitem; it += NT) {
            int t, k;
            item(it, t, k);
            const float2* z = r + t * N;
            const int nk = (k == 0) ? 0 : N - k;
            float2 xk, xnk;
            rfft_split(z[k], z[nk], k, logN, tw, xk, xnk);
            float2* X = xs + (size_t)(Q - 1 + t) * cs;
            X[k] = xk;
            if (N - k != k) X[N - k] = xnk;
            if (k == 0) X[N + 1] = make_float2(0.f, 0.f);   // row padding
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < MAXI; ++i) {
            const int it = tid + i * NT;
            acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (it < nitem) {
                int t, col;
                item(it, t, col);
                for (int p = 0; p <= t && p < Q; ++p) acc[i] = f4mac(acc[i], X4(Q - 1 + t - p, col), H4(p, col));
            }
        }
    }
    if (early) cudaGridDependencySynchronize();

    // ---- dependent inputs: older spectra, partial sums, due output slices ---------
    ring_runs(sold0, Q - 1, [&](int s0, int r0, int n) {
        const float4* src = reinterpret_cast<const float4*>(tk.X + (size_t)s0 * cs);
        float4* dst = reinterpret_cast<float4*>(xs + (size_t)r0 * cs);
        for (int i = tid; i < n * ncol; i += NT) cp_async16(dst + i, src + i);
    });
    float4 ya[MAXI];
#pragma unroll
    for (int i = 0; i < MAXI; ++i) {
        const int it = tid + i * NT;
        if (nrows > 0 && it < nitem) {
            int t, col;
            item(it, t, col);
            const float4* y4 = reinterpret_cast<const float4*>(tk.Yp + (size_t)((b + t) & (nbuf - 1)) * cs + 2 * col);
            const size_t rstep = (size_t)nbuf * cs / 2;   // float4 per row
            ya[i] = __ldcg(y4);
            for (int q = 1; q < nrows; ++q) ya[i] = f4add(ya[i], __ldcg(y4 + q * rstep));
        }
    }
    const int Le = tk.M - 1 < kEmitLevels ? tk.M - 1 : kEmitLevels;
    const long long t_new = c * (long long)N;
    const int nq_out = (K * N) >> 2;
    {
        float4 ev[MAXE][kEmitLevels];
#pragma unroll
        for (int i = 0; i < MAXE; ++i) {
            const int e4 = tid + i * NT;
#pragma unroll
            for (int L = 0; L < kEmitLevels; ++L)
                if (L < Le && e4 < nq_out)
                    ev[i][L] = __ldcg(reinterpret_cast<const float4*>(tk.eyring[L] + ((t_new + 4 * e4) & tk.emask[L])));
        }
#pragma unroll
        for (int i = 0; i < MAXE; ++i) {
            const int e4 = tid + i * NT;
            if (e4 >= nq_out || tk.M < 2) continue;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int L = 0; L < kEmitLevels; ++L)
                if (L < Le) v = f4add(v, ev[i][L]);
            for (int L = kEmitLevels + 1; L < tk.M; ++L) {   // rare: more than 5 levels
                const DevLevel& l2 = bank.lv[tk.lv_index + L];
                v = f4add(v, __ldcg(reinterpret_cast<const float4*>(l2.yring + ((t_new + 4 * e4) & l2.rmask))));
            }
            *reinterpret_cast<float4*>(emit + 4 * e4) = v;
        }
    }
    // this step's input appended to the PC's ring (blocks c .. c + K - 1)
#pragma unroll
    for (int i = 0; i < MAXW; ++i) {
        const int qd = tid + i * NT;
        const int bi = qd >> (logN - 2);
        if (qd < nqw && bi >= 1) {
            const long long ta = (c + bi - 1) * (long long)N + 4LL * (qd & (qpb - 1));
            *reinterpret_cast<float4*>(tk.xring + (ta & tk.rin_mask)) = wv[i];
        }
    }
    cp_async_wait_all();
    __syncthreads();   // every thread's older-spectra copies have landed
    // the new spectra into the ring only now: a slot read above may be one of
    // them.  With fewer parts than blocks (one-level PCs) only the newest P
    // blocks keep a slot.
    {
        const int t_keep = K > P ? K - P : 0;
        int s0 = snew0 + t_keep;
        if (s0 >= P) s0 -= P;
        ring_runs(s0, K - t_keep, [&](int sr, int r0, int n) {
            float4* dst = reinterpret_cast<float4*>(tk.X + (size_t)sr * cs);
            const float4* src = reinterpret_cast<const float4*>(xs + (size_t)(Q - 1 + t_keep + r0) * cs);
            for (int i = tid; i < n * ncol; i += NT) dst[i] = src[i];
        });
    }
    // older spectra: the thread's items advance together over p (each still
    // sums p ascending), so their shared-memory loads overlap
    {
        int ti[MAXI], ci[MAXI];
#pragma unroll
        for (int i = 0; i < MAXI; ++i) {
            const int it = tid + i * NT;
            ti[i] = Q;   // no parts for an item beyond the end
            ci[i] = 0;
            if (it < nitem) item(it, ti[i], ci[i]);
        }
#pragma unroll 2
        for (int p = 1; p < Q; ++p) {
#pragma unroll
            for (int i = 0; i < MAXI; ++i)
                if (p > ti[i]) acc[i] = f4mac(acc[i], X4(Q - 1 + ti[i] - p, ci[i]), H4(p, ci[i]));
        }
#pragma unroll
        for (int i = 0; i < MAXI; ++i) {
            if (tid + i * NT >= nitem) continue;
            float4 a = acc[i];
            if (nrows > 0) a = f4add(a, ya[i]);
            *reinterpret_cast<float4*>(ys + (size_t)ti[i] * cs + 2 * ci[i]) = a;
        }
    }
    __syncthreads();
    for (int it = tid; it < nitem; it += NT) {   // inverse pre-pass into sb
        int t, k;
        item(it, t, k);
        const float2* Y = ys + (size_t)t * cs;
        float2 zk, znk;
        irfft_merge(Y[k], Y[N - k], k, logN, tw, zk, znk);
        float2* s = sb + t * N;
        s[k] = zk;
        if (k != 0 && k != half) s[N - k] = znk;
    }
    __syncthreads();
    const float* yo = reinterpret_cast<const float*>(fftb(true));

    // ---- output: K base blocks, each the first N samples of its inverse --------------
    float* out = rs.io.out + io_step * rs.io.out_step;
    const long long osamp = rs.io.out_sample, och = rs.io.out_ch;
    const int KN = K * N;
    float* orow = out + (long long)tk.out_ch * och;
    if (tk.mix_mode == 1 && tk.zero_outs == 0 && osamp == 1 && (rs.io.out_step & 3) == 0 &&
        (reinterpret_cast<uintptr_t>(orow) & 15) == 0) {   // contiguous channel rows: float4 stores
        for (int i4 = tid; 4 * i4 < KN; i4 += NT) {
            const int i = 4 * i4, t = i >> logN, j = i & (N - 1);
            float4 v = *reinterpret_cast<const float4*>(yo + (size_t)t * 2 * N + j);
            if (tk.M > 1) v = f4add(v, *reinterpret_cast<const float4*>(emit + i));
            *reinterpret_cast<float4*>(orow + t * rs.io.out_step + j) = v;
        }
        return;
    }
    for (int i = tid; i < KN; i += NT) {
        const int t = i >> logN, j = i & (N - 1);
        float v = yo[(size_t)t * 2 * N + j];
        if (tk.M > 1) v += emit[i];
        const long long o = t * rs.io.out_step + j * osamp;
        if (tk.mix_mode == 1) out[o + (long long)tk.out_ch * och] = v;
        else if (tk.mix_mode == 2) tk.pcout[i] = v;
        for (int z = 0; z < tk.zero_outs; ++z) out[o + (long long)bank.zero_list[tk.zero_off + z] * och] = 0.0f;
    }
    if (tk.mix_mode != 2) return;
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const int o = tk.out_ch;
        const int cnt = bank.out_off[o + 1] - bank.out_off[o];
        *s_last = (atomicAdd(&bank.mix_cnt[o], 1) == cnt - 1);
    }
    __syncthreads();
    if (!*s_last) return;
    __threadfence();
    const int o = tk.out_ch;
    const int j0 = bank.out_off[o], j1 = bank.out_off[o + 1];
    for (int i = tid; i < KN; i += NT) {
        const int t = i >> logN, j = i & (N - 1);
        float v = 0.0f;
        for (int jj = j0; jj < j1; ++jj) v += __ldcg(&bank.pcs[bank.out_pcs[jj]].pcout[i]);
        out[t * rs.io.out_step + j * osamp + (long long)o * och] = v;
    }
    if (tid == 0) bank.mix_cnt[o] = 0;
}

// ---------------------------------------------------------------------------
// The step kernel: CTA i runs task i of this step's task list.
// ---------------------------------------------------------------------------
// MULTI: the bank runs several base blocks per step (level-0 fires take
// fire_multi); a separate instance so the one-block kernel keeps its registers.
// LANES: threads per spread part-group (bins per spread task / 2), the tile
// width of the handle, one instance per width.
template <class C, bool MULTI = false, int LANES = 64>
__global__ void __launch_bounds__(C::NT, C::PREFETCH ? 3 : 1) step_kernel(Bank bank, const Task* __restrict__ tasks, RunState rs_val,
                                                     const RunState* rs_dev, int step_in_batch) {
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(16) Task tk;
    __shared__ __align__(16) RunState rs;
    __shared__ int s_last;
    const int tid = threadIdx.x;
    // the next step's CTAs may start their independent part now; they wait in
    // cudaGridDependencySynchronize() until this grid has completed
    cudaTriggerProgrammaticLaunchCompletion();
    if (tid < 12) {
        reinterpret_cast<int4*>(&tk)[tid] = __ldg(reinterpret_cast<const int4*>(tasks + blockIdx.x) + tid);
    } else if (tid >= 32 && tid < 37) {
        const int j = tid - 32;
        if (rs_dev) reinterpret_cast<int4*>(&rs)[j] = __ldcg(reinterpret_cast<const int4*>(rs_dev) + j);
    }
    if (!rs_dev && tid == 64) rs = rs_val;
    __syncthreads();
    const long long c = rs.step_base + step_in_batch;
    const int kb = MULTI ? bank.kb : 1;
    if (tk.kind == 1) {
        cudaGridDependencySynchronize();
        if constexpr (MULTI) {
            if (tk.T == 1) {   // level 0: the next step's kb blocks in one task
                if (kb == 2) spread_multi<C::NT, 2>(tk, c, dyn_smem);
                else spread_multi<C::NT, 4>(tk, c, dyn_smem);
                return;
            }
        }
        spread_lanes<C::NT, (LANES < C::NT ? LANES : C::NT)>(tk, c, dyn_smem, kb);
        return;
    }
    if constexpr (MULTI && C::PREFETCH) {
        if (tk.T == 1) {
            fire_multi<C>(bank, tk, rs, c, reinterpret_cast<float2*>(dyn_smem), &s_last);
            return;
        }
    }
    fire_body<C, true>(bank, tk, rs, c, reinterpret_cast<float2*>(dyn_smem), &s_last);
}

// ---------------------------------------------------------------------------
// Serving pool: PCs join and leave between steps, so instead of per-phase
// task lists every CTA maps to one (descriptor, sub-task) pair of a map that
// changes only on admission or release.  Sub-task 0 fires the descriptor's
// level when its block completes at this step; sub-task s >= 1 is the s-th
// bin tile of the level's spread slice for this step (level 0: all bins,
// parts >= 2; level L: slice (phase - 1) of T_L - 1, parts >= 1).  Tiles or
// fires with nothing to do this step return at once.
// ---------------------------------------------------------------------------
template <class C>
__global__ void __launch_bounds__(C::NT) pool_kernel(Bank bank, const Task* __restrict__ slots,
                                                     const PoolCta* __restrict__ map, RunState rs_val) {
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(16) Task tk;
    __shared__ __align__(16) RunState rs;
    __shared__ int s_last;
    const int tid = threadIdx.x;
    const PoolCta pm = map[blockIdx.x];
    if (tid < 12) reinterpret_cast<int4*>(&tk)[tid] = __ldg(reinterpret_cast<const int4*>(slots + pm.slot) + tid);
    if (tid == 64) rs = rs_val;
    __syncthreads();
    const long long c = rs.step_base;
    const long long cl = c - tk.origin;   // the PC's own step count
    if (!tk.active || cl < 0) return;
    const long long q = cl + 1 + tk.s_blocks;
    if (pm.sub == 0) {
        if (q % tk.T != 0) return;
        fire_body<C, false>(bank, tk, rs, c, reinterpret_cast<float2*>(dyn_smem), &s_last);
        return;
    }
    int lo, hi, p_lo;
    if (tk.T == 1) {
        if (tk.P < 3) return;
        lo = 0;
        hi = tk.cs;
        p_lo = 2;
    } else {
        if (tk.P < 2) return;
        const int phi = (int)(q % tk.T);
        if (phi == 0) return;
        const int j = phi - 1, nch = tk.T - 1;
        lo = (int)(((long long)j * tk.cs / nch) & ~1LL);
        hi = (j == nch - 1) ? tk.cs : (int)(((long long)(j + 1) * tk.cs / nch) & ~1LL);
        p_lo = 1;
    }
    const int k0 = lo + (pm.sub - 1) * kSpreadBins;
    if (k0 >= hi) return;
    __syncthreads();   // everyone has read the fire form of the record
    if (tid == 0) {
        tk.kind = 1;
        tk.k0 = k0;
        tk.k1 = min(hi, k0 + kSpreadBins);
        tk.M = 0;        // default bins per task
        tk.p_lo = p_lo;
        tk.in_ch = 0;    // all parts from p_lo
        tk.out_ch = 0;   // partial-sum row 0
    }
    __syncthreads();
    spread_body<C::NT>(tk, c, dyn_smem, 1);
}

cudaError_t launch_pool_class(int cls, int grid, int maxN, const Bank& bank, const Task* slots, const PoolCta* map,
                              const RunState& rs, cudaStream_t st) {
    if (grid <= 0) return cudaSuccess;
    const size_t smem = class_smem_bytes(cls, maxN);
    switch (cls) {
        case 0: pool_kernel<Cls0><<<grid, Cls0::NT, smem, st>>>(bank, slots, map, rs); break;
        case 1: pool_kernel<Cls1><<<grid, Cls1::NT, smem, st>>>(bank, slots, map, rs); break;
        default: pool_kernel<Cls2><<<grid, Cls2::NT, smem, st>>>(bank, slots, map, rs); break;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Filter spectra: H = rfft([0_N, h_row]) / 2N for one row per CTA.
// ---------------------------------------------------------------------------
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) spectra_kernel(const SpectraJob* __restrict__ jobs, const float2* W,
                                                     int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    const SpectraJob jb = jobs[blockIdx.x];
    const int N = jb.N;
    float2* twt = s + N;
    const int tid = threadIdx.x;
    // window [0_N, h[0..N)]: complex pair n holds samples 2n, 2n+1
    for (int n = tid; n < N; n += NT) {
        float a = 0.f, b = 0.f;
        const int i = 2 * n - N;
        if (i >= 0) {
            if (i < jb.len) a = jb.src[i];
            if (i + 1 < jb.len) b = jb.src[i + 1];
        }
        s[n] = make_float2(a, b);
    }
    load_twiddles<NT>(twt, jb.logN, W, wlog);
    __syncthreads();
    const Twiddles tw{twt, jb.logN};
    fft_smem<NT, MAXB>(s, N, jb.logN, tw, false);
    const float inv = 1.0f / (float)(2 * N);
    const int half = N >> 1;
    for (int k = tid; k <= half; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, jb.logN, tw, xk, xnk);
        jb.dst[k] = make_float2(xk.x * inv, xk.y * inv);
        if (N - k != k) jb.dst[N - k] = make_float2(xnk.x * inv, xnk.y * inv);
    }
}

// Spread tasks of levels >= 1 with several base blocks per step: their own
// launch beside the step chain (they feed only the levels' deferred fires).
constexpr int kSideNT = 256;
__global__ void __launch_bounds__(kSideNT) spread_kernel(const Task* __restrict__ tasks, RunState rs_val,
                                                        const RunState* rs_dev, int step_in_batch) {
    __shared__ float4 red[kSideNT];
    __shared__ __align__(16) Task tk;
    __shared__ long long step_base;
    const int tid = threadIdx.x;
    if (tid < 12) reinterpret_cast<int4*>(&tk)[tid] = __ldg(reinterpret_cast<const int4*>(tasks + blockIdx.x) + tid);
    if (tid == 32) step_base = rs_dev ? __ldcg(&rs_dev->step_base) : rs_val.step_base;
    __syncthreads();
    spread_body<kSideNT>(tk, step_base + step_in_batch, red, 1);
}

cudaError_t launch_side_spreads(int grid, const Task* tasks, const RunState& rs, const RunState* rs_dev,
                                int step_in_batch, cudaStream_t st) {
    if (grid <= 0) return cudaSuccess;
    spread_kernel<<<grid, kSideNT, 0, st>>>(tasks, rs, rs_dev, step_in_batch);
    return cudaGetLastError();
}

__global__ void set_state_kernel(RunState* dst, RunState v) { *dst = v; }

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
int fire_class_of(int N) { return N <= Cls0::MAXN ? 0 : (N <= Cls1::MAXN ? 1 : (N <= Cls2::MAXN ? 2 : 3)); }
static_assert(Cls2::MAXN == kMaxBlockOneCta, "class 2 is the largest one-CTA class");

static const int kNT[3] = {Cls0::NT, Cls1::NT, Cls2::NT};
static const bool kPrefetch[3] = {Cls0::PREFETCH, Cls1::PREFETCH, Cls2::PREFETCH};
int class_threads(int cls) { return cls == 3 ? 512 : kNT[cls]; }
int spread_task_bins() { return kSpreadBins; }
int spread_task_parts() { return kSpreadParts; }
bool spread_bins_ok(int bins) { return bins == 64 || bins == 128 || bins == 256 || bins == 512; }

size_t class_smem_bytes(int cls, int maxN) {
    if (cls == 3) return cluster_smem_bytes();
    size_t b = fire_smem_bytes(maxN, kPrefetch[cls]);
    const size_t red = sizeof(float4) * (size_t)kNT[cls];   // spread part-group partials
    return b > red ? b : red;
}

size_t step_smem_bytes(int cls, int maxN, const Bank& bank) {
    size_t b = class_smem_bytes(cls, maxN);
    if (cls == 0 && bank.kb > 1) b = std::max(b, multi_smem_bytes(bank.N0, bank.kb, bank.kq));
    return b;
}

int multi_fire_parts(int N0, int K) {
    int q = 2 * K;
    while (q < kMaxMultiParts && multi_smem_bytes(N0, K, q + 1) <= kMultiSmemCap) ++q;
    return q;
}

int max_step_blocks(int N0) {
    if (N0 < 16 || N0 > Cls0::MAXN) return 1;
    int k = 1;
    while (2 * k * N0 <= kMaxStepSamples && 2 * k <= kMaxStepBlocks) k *= 2;
    return k;
}

cudaError_t prepare_kernels() {
    cudaError_t e = prepare_cluster_kernels();
    if (e != cudaSuccess) return e;
    size_t s0 = class_smem_bytes(0, Cls0::MAXN);
    for (int N = 16; N <= Cls0::MAXN; N *= 2)
        for (int k = 2; k <= max_step_blocks(N); k *= 2) s0 = std::max(s0, multi_smem_bytes(N, k, multi_fire_parts(N, k)));
    for (auto fn : {step_kernel<Cls0>, step_kernel<Cls0, false, 32>, step_kernel<Cls0, false, 128>,
                    step_kernel<Cls0, false, 256>}) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)class_smem_bytes(0, Cls0::MAXN));
        if (e != cudaSuccess) return e;
    }
    e = cudaFuncSetAttribute(step_kernel<Cls0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s0);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(step_kernel<Cls1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)std::max(class_smem_bytes(1, Cls1::MAXN), kWholeSmSmem));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(step_kernel<Cls2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)std::max(class_smem_bytes(2, Cls2::MAXN), kWholeSmSmem));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(spectra_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(12 * 16384));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pool_kernel<Cls0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)class_smem_bytes(0, Cls0::MAXN));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pool_kernel<Cls1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)class_smem_bytes(1, Cls1::MAXN));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pool_kernel<Cls2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)class_smem_bytes(2, Cls2::MAXN));
    return e;
}

cudaError_t launch_step_class(int cls, int grid, int maxN, const Bank& bank, const Task* tasks, const RunState& rs,
                              const RunState* rs_dev, int step_in_batch, cudaStream_t st, bool pdl, int prio,
                              bool whole_sm) {
    if (grid <= 0) return cudaSuccess;
    if (cls == 3) return launch_cluster_fire(grid, bank, tasks, rs, rs_dev, step_in_batch, st, pdl, prio);
    static int least = 0, greatest = 0;
    static const bool have_range = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess;
    // programmatic dependent launch: this step's CTAs may be scheduled while
    // the previous step kernel in the stream finishes (their static prologue
    // reads only data no step writes; see cudaGridDependencySynchronize).
    // Callers pass pdl = false when the preceding work is anything else.
    // A priority lets the block scheduler place the step chain's CTAs ahead
    // of deferred fires that run beside it.
    cudaLaunchAttribute attr[2];
    int na = 0;
    if (pdl) {
        attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if (prio != 0 && have_range) {
        attr[na].id = cudaLaunchAttributePriority;
        attr[na].val.priority = prio > 0 ? greatest : least;
        ++na;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kNT[cls]);
    cfg.dynamicSmemBytes = step_smem_bytes(cls, maxN, bank);
    if (whole_sm && cls != 0) cfg.dynamicSmemBytes = std::max(cfg.dynamicSmemBytes, kWholeSmSmem);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = na;
    switch (cls) {
        case 0:
            if (bank.kb > 1) return cudaLaunchKernelEx(&cfg, step_kernel<Cls0, true>, bank, tasks, rs, rs_dev, step_in_batch);
            switch (bank.tb) {   // the handle's spread tile width
                case 64: return cudaLaunchKernelEx(&cfg, step_kernel<Cls0, false, 32>, bank, tasks, rs, rs_dev, step_in_batch);
                case 256: return cudaLaunchKernelEx(&cfg, step_kernel<Cls0, false, 128>, bank, tasks, rs, rs_dev, step_in_batch);
                case 512: return cudaLaunchKernelEx(&cfg, step_kernel<Cls0, false, 256>, bank, tasks, rs, rs_dev, step_in_batch);
                default: return cudaLaunchKernelEx(&cfg, step_kernel<Cls0>, bank, tasks, rs, rs_dev, step_in_batch);
            }
        case 1: return cudaLaunchKernelEx(&cfg, step_kernel<Cls1>, bank, tasks, rs, rs_dev, step_in_batch);
        default: return cudaLaunchKernelEx(&cfg, step_kernel<Cls2>, bank, tasks, rs, rs_dev, step_in_batch);
    }
}

cudaError_t launch_spectra(int cls, int njobs, int maxN, const SpectraJob* jobs, const float2* W, int wlog,
                           cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    if (cls == 3) return launch_cluster_spectra(njobs, jobs, W, wlog, st);
    const size_t smem = (size_t)12 * maxN;
    switch (cls) {
        case 0: spectra_kernel<128, 2><<<njobs, 128, smem, st>>>(jobs, W, wlog); break;
        case 1: spectra_kernel<256, 4><<<njobs, 256, smem, st>>>(jobs, W, wlog); break;
        default: spectra_kernel<512, 8><<<njobs, 512, smem, st>>>(jobs, W, wlog); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_set_state(RunState* dst, const RunState& v, cudaStream_t st) {
    set_state_kernel<<<1, 1, 0, st>>>(dst, v);
    return cudaGetLastError();
}

}  // namespace pcg
