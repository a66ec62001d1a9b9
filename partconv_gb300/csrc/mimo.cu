// mimo.cu -- n_in x n_out MIMO partitioned convolution with per-bin channel
// sums: y_o = sum_i x_i * h_{i,o} over every (input, output) path.
//
// The reference would run one PartConvFilter per path and sum the outputs in
// time (src/partconvMulti.cpp:911-921), recomputing each input's spectrum for
// every output.  Here every input's block spectrum is computed once per
// level block and each output's FDL sums over inputs per bin:
//   Y_o[k] = sum_i sum_p X_i[b-p][k] H_{i,o,p}[k],
// followed by one inverse FFT per output and level block.  The level
// schedule is the engine's minimum-latency one (matlab/MFDL_part_conv.m
// structure; layouts must pass its relaxed check).
//
// A base step is three kernels (programmatic dependent launches):
//   K1 input FFTs     -- every (input, level) whose block completes: window,
//                        real FFT, spectrum ring slot b mod P (level 0 also
//                        appends the step's samples to the input ring);
//   K2 MAC tasks      -- fire sums for the (output, level) blocks due now:
//                        Yf_o = sum_i X_i[b] H_{i,o,0} (+ X_i[b-1] H_{i,o,1}
//                        for level 0) + the partial sums; and spread tasks
//                        that build the partial sums over the older parts for
//                        later blocks, split by output, bin tile and input
//                        range (reduced in a fixed order when consumed);
//   K3 output IFFTs   -- inverse FFT of Yf_o, output ring (levels >= 1) or
//                        the step's output: level 0 plus the due slices of
//                        the other levels, in level order.
// H is streamed once per block: the MAC is bound by HBM bandwidth.  It is
// stored tile-major, [output][bin tile][input][part][bins of the tile], with
// each level's bins cut into fixed tiles (the bin slices the MAC tasks take),
// so one MAC task streams one contiguous range of H (about 40 KB: its inputs'
// rows of the tile, parts adjacent, in the order it sums them) instead of a
// 0.4 KB segment of every (input, part) row.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/partconv_gb300.h"
#include "engine_types.h"
#include "fft_smem.cuh"
#include "kernels.h"

using namespace pcg;

namespace {

constexpr int kWlog = 15;
constexpr int kMacNT = 128;        // MAC CTA: threads = (bin-pair column, term group) pairs
constexpr int kMacMaxBins = 128;   // widest bin tile (64 columns of two bins: two term groups)
constexpr int kMaxMimoLevels = 8;
constexpr int kMaxMacTerms = 2048;  // (input, part) terms one MAC task sums

struct MLevel {
    int N, logN, P, T, s_blocks, cs, rmask, npart;
    int ntile;           // bin tiles of a row
    const int* tstart;   // [ntile + 1]: first bin of each tile (the last entry is cs)
    float2* H;      // [nO][tile][nI][P][tile width]
    float2* X;      // [nI][P][cs]
    float2* Yp;     // [nO][npart][2][cs]
    float2* Yf;     // [nO][cs]
    float* yring;   // [nO][rmask + 1]
};

struct MBank {
    const float2* W;
    int wlog, N0, nI, nO, M, pad;
    MLevel lv[kMaxMimoLevels];
};

// one task of one stage; kind: 0 input FFT, 1 fire sum, 2 spread, 3 output IFFT
struct MTask {
    int kind, level, ch, k0;
    int k1, i0, i1, part;
};

__device__ __forceinline__ long long imod(long long a, long long m) {
    long long r = a % m;
    return r < 0 ? r + m : r;
}
__device__ __forceinline__ float4 f4mac(float4 acc, float4 x, float4 h) {
    acc.x += x.x * h.x - x.y * h.y;
    acc.y += x.x * h.y + x.y * h.x;
    acc.z += x.z * h.z - x.w * h.w;
    acc.w += x.z * h.w + x.w * h.z;
    return acc;
}
__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// L2 eviction policy for a MAC task's filter rows: the level-0 rows (read
// every base step) are evicted last, the larger levels' rows, which stream
// through once per level block, first
__device__ __forceinline__ unsigned long long l2_policy(bool keep) {
    unsigned long long p;
    if (keep)
        asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    else
        asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// 16-byte read-only load with an L2 cache policy, not kept in L1
__device__ __forceinline__ float4 ld_policy(const float4* ptr, unsigned long long pol) {
    float4 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(ptr), "l"(pol));
    return v;
}

__device__ __forceinline__ long long block_of(const MLevel& l, long long c) {   // newest block fired by step c
    return (c + 1 + l.s_blocks) / l.T - 1;
}

// ---------------------------------------------------------------------------
// K1: input FFTs
// ---------------------------------------------------------------------------
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) mimo_xfft_kernel(const MBank* __restrict__ bank_p, const MTask* __restrict__ tasks,
                                                       RunState rs, float* __restrict__ xring, int rin_mask) {
    extern __shared__ float4 dyn_smem[];
    cudaTriggerProgrammaticLaunchCompletion();
    const MBank& bank = *bank_p;
    const MTask t = tasks[blockIdx.x];
    const MLevel& l = bank.lv[t.level];
    const int N = l.N, logN = l.logN, tid = threadIdx.x, N0 = bank.N0;
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const long long c = rs.step_base;
    const long long t_new = c * (long long)N0, t_end = t_new + N0;
    const float* in = rs.io.in + (c - rs.io.step0) * rs.io.in_step + (long long)t.ch * rs.io.in_ch;
    float* xr = xring + (size_t)t.ch * (rin_mask + 1);
    load_twiddles<NT>(twt, logN, bank.W, bank.wlog);
    const long long isamp = rs.io.in_sample;
    const long long b = block_of(l, c);
    float2* Xs = l.X + ((size_t)t.ch * l.P + (size_t)imod(b, l.P)) * l.cs;
    // A window that lies wholly in this call's input is transformed before
    // the dependency wait (it reads only the input), its spectrum held in
    // registers until after the wait, when the spectrum ring may be written.
    constexpr int KMAX = 2 * MAXB + 1;   // bin pairs per thread (N <= 4 NT MAXB)
    const bool early = MAXB <= 2 && (c - rs.io.step0) * N0 >= 2LL * N - N0;
    float2 xk_r[MAXB <= 2 ? KMAX : 1][2];
    if constexpr (MAXB <= 2) {
        if (early) {
            for (int n = tid; n < N; n += NT) {
                const long long j = t_end - 2LL * N + 2LL * n - t_new;   // may be negative: earlier blocks
                s[n] = make_float2(in[j * isamp], in[(j + 1) * isamp]);
            }
            __syncthreads();
            const Twiddles tw{twt, logN};
            fft_smem<NT, MAXB>(s, N, logN, tw, false);
#pragma unroll
            for (int q = 0; q < KMAX; ++q) {
                const int k = tid + q * NT;
                if (k <= N / 2) rfft_split(s[k], s[k == 0 ? 0 : N - k], k, logN, tw, xk_r[q][0], xk_r[q][1]);
            }
        }
    }
    cudaGridDependencySynchronize();
    if constexpr (MAXB <= 2) {
        if (early) {
#pragma unroll
            for (int q = 0; q < KMAX; ++q) {
                const int k = tid + q * NT;
                if (k <= N / 2) {
                    Xs[k] = xk_r[q][0];
                    if (N - k != k) Xs[N - k] = xk_r[q][1];
                }
            }
            if (t.level == 0)   // the ring keeps the input history for later calls
                for (int i = tid; i < N0; i += NT) xr[(t_new + i) & rin_mask] = in[i * isamp];
            return;
        }
    }
    for (int n = tid; n < N; n += NT) {
        const long long ta = t_end - 2LL * N + 2LL * n;
        float a, bb;
        if (ta >= t_new) {
            const long long j = ta - t_new;
            a = in[j * isamp];
            bb = in[(j + 1) * isamp];
            if (t.level == 0) {
                xr[ta & rin_mask] = a;
                xr[(ta + 1) & rin_mask] = bb;
            }
        } else {
            a = __ldcg(&xr[ta & rin_mask]);
            bb = __ldcg(&xr[(ta + 1) & rin_mask]);
        }
        s[n] = make_float2(a, bb);
    }
    __syncthreads();
    const Twiddles tw{twt, logN};
    fft_smem<NT, MAXB>(s, N, logN, tw, false);
    for (int k = tid; k <= N / 2; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, logN, tw, xk, xnk);
        Xs[k] = xk;
        if (N - k != k) Xs[N - k] = xnk;
    }
}

// ---------------------------------------------------------------------------
// K2: MAC tasks (fire sums and spread partial sums)
//
// Measured on the 64 x 64 workload (us per launch): this kernel 30.7; with
// at most four term groups of 32 columns (a third of the threads idle on
// 44-bin tiles) 31.0; with the row-major H before the tile-major one 32.5.
// Rejected:
//   * H streamed into shared memory by cp.async stages (4 x 8 KB per CTA, no
//     registers held by the copies): 67 -- the input-spectrum loads became a
//     chain of round trips per stage, behind two barriers each;
//   * a task's whole H tile copied into shared memory by cp.async before the
//     grid dependency wait, input spectra through registers one batch ahead:
//     46.6-48.6 -- 46 KB per CTA leaves four CTAs per SM, and each CTA's
//     input-spectrum round trips start only once its tile has landed;
//   * four outputs per task, one input-spectrum load feeding four filter
//     loads (twice the filter bytes in flight per thread, a quarter of the
//     CTAs): 32.4;
//   * terms in part-major order (consecutive inputs of one part; input
//     spectra then far apart): 35.1;
//   * the filter loads as ld.global.nc.L1::no_allocate with a 128- or
//     256-byte L2 prefetch size instead of __ldcs: 30.49 against 30.51;
//   * 256-thread CTAs (four per SM): 31.4; 64-thread CTAs: 47.8.
//   * the larger levels' tasks first in the launch (level 0's last): 30.6;
//   * input spectra through L1 (__ldg): 28.2 against 28.5, not worth relying
//     on the read-only path for data the previous kernel wrote;
//   * (probes) level-0 tasks alone 16.2, level-1 tasks alone 21.4, and 21.7
//     with the level-1 filter loads at the addresses of an interleaved
//     [term][task][column] layout: DRAM page locality is not what limits it.
// Kept: the level-0 filter rows (68 MB, read every base step) loaded with an
// L2 evict-last policy and the larger levels' rows with evict-first, so more
// of the level-0 rows survive in L2 between steps: 30.5 -> 28.5 (evict-normal
// for level 0: 28.8).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMacNT, 8) mimo_mac_kernel(const MBank* __restrict__ bank_p,
                                                          const MTask* __restrict__ tasks, RunState rs) {
    __shared__ float4 red[kMacNT];
    cudaTriggerProgrammaticLaunchCompletion();
    const MBank& bank = *bank_p;
    const MTask t = tasks[blockIdx.x];
    const MLevel& l = bank.lv[t.level];
    // ncol bin-pair columns (a float4 each) x G term groups; consecutive
    // threads walk a row of the tile, then the next term's row, which
    // follows it in memory
    const int ncol = (t.k1 - t.k0) >> 1;
    const int G = kMacNT / ncol;
    const int lane = threadIdx.x % ncol, g = threadIdx.x / ncol;
    const int k = t.k0 + 2 * lane;
    const bool active = g < G;
    const int o = t.ch, P = l.P, cs = l.cs, nI = bank.nI;
    const long long c = rs.step_base;

    // (input, part) iteration space
    long long bt;
    int p_lo, np, i0, ni;
    if (t.kind == 1) {   // fire sum: parts 0 (and 1 for level 0) of the block due now
        bt = block_of(l, c);
        p_lo = 0;
        np = (l.T == 1 && P >= 2) ? 2 : 1;
        i0 = 0;
        ni = nI;
    } else {             // spread: parts p >= p_lo of a later block
        bt = (l.T == 1) ? c + 1 : (c + 1 + l.s_blocks) / l.T;
        p_lo = (l.T == 1) ? 2 : 1;
        np = P - p_lo;
        i0 = t.i0;
        ni = t.i1 - t.i0;
    }
    const int J = ni * np;
    // row offsets (in float4 units) of every (input, part) term, computed
    // once per CTA so the streaming loop carries no index arithmetic
    __shared__ int xoff[kMaxMacTerms], hoff[kMaxMacTerms];
    const int slot_bt = (int)imod(bt, P);
    for (int j = threadIdx.x; j < J; j += kMacNT) {
        const int i = i0 + j / np;
        const int p = p_lo + j % np;
        int sl = slot_bt - p;
        if (sl < 0) sl += P;
        xoff[j] = ((i * P + sl) * cs) >> 1;
        hoff[j] = ((i * P + p) * (t.k1 - t.k0)) >> 1;
    }
    __syncthreads();
    // the tables depend only on the task and the step: built before the
    // wait for the input spectra of this step
    cudaGridDependencySynchronize();
    // this task's tile of H: [input][part][width] at o nI P cs + k0 nI P
    const float4* H4 = reinterpret_cast<const float4*>(l.H + (size_t)o * nI * P * cs + (size_t)t.k0 * nI * P + (k - t.k0));
    const float4* X4 = reinterpret_cast<const float4*>(l.X + k);
    const unsigned long long hpol = l2_policy(t.level == 0);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        // eight 128-thread CTAs per SM (64 registers): more, smaller CTAs in
        // flight hide HBM latency better than deeper per-thread unrolling
        constexpr int U = 4;
        for (int j0 = g; j0 < J; j0 += U * G) {
            float4 xv[U], hv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u * G;
                if (j < J) {
                    xv[u] = __ldcg(X4 + xoff[j]);
                    hv[u] = ld_policy(H4 + hoff[j], hpol);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (j0 + u * G < J) acc = f4mac(acc, xv[u], hv[u]);
        }
    }
    if (g > 0 && active) red[(g - 1) * ncol + lane] = acc;
    __syncthreads();
    if (g != 0) return;
    for (int j = 1; j < G; ++j) acc = f4add(acc, red[(j - 1) * ncol + lane]);
    if (t.kind == 1) {
        const bool has_spread = (l.T == 1) ? P >= 3 : P >= 2;
        if (has_spread) {
            const int buf = (l.T == 1) ? (int)(bt & 1) : 0;
            for (int q = 0; q < l.npart; ++q)
                acc = f4add(acc, __ldcg(reinterpret_cast<const float4*>(
                                     l.Yp + (((size_t)o * l.npart + q) * 2 + buf) * cs + k)));
        }
        *reinterpret_cast<float4*>(l.Yf + (size_t)o * cs + k) = acc;
    } else {
        const int buf = (l.T == 1) ? (int)(bt & 1) : 0;
        *reinterpret_cast<float4*>(l.Yp + (((size_t)o * l.npart + t.part) * 2 + buf) * cs + k) = acc;
    }
}

// ---------------------------------------------------------------------------
// K3: output IFFTs and the step's output
// ---------------------------------------------------------------------------
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) mimo_yifft_kernel(const MBank* __restrict__ bank_p,
                                                        const MTask* __restrict__ tasks, RunState rs) {
    extern __shared__ float4 dyn_smem[];
    cudaTriggerProgrammaticLaunchCompletion();
    const MBank& bank = *bank_p;
    const MTask t = tasks[blockIdx.x];
    const MLevel& l = bank.lv[t.level];
    const int N = l.N, logN = l.logN, tid = threadIdx.x, N0 = bank.N0, o = t.ch;
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    load_twiddles<NT>(twt, logN, bank.W, bank.wlog);
    cudaGridDependencySynchronize();
    __syncthreads();
    const Twiddles tw{twt, logN};
    const float2* Y = l.Yf + (size_t)o * l.cs;
    for (int k = tid; k <= N / 2; k += NT) {
        float2 zk, znk;
        irfft_merge(__ldcg(&Y[k]), __ldcg(&Y[N - k]), k, logN, tw, zk, znk);
        s[k] = zk;
        if (k != 0 && k != N / 2) s[N - k] = znk;
    }
    __syncthreads();
    fft_smem<NT, MAXB>(s, N, logN, tw, true);
    const float* sf = reinterpret_cast<const float*>(s);
    const long long c = rs.step_base;
    if (t.level > 0) {
        const long long t0 = block_of(l, c) * (long long)N;
        float* yr = l.yring + (size_t)o * (l.rmask + 1);
        for (int i = tid; i < N; i += NT) yr[(t0 + i) & l.rmask] = sf[i];
        return;
    }
    const long long t_new = c * (long long)N0;
    float* out = rs.io.out + (c - rs.io.step0) * rs.io.out_step + (long long)o * rs.io.out_ch;
    for (int i = tid; i < N0; i += NT) {
        float v = sf[i];
        for (int L = 1; L < bank.M; ++L) {
            const MLevel& l2 = bank.lv[L];
            v += __ldcg(&l2.yring[(size_t)o * (l2.rmask + 1) + ((t_new + i) & l2.rmask)]);
        }
        out[i * rs.io.out_sample] = v;
    }
}

// filter spectra of one path row: H[o][i][p] = rfft([0_N, h_{i,o}[start + pN ...]]) / 2N
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) mimo_spectra_kernel(const float* __restrict__ irs, int ir_len, int nI, int nO,
                                                          int N, int logN, int P, int cs, long long start, float2* H,
                                                          const int* __restrict__ tstart, int ntile,
                                                          const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const int row = blockIdx.x;   // (o * nI + i) * P + p
    const int p = row % P, io = row / P, i = io % nI, o = io / nI;
    const float* h = irs + ((size_t)i * nO + o) * ir_len;
    const long long base = start + (long long)p * N;
    for (int n = threadIdx.x; n < N; n += NT) {
        const int j = 2 * n - N;
        float a = 0.f, b = 0.f;
        if (j >= 0) {
            if (base + j < ir_len) a = h[base + j];
            if (base + j + 1 < ir_len) b = h[base + j + 1];
        }
        s[n] = make_float2(a, b);
    }
    load_twiddles<NT>(twt, logN, W, wlog);
    __syncthreads();
    const Twiddles tw{twt, logN};
    fft_smem<NT, MAXB>(s, N, logN, tw, false);
    const float inv = 1.0f / (float)(2 * N);
    // bin k of path (i, o), part p goes to its tile: H[o][tile][i][p][k - tile start]
    float2* Ho = H + (size_t)o * nI * P * cs;
    const int ip = i * P + p;
    auto put = [&](int kb, float2 v) {
        int lo = 0, hi = ntile;   // tile t with tstart[t] <= kb < tstart[t + 1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (tstart[mid] <= kb) lo = mid;
            else hi = mid;
        }
        const int k0 = tstart[lo], w = tstart[lo + 1] - k0;
        Ho[(size_t)k0 * nI * P + (size_t)ip * w + (kb - k0)] = v;
    };
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, logN, tw, xk, xnk);
        put(k, make_float2(xk.x * inv, xk.y * inv));
        if (N - k != k) put(N - k, make_float2(xnk.x * inv, xnk.y * inv));
    }
}

int cls_of(int N) { return N <= 1024 ? 0 : (N <= 4096 ? 1 : 2); }

cudaLaunchConfig_t pdl_cfg(int grid, int nt, size_t smem, cudaStream_t st, cudaLaunchAttribute* attr, bool pdl) {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cfg;
}

}  // namespace

struct pcm_handle {
    int verbosity = 0;
    std::string err;
    bool ready = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    int fs = 0, N0 = 0, nI = 0, nO = 0, M = 0, H = 1, maxN = 0, fft_cls = 0;
    std::vector<int> N, P;
    std::vector<void*> allocs;
    MBank hbank{};
    MBank* d_bank = nullptr;
    float* xring = nullptr;
    int rin_mask = 0;
    // per stage and phase: tasks at d_tasks + off, count cnt
    MTask* d_tasks = nullptr;
    std::vector<int> off[3], cnt[3];
    std::vector<double> mac_bytes;   // algorithmic bytes of K2 per phase
    std::vector<std::vector<int>> tiles;   // per level: bin tile starts (last entry cs)
    size_t state_bytes_total = 0;
    std::vector<std::pair<void*, size_t>> state;   // zeroed by reset
    long long frame_num = 0;
    long long launches = 0;
    long long device_bytes = 0;
};

namespace {

int mfail(pcm_handle* h, int code, const std::string& m) {
    h->err = m;
    return code;
}

#define MCK(call, where)                                                                                   \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return mfail(h, PC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
cudaError_t malloc_zero(pcm_handle* h, T** p, size_t n, bool is_state) {
    const size_t bytes = sizeof(T) * std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) return e;
    h->allocs.push_back(*p);
    h->device_bytes += bytes;
    if (is_state) h->state.push_back({*p, bytes});
    return cudaMemsetAsync(*p, 0, bytes, h->stream);
}

void mfree(pcm_handle* h) {
    if (h->device >= 0) cudaSetDevice(h->device);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    h->state.clear();
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    h->ready = false;
}

cudaError_t launch_fft_stage(pcm_handle* h, int stage, int grid, const MTask* tasks, const RunState& rs,
                             cudaStream_t st, bool pdl) {
    cudaLaunchAttribute attr[1];
    const int NT = h->fft_cls == 0 ? 256 : 512;
    const size_t smem = (size_t)12 * h->maxN;
    cudaLaunchConfig_t cfg = pdl_cfg(grid, NT, smem, st, attr, pdl);
    if (stage == 0) {
        switch (h->fft_cls) {
            case 0: return cudaLaunchKernelEx(&cfg, mimo_xfft_kernel<256, 1>, (const MBank*)h->d_bank, tasks, rs, h->xring, h->rin_mask);
            case 1: return cudaLaunchKernelEx(&cfg, mimo_xfft_kernel<512, 2>, (const MBank*)h->d_bank, tasks, rs, h->xring, h->rin_mask);
            default: return cudaLaunchKernelEx(&cfg, mimo_xfft_kernel<512, 8>, (const MBank*)h->d_bank, tasks, rs, h->xring, h->rin_mask);
        }
    }
    switch (h->fft_cls) {
        case 0: return cudaLaunchKernelEx(&cfg, mimo_yifft_kernel<256, 1>, (const MBank*)h->d_bank, tasks, rs);
        case 1: return cudaLaunchKernelEx(&cfg, mimo_yifft_kernel<512, 2>, (const MBank*)h->d_bank, tasks, rs);
        default: return cudaLaunchKernelEx(&cfg, mimo_yifft_kernel<512, 8>, (const MBank*)h->d_bank, tasks, rs);
    }
}

cudaError_t launch_mac(pcm_handle* h, int grid, const MTask* tasks, const RunState& rs, cudaStream_t st, bool pdl) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = pdl_cfg(grid, kMacNT, 0, st, attr, pdl);
    return cudaLaunchKernelEx(&cfg, mimo_mac_kernel, (const MBank*)h->d_bank, tasks, rs);
}

// one base step; kernel k of the step is timed by ev[k] pairs when given
int mimo_step(pcm_handle* h, const RunState& rs, cudaStream_t st, bool first, cudaEvent_t* ev) {
    const int ph = (int)(rs.step_base & (h->H - 1));
    for (int stage = 0; stage < 3; ++stage) {
        const int n = h->cnt[stage][ph];
        if (n <= 0) continue;
        if (ev) cudaEventRecord(ev[2 * stage], st);
        const MTask* tk = h->d_tasks + h->off[stage][ph];
        cudaError_t e = stage == 1 ? launch_mac(h, n, tk, rs, st, !first && !ev)
                                   : launch_fft_stage(h, stage == 0 ? 0 : 1, n, tk, rs, st, !first && !ev);
        if (ev) cudaEventRecord(ev[2 * stage + 1], st);
        if (e != cudaSuccess) return mfail(h, PC_ERR_CUDA, std::string("MIMO step launch: ") + cudaGetErrorString(e));
        h->launches += 1;
        first = false;
    }
    return PC_OK;
}

}  // namespace

extern "C" {

pcm_handle* pcm_create(int verbosity) {
    pcm_handle* h = new (std::nothrow) pcm_handle();
    if (h) h->verbosity = verbosity;
    return h;
}

int pcm_setup(pcm_handle* h, int fs, int buffer_size, int n_in, int n_out, int M, const int* N, int* P,
              const float* irs, int ir_len) {
    if (!h) return PC_ERR_ARG;
    if (h->ready) return mfail(h, PC_ERR_STATE, "setup called twice without cleanup");
    if (!N || !P || !irs || n_in < 1 || n_out < 1 || ir_len < 1 || M < 1)
        return mfail(h, PC_ERR_ARG, "bad MIMO setup arguments");
    if (M > kMaxMimoLevels) return mfail(h, PC_ERR_LIMIT, "too many levels for the MIMO engine");
    if (N[0] != buffer_size || buffer_size < 16) return mfail(h, PC_ERR_LAYOUT, "first block size must equal buffer_size (>= 16)");
    std::vector<int> Nv(N, N + M), Pv(P, P + M);
    char msg[256];
    int r = pc_check_layout(M, Nv.data(), Pv.data(), ir_len, 1, nullptr, msg, sizeof msg);
    if (r) return mfail(h, r, msg);
    if (Nv[M - 1] > kMaxBlockOneCta)
        return mfail(h, PC_ERR_LIMIT, "MIMO levels are limited to blocks of 16384 (larger blocks: pc_* engine)");
    for (int i = 0; i < M; ++i) P[i] = Pv[i];
    MCK(cudaGetDevice(&h->device), "cudaGetDevice");
    MCK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
    h->fs = fs;
    h->N0 = buffer_size;
    h->nI = n_in;
    h->nO = n_out;
    h->M = M;
    h->N = Nv;
    h->P = Pv;
    h->maxN = Nv.back();
    h->H = std::max(1, Nv.back() / buffer_size);
    h->fft_cls = cls_of(h->maxN);
    if (h->fft_cls == 2) {
        MCK(cudaFuncSetAttribute(mimo_xfft_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384), "attr");
        MCK(cudaFuncSetAttribute(mimo_yifft_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384), "attr");
        MCK(cudaFuncSetAttribute(mimo_spectra_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384), "attr");
    }
    // twiddles
    float2* W = nullptr;
    {
        std::vector<float2> Wh((size_t)1 << kWlog);
        for (size_t m = 0; m < Wh.size(); ++m) {
            const double a = -2.0 * M_PI * (double)m / (double)Wh.size();
            Wh[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        MCK(malloc_zero(h, &W, Wh.size(), false), "alloc");
        MCK(cudaMemcpyAsync(W, Wh.data(), sizeof(float2) * Wh.size(), cudaMemcpyHostToDevice, h->stream), "upload");
        MCK(cudaStreamSynchronize(h->stream), "sync");
    }
    int rin = 1;
    while (rin < 2 * h->maxN) rin <<= 1;
    h->rin_mask = rin - 1;
    MCK(malloc_zero(h, &h->xring, (size_t)n_in * rin, true), "alloc");
    float* d_irs = nullptr;
    MCK(malloc_zero(h, &d_irs, (size_t)n_in * n_out * ir_len, false), "alloc");
    MCK(cudaMemcpyAsync(d_irs, irs, sizeof(float) * (size_t)n_in * n_out * ir_len, cudaMemcpyHostToDevice, h->stream),
        "upload IRs");
    MBank& B = h->hbank;
    B.wlog = kWlog;
    B.N0 = buffer_size;
    B.nI = n_in;
    B.nO = n_out;
    B.M = M;
    B.W = W;
    long s = 0;
    for (int L = 0; L < M; ++L) {
        MLevel& l = B.lv[L];
        l.N = Nv[L];
        l.logN = (int)std::lround(std::log2((double)Nv[L]));
        l.P = Pv[L];
        l.T = Nv[L] / buffer_size;
        l.s_blocks = (int)(s / buffer_size);
        l.cs = Nv[L] + 2;
        long R = Nv[L];
        while (R < s + buffer_size) R <<= 1;
        l.rmask = (int)R - 1;
        // input ranges per spread task (about 8 inputs each, more ranges when
        // a range times the older parts exceeds what one MAC task sums)
        const int p_lo = l.T == 1 ? 2 : 1;
        l.npart = std::max(1, std::min(n_in, 8));
        while (l.npart < n_in && (long)((n_in + l.npart - 1) / l.npart) * std::max(l.P - p_lo, 0) > kMaxMacTerms)
            l.npart *= 2;
        l.npart = std::min(l.npart, n_in);
        if ((long)((n_in + l.npart - 1) / l.npart) * std::max(l.P - p_lo, 0) > kMaxMacTerms ||
            (long)n_in * 2 > kMaxMacTerms || (long)n_in * l.P * l.cs >= (1L << 31))
            return mfail(h, PC_ERR_LIMIT, "MIMO layout too large for one MAC task (inputs x parts)");
        // the level's fixed bin tiles: the slices its MAC tasks take (level 0:
        // the whole row; larger levels: each phase's slice of bins), cut into
        // tiles of at most kMacMaxBins bins
        {
            std::vector<int> ts;
            // a MAC CTA runs floor(kMacNT / columns) term groups over a tile's
            // columns: pick the tile count that keeps most threads busy (a
            // small charge per extra tile for its CTA's fixed work)
            auto tiles_of = [&](int lo, int hi) {
                const int n = hi - lo;
                int best_nt = 0;
                double best = -1.0;
                for (int nt = (n + kMacMaxBins - 1) / kMacMaxBins; nt <= 16; ++nt) {
                    const int per = ((n + nt - 1) / nt + 1) & ~1;
                    if (per < 2 || (nt - 1) * per >= n) continue;
                    double busy = 0.0;
                    for (int k = lo; k < hi; k += per) {
                        const int nc = (std::min(per, hi - k)) >> 1;
                        busy += (double)((kMacNT / nc) * nc) / kMacNT;
                    }
                    const double score = busy / nt - 0.05 * nt;
                    if (score > best) {
                        best = score;
                        best_nt = nt;
                    }
                }
                const int per = ((n + best_nt - 1) / best_nt + 1) & ~1;
                for (int k = lo; k < hi; k += per) ts.push_back(k);
            };
            if (l.T > 1 && l.P >= 2) {
                const int nch = l.T - 1;
                for (int j = 0; j < nch; ++j) {
                    const int lo = (int)(((long)j * l.cs / nch) & ~1L);
                    const int hi = (j == nch - 1) ? l.cs : (int)(((long)(j + 1) * l.cs / nch) & ~1L);
                    if (hi > lo) tiles_of(lo, hi);
                }
            } else {
                tiles_of(0, l.cs);
            }
            ts.push_back(l.cs);
            l.ntile = (int)ts.size() - 1;
            int* d_ts = nullptr;
            MCK(malloc_zero(h, &d_ts, ts.size(), false), "alloc tiles");
            MCK(cudaMemcpyAsync(d_ts, ts.data(), sizeof(int) * ts.size(), cudaMemcpyHostToDevice, h->stream),
                "upload tiles");
            l.tstart = d_ts;
            h->tiles.push_back(ts);
        }
        MCK(malloc_zero(h, &l.H, (size_t)n_out * n_in * l.P * l.cs, false), "alloc H");
        MCK(malloc_zero(h, &l.X, (size_t)n_in * l.P * l.cs, true), "alloc");
        MCK(malloc_zero(h, &l.Yp, (size_t)n_out * l.npart * 2 * l.cs, true), "alloc");
        MCK(malloc_zero(h, &l.Yf, (size_t)n_out * l.cs, true), "alloc");
        MCK(malloc_zero(h, &l.yring, (size_t)n_out * R, true), "alloc");
        const size_t smem = (size_t)12 * l.N;
        const int rows = n_out * n_in * l.P;
        switch (cls_of(l.N)) {
            case 0:
                mimo_spectra_kernel<256, 1><<<rows, 256, smem, h->stream>>>(d_irs, ir_len, n_in, n_out, l.N, l.logN, l.P,
                                                                            l.cs, s, l.H, l.tstart, l.ntile, W, kWlog);
                break;
            case 1:
                mimo_spectra_kernel<512, 2><<<rows, 512, smem, h->stream>>>(d_irs, ir_len, n_in, n_out, l.N, l.logN, l.P,
                                                                            l.cs, s, l.H, l.tstart, l.ntile, W, kWlog);
                break;
            default:
                mimo_spectra_kernel<512, 8><<<rows, 512, smem, h->stream>>>(d_irs, ir_len, n_in, n_out, l.N, l.logN, l.P,
                                                                            l.cs, s, l.H, l.tstart, l.ntile, W, kWlog);
                break;
        }
        MCK(cudaGetLastError(), "MIMO spectra");
        h->launches += 1;
        s += (long)Nv[L] * Pv[L];
    }
    MCK(malloc_zero(h, &h->d_bank, 1, false), "alloc");
    MCK(cudaMemcpyAsync(h->d_bank, &B, sizeof(MBank), cudaMemcpyHostToDevice, h->stream), "upload bank");

    // ---- per-phase task lists --------------------------------------------------------
    std::vector<std::vector<MTask>> lists[3];
    for (auto& v : lists) v.assign(h->H, {});
    h->mac_bytes.assign(h->H, 0.0);
    for (int g = 0; g < h->H; ++g) {
        for (int L = 0; L < M; ++L) {
            const MLevel& l = B.lv[L];
            const double C = l.N + 1.0;
            const bool fires = (g + 1 + l.s_blocks) % l.T == 0;
            if (fires) {
                for (int i = 0; i < n_in; ++i) lists[0][g].push_back(MTask{0, L, i, 0, 0, 0, 0, 0});
                const std::vector<int>& ts = h->tiles[L];   // the level's fixed tiles
                for (int o = 0; o < n_out; ++o)
                    for (size_t t = 0; t + 1 < ts.size(); ++t)
                        lists[1][g].push_back(MTask{1, L, o, ts[t], ts[t + 1], 0, n_in, 0});
                for (int o = 0; o < n_out; ++o) lists[2][g].push_back(MTask{3, L, o, 0, 0, 0, 0, 0});
                const int np = (l.T == 1 && l.P >= 2) ? 2 : 1;
                // H rows of parts 0 (and 1) of every path, X rows once per input
                h->mac_bytes[g] += 8.0 * C * ((double)n_out * n_in * np + (double)n_in * np);
            }
            // spread: level 0 every step over parts >= 2; other levels in the
            // T-1 steps after their block, a slice of bins per step
            int lo = 0, hi = 0, p_lo = 1;
            if (l.T == 1) {
                if (l.P < 3) continue;
                lo = 0;
                hi = l.cs;
                p_lo = 2;
            } else {
                if (l.P < 2) continue;
                const int phi = (g + 1 + l.s_blocks) % l.T;
                if (phi == 0) continue;
                const int j = phi - 1, nch = l.T - 1;
                lo = (int)(((long)j * l.cs / nch) & ~1L);
                hi = (j == nch - 1) ? l.cs : (int)(((long)(j + 1) * l.cs / nch) & ~1L);
            }
            if (hi <= lo) continue;
            std::vector<std::pair<int, int>> tl;   // the level's fixed tiles within [lo, hi)
            const std::vector<int>& ts = h->tiles[L];
            for (size_t t = 0; t + 1 < ts.size(); ++t)
                if (ts[t] >= lo && ts[t + 1] <= hi) tl.push_back({ts[t], ts[t + 1]});
            for (int o = 0; o < n_out; ++o)
                for (auto& kk : tl)
                    for (int q = 0; q < l.npart; ++q) {
                        const int i0 = (int)((long)q * n_in / l.npart), i1 = (int)((long)(q + 1) * n_in / l.npart);
                        lists[1][g].push_back(MTask{2, L, o, kk.first, kk.second, i0, i1, q});
                    }
            h->mac_bytes[g] += 8.0 * (hi - lo) * ((double)n_out * n_in * (l.P - p_lo) + (double)n_in * (l.P - p_lo));
        }
    }
    size_t ntask = 0;
    for (int st = 0; st < 3; ++st) {
        h->off[st].assign(h->H, 0);
        h->cnt[st].assign(h->H, 0);
        for (int g = 0; g < h->H; ++g) {
            h->off[st][g] = (int)ntask;
            h->cnt[st][g] = (int)lists[st][g].size();
            ntask += lists[st][g].size();
        }
    }
    std::vector<MTask> all;
    all.reserve(ntask);
    for (int st = 0; st < 3; ++st)
        for (int g = 0; g < h->H; ++g) all.insert(all.end(), lists[st][g].begin(), lists[st][g].end());
    MCK(malloc_zero(h, &h->d_tasks, all.size(), false), "alloc tasks");
    MCK(cudaMemcpyAsync(h->d_tasks, all.data(), sizeof(MTask) * all.size(), cudaMemcpyHostToDevice, h->stream),
        "upload tasks");
    MCK(cudaStreamSynchronize(h->stream), "setup sync");
    cudaFree(d_irs);
    h->allocs.erase(std::find(h->allocs.begin(), h->allocs.end(), (void*)d_irs));
    h->device_bytes -= (long long)sizeof(float) * n_in * n_out * ir_len;
    h->frame_num = 0;
    h->ready = true;
    return PC_OK;
}

int pcm_process_device(pcm_handle* h, float* d_out, const float* d_in, long long frames, int layout, void* stream) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return mfail(h, PC_ERR_STATE, "process before setup");
    if (!d_out || !d_in || frames <= 0 || frames % h->N0)
        return mfail(h, PC_ERR_ARG, "frames must be a positive multiple of buffer_size");
    cudaSetDevice(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    RunState rs{};
    rs.io.in = d_in;
    rs.io.out = d_out;
    rs.io.step0 = h->frame_num;
    if (layout == PC_PLANAR) {
        rs.io.in_step = h->N0;
        rs.io.in_sample = 1;
        rs.io.in_ch = frames;
        rs.io.out_step = h->N0;
        rs.io.out_sample = 1;
        rs.io.out_ch = frames;
    } else {
        rs.io.in_step = (long long)h->N0 * h->nI;
        rs.io.in_sample = h->nI;
        rs.io.in_ch = 1;
        rs.io.out_step = (long long)h->N0 * h->nO;
        rs.io.out_sample = h->nO;
        rs.io.out_ch = 1;
    }
    const long long nsteps = frames / h->N0;
    for (long long s = 0; s < nsteps; ++s) {
        rs.step_base = h->frame_num + s;
        int r = mimo_step(h, rs, st, s == 0, nullptr);
        if (r) return r;
    }
    h->frame_num += nsteps;
    return PC_OK;
}

int pcm_reset(pcm_handle* h) {
    if (!h) return PC_ERR_ARG;
    h->frame_num = 0;
    if (!h->ready) return PC_OK;
    cudaSetDevice(h->device);
    for (auto& z : h->state) MCK(cudaMemsetAsync(z.first, 0, z.second, h->stream), "reset");
    MCK(cudaStreamSynchronize(h->stream), "reset sync");
    return PC_OK;
}

int pcm_profile_kernels(pcm_handle* h, long long nsteps, pc_kernel_stats* out, int max_kinds, int* n_kinds) {
    if (!h || !h->ready || nsteps < 1 || !out) return PC_ERR_ARG;
    cudaSetDevice(h->device);
    // every step reads and writes the first block of zero-filled scratch I/O
    float* io = nullptr;
    const size_t ion = (size_t)h->N0 * std::max(h->nI, h->nO);
    MCK(cudaMalloc(&io, sizeof(float) * ion * 2), "profile buffer");
    cudaMemsetAsync(io, 0, sizeof(float) * ion * 2, h->stream);
    RunState rs{};
    rs.io.in = io;
    rs.io.out = io + ion;
    rs.io.step0 = 0;
    rs.io.in_sample = h->nI;
    rs.io.in_ch = 1;
    rs.io.out_sample = h->nO;
    rs.io.out_ch = 1;
    double ms[3] = {0, 0, 0}, bytes[3] = {0, 0, 0};
    long long cnt[3] = {0, 0, 0};
    std::vector<cudaEvent_t> evs;
    std::vector<int> phases;
    for (long long s = 0; s < nsteps; ++s) {
        cudaEvent_t e[6];
        for (auto& x : e) {
            cudaEventCreate(&x);
            evs.push_back(x);
        }
        rs.step_base = h->frame_num + s;
        phases.push_back((int)(rs.step_base & (h->H - 1)));
        int r = mimo_step(h, rs, h->stream, true, e);
        if (r) return r;
    }
    h->frame_num += nsteps;
    MCK(cudaStreamSynchronize(h->stream), "profile sync");
    for (long long s = 0; s < nsteps; ++s) {
        for (int k = 0; k < 3; ++k) {
            if (h->cnt[k][phases[s]] <= 0) continue;
            float t = 0;
            cudaEventElapsedTime(&t, evs[6 * s + 2 * k], evs[6 * s + 2 * k + 1]);
            ms[k] += t;
            cnt[k] += 1;
            if (k == 1) bytes[k] += h->mac_bytes[phases[s]];
        }
    }
    for (auto e : evs) cudaEventDestroy(e);
    cudaFree(io);
    static const char* names[3] = {"mimo_xfft", "mimo_mac", "mimo_yifft"};
    int n = 0;
    for (int k = 0; k < 3 && n < max_kinds; ++k) {
        if (!cnt[k]) continue;
        std::snprintf(out[n].name, sizeof out[n].name, "%s", names[k]);
        out[n].launches = cnt[k];
        out[n].total_ms = ms[k];
        out[n].alg_bytes = bytes[k];
        ++n;
    }
    if (n_kinds) *n_kinds = n;
    return PC_OK;
}

long long pcm_device_bytes(const pcm_handle* h) { return h ? h->device_bytes : 0; }
long long pcm_kernel_launches(const pcm_handle* h) { return h ? h->launches : 0; }
const char* pcm_last_error(const pcm_handle* h) { return h ? h->err.c_str() : ""; }

void pcm_destroy(pcm_handle* h) {
    if (!h) return;
    mfree(h);
    delete h;
}

}  // extern "C"
