// step_kernels.cu -- the per-base-block kernels of the partitioned
// convolution engine (sm_103a).
//
// One base step c (one run() callback of N0 frames) is, for every PC:
//   * fire tasks: each level L whose input block completes in this step
//     ((c + 1) N0 + s_L == (b + 1) N_L) computes its block b in one CTA:
//     load the newest 2 N_L input samples, real FFT (shared-memory Stockham),
//     store the spectrum in ring slot b mod P_L, Y = X_b H_0 + sum_{p>=1}
//     (level 0: the full FDL MAC over all parts, p ascending, like
//     PartConvFilter::runLevel, src/partconv.cpp:354-490; other levels: the
//     p >= 1 sum was precomputed by spread tasks), inverse FFT, keep the first
//     N_L samples (overlap-save with the block at offset N_L,
//     matlab/FDL_part_conv.m:18-20).  Level 0's CTA also emits the step's
//     output: its own block plus the due N0-slice of every other level's
//     output ring, in level order (PartConvFilter::output,
//     src/partconv.cpp:616-631), and mixes it into the output channel
//     (src/partconvMulti.cpp:911-921).
//   * spread tasks: the streaming FDL MAC Yp[k] = sum_{p=1}^{P-1}
//     X[(b+1-p) mod P][k] H[p][k] for the next block of a level, a slice of
//     bins per step, so a large level's MAC is spread over the N_L/N0 - 1
//     base steps between its blocks (the role of the per-level worker threads
//     of src/partconvMulti.cpp:930-1013).
// Fire and spread tasks of one step touch disjoint data, so they run as
// independent kernels; the next step depends on both.
#include <cuda_runtime.h>

#include "engine_types.h"
#include "fft_smem.cuh"
#include "kernels.h"

namespace pcg {

__device__ __forceinline__ const RunState& pick_state(const RunState& v, const RunState* d) {
    return d ? *d : v;
}

__device__ __forceinline__ long long imod(long long a, long long m) {
    long long r = a % m;
    return r < 0 ? r + m : r;
}

// ---------------------------------------------------------------------------
// Fire kernel: one CTA per firing level block.
// ---------------------------------------------------------------------------
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) fire_kernel(Bank bank, const FireTask* __restrict__ tasks,
                                                  const int* __restrict__ off, RunState rs_val,
                                                  const RunState* rs_dev, int step_in_batch) {
    extern __shared__ float2 s[];
    __shared__ int s_last;
    const RunState& rs = pick_state(rs_val, rs_dev);
    const long long c = rs.step_base + step_in_batch;
    const int phase = (int)(c & (long long)(bank.H - 1));
    const int t = off[phase] + blockIdx.x;
    if (t >= off[phase + 1]) return;

    const DevLevel lv = bank.lv[tasks[t].level];
    const DevPC pc = bank.pcs[lv.pc];
    const int N = lv.N, logN = lv.logN;
    const int N0 = bank.N0;
    const int tid = threadIdx.x;
    const long long t_new = c * (long long)N0;            // first sample of this step
    const long long t_end = t_new + N0;                   // newest sample + 1
    const long long io_step = c - rs.io.step0;
    const float* in = rs.io.in + io_step * rs.io.in_step + (long long)pc.in_ch * rs.io.in_ch;
    const float scale = pc.scale;
    const bool is_l0 = (tasks[t].level == pc.lv0);

    // -- window: newest 2N samples as N complex pairs ----------------------
    for (int n = tid; n < N; n += NT) {
        const long long ta = t_end - 2LL * N + 2LL * n;
        float a, b;
        if (ta >= t_new) {
            const long long i = ta - t_new;
            a = in[i * rs.io.in_sample] * scale;
            b = in[(i + 1) * rs.io.in_sample] * scale;
        } else {
            a = pc.xring[ta & pc.rin_mask];
            b = pc.xring[(ta + 1) & pc.rin_mask];
        }
        s[n] = make_float2(a, b);
    }
    if (is_l0) {
        // append this step's input to the PC's time-domain ring
        for (int i = tid; i < N0; i += NT) pc.xring[(t_new + i) & pc.rin_mask] = in[i * rs.io.in_sample] * scale;
    }
    __syncthreads();

    fft_smem<NT, MAXB>(s, N, logN, bank.W, bank.wlog, false);

    // -- split, FDL MAC, inverse merge --------------------------------------
    const long long q = c + 1 + lv.s_blocks;
    const long long b = q / lv.T - 1;
    const int slot = (int)imod(b, lv.P);
    float2* __restrict__ Xs = lv.X + (size_t)slot * lv.cs;
    const float2* __restrict__ H = lv.H;
    const int half = N >> 1;
    for (int k = tid; k <= half; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, N, logN, bank.W, bank.wlog, xk, xnk);
        const int bk = k, bnk = N - k;   // k == 0 pairs bin 0 with bin N
        Xs[bk] = xk;
        if (bnk != bk) Xs[bnk] = xnk;
        float2 yk = cmul(xk, __ldg(&H[bk]));
        float2 ynk = cmul(xnk, __ldg(&H[bnk]));
        if (lv.T == 1) {
            for (int p = 1; p < lv.P; ++p) {
                const int sl = (int)imod(b - p, lv.P);
                const float2* Xp = lv.X + (size_t)sl * lv.cs;
                const float2* Hp = H + (size_t)p * lv.cs;
                yk = cadd(yk, cmul(Xp[bk], __ldg(&Hp[bk])));
                ynk = cadd(ynk, cmul(Xp[bnk], __ldg(&Hp[bnk])));
            }
        } else {
            yk = cadd(yk, lv.Yp[bk]);
            ynk = cadd(ynk, lv.Yp[bnk]);
        }
        float2 zk, znk;
        irfft_merge(yk, ynk, k, N, logN, bank.W, bank.wlog, zk, znk);
        s[k] = zk;
        if (k != 0 && k != half) s[N - k] = znk;
    }
    __syncthreads();

    fft_smem<NT, MAXB>(s, N, logN, bank.W, bank.wlog, true);

    const float* sf = reinterpret_cast<const float*>(s);   // y[i] = sf[i] for i < 2N
    if (!is_l0) {
        // level block b covers output samples [b N, (b+1) N)
        const long long t0 = b * (long long)N;
        for (int i = tid; i < N; i += NT) lv.yring[(t0 + i) & lv.rmask] = sf[i];
        return;
    }

    // -- level 0: emit this step's output --------------------------------------
    float* out = rs.io.out + io_step * rs.io.out_step;
    const long long osamp = rs.io.out_sample;
    for (int i = tid; i < N0; i += NT) {
        float v = sf[i];
        for (int L = 1; L < pc.M; ++L) {
            const DevLevel& l2 = bank.lv[pc.lv0 + L];
            v += l2.yring[(t_new + i) & l2.rmask];
        }
        if (pc.mix_mode == 1) out[i * osamp + (long long)pc.out_ch * rs.io.out_ch] = v;
        else if (pc.mix_mode == 2) pc.pcout[i] = v;
        for (int z = 0; z < pc.zero_outs; ++z)
            out[i * osamp + (long long)bank.zero_list[pc.zero_off + z] * rs.io.out_ch] = 0.0f;
    }
    if (pc.mix_mode != 2) return;

    // several PCs feed this output: the last one to arrive sums them in PC
    // order (deterministic, no atomics on samples)
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const int o = pc.out_ch;
        const int cnt = bank.out_off[o + 1] - bank.out_off[o];
        s_last = (atomicAdd(&bank.mix_cnt[o], 1) == cnt - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int o = pc.out_ch;
    const int j0 = bank.out_off[o], j1 = bank.out_off[o + 1];
    for (int i = tid; i < N0; i += NT) {
        float v = 0.0f;
        for (int j = j0; j < j1; ++j) v += __ldcg(&bank.pcs[bank.out_pcs[j]].pcout[i]);
        out[i * osamp + (long long)o * rs.io.out_ch] = v;
    }
    if (tid == 0) bank.mix_cnt[o] = 0;
}

// ---------------------------------------------------------------------------
// Spread kernel: partial FDL MAC over parts p >= 1, two bins per thread.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT) spread_kernel(Bank bank, const SpreadTask* __restrict__ tasks,
                                                    const int* __restrict__ off, RunState rs_val,
                                                    const RunState* rs_dev, int step_in_batch) {
    const RunState& rs = pick_state(rs_val, rs_dev);
    const long long c = rs.step_base + step_in_batch;
    const int phase = (int)(c & (long long)(bank.H - 1));
    const int t = off[phase] + blockIdx.x;
    if (t >= off[phase + 1]) return;
    const SpreadTask tk = tasks[t];
    const DevLevel lv = bank.lv[tk.level];
    const int k = tk.k0 + 2 * threadIdx.x;
    if (k >= tk.k1) return;
    const long long q = c + 1 + lv.s_blocks;
    const long long b = q / lv.T - 1;   // newest block already fired
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int sl = (int)imod(b, lv.P);        // slot of block b + 1 - p for p = 1
    const float4* X4 = reinterpret_cast<const float4*>(lv.X + k);
    const float4* H4 = reinterpret_cast<const float4*>(lv.H + k);
    const int rs4 = lv.cs >> 1;         // row stride in float4
#pragma unroll 4
    for (int p = 1; p < lv.P; ++p) {
        const float4 x = __ldcg(X4 + (size_t)sl * rs4);
        const float4 h = __ldg(H4 + (size_t)p * rs4);
        acc.x += x.x * h.x - x.y * h.y;
        acc.y += x.x * h.y + x.y * h.x;
        acc.z += x.z * h.z - x.w * h.w;
        acc.w += x.z * h.w + x.w * h.z;
        sl = (sl == 0) ? lv.P - 1 : sl - 1;
    }
    reinterpret_cast<float4*>(lv.Yp + k)[0] = acc;
}

// ---------------------------------------------------------------------------
// Filter spectra: H = rfft([0_N, h_row]) / 2N for one row per CTA.
// ---------------------------------------------------------------------------
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) spectra_kernel(const SpectraJob* __restrict__ jobs, const float2* W,
                                                     int wlog) {
    extern __shared__ float2 s[];
    const SpectraJob jb = jobs[blockIdx.x];
    const int N = jb.N;
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
    __syncthreads();
    fft_smem<NT, MAXB>(s, N, jb.logN, W, wlog, false);
    const float inv = 1.0f / (float)(2 * N);
    const int half = N >> 1;
    for (int k = tid; k <= half; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, N, jb.logN, W, wlog, xk, xnk);
        jb.dst[k] = make_float2(xk.x * inv, xk.y * inv);
        if (N - k != k) jb.dst[N - k] = make_float2(xnk.x * inv, xnk.y * inv);
    }
}

__global__ void set_state_kernel(RunState* dst, RunState v) { *dst = v; }

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
static int class_of(int N) { return N <= 1024 ? 0 : (N <= 4096 ? 1 : 2); }

int fire_class_of(int N) { return class_of(N); }

static const int kFireNT[3] = {128, 256, 512};
int fire_threads(int cls) { return kFireNT[cls]; }

cudaError_t prepare_kernels() {
    cudaError_t e;
    e = cudaFuncSetAttribute(fire_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 16384 * 8);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fire_kernel<256, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 8);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(spectra_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 16384 * 8);
    return e;
}

cudaError_t launch_fire(int cls, int grid, int maxN, const Bank& bank, const FireTask* tasks, const int* off,
                        const RunState& rs, const RunState* rs_dev, int step_in_batch, cudaStream_t st) {
    if (grid <= 0) return cudaSuccess;
    const size_t smem = (size_t)maxN * sizeof(float2);
    switch (cls) {
        case 0: fire_kernel<128, 2><<<grid, 128, smem, st>>>(bank, tasks, off, rs, rs_dev, step_in_batch); break;
        case 1: fire_kernel<256, 4><<<grid, 256, smem, st>>>(bank, tasks, off, rs, rs_dev, step_in_batch); break;
        default: fire_kernel<512, 8><<<grid, 512, smem, st>>>(bank, tasks, off, rs, rs_dev, step_in_batch); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_spread(int grid, const Bank& bank, const SpreadTask* tasks, const int* off, const RunState& rs,
                          const RunState* rs_dev, int step_in_batch, cudaStream_t st) {
    if (grid <= 0) return cudaSuccess;
    spread_kernel<kSpreadNT><<<grid, kSpreadNT, 0, st>>>(bank, tasks, off, rs, rs_dev, step_in_batch);
    return cudaGetLastError();
}

cudaError_t launch_spectra(int cls, int njobs, int maxN, const SpectraJob* jobs, const float2* W, int wlog,
                           cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    const size_t smem = (size_t)maxN * sizeof(float2);
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
