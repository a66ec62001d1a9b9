// adjoint.cu -- differentiable partitioned convolution: block-parallel FDL
// forward pass and hand-written adjoint kernels.
//
// For a batch of signals x_s (length T) and one IR h, y_s = (x_s * h)[0:T]
// with the IR cut into the levels of a partition layout (level L: N_L-sample
// blocks, P_L parts, taps [s_L, s_L + N_L P_L)).  The whole signal is known,
// so every block of a level is computed in parallel (offline form of the
// streaming FDL of PartConvFilter::runLevel, src/partconv.cpp:354-490):
//   X_b  = rfft(x_L window [(b-1)N, (b+1)N)),  x_L[m] = x[m - s_L]
//   Y_b  = sum_p X_{b-p} H_p,  H_p = rfft([0_N, h_p]) / 2N
//   y_L block b = irfft(Y_b)[0:N]
// Backward with g = dL/dy:
//   dL/dx (adjoint, anti-causal, conjugated spectra):
//     G'_c = rfft(g[cN + s_L, cN + s_L + 2N)),
//     gx_L block b = irfft(sum_p (-1)^k conj(H_p) G'_{b+p})[0:N]
//   dL/dh (partitioned cross-correlation of the input with the gradient):
//     GP_b = rfft([g block b, 0_N]),  D_p = sum_s sum_b conj(GP_b) X_{b-p},
//     dh[s_L + pN + q] = irfft(D_p)[N - q] / 2N,  0 <= q < N.
// Levels are summed in ascending order (PartConvFilter::output,
// src/partconv.cpp:616-631).  The caller provides the workspace (no
// allocation here); the input spectra X can be kept from the forward pass or
// recomputed in the backward pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
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
constexpr int kMaxDLevels = 8;
constexpr int kDhChunks = 16;   // partial sums of the dL/dh reduction (fixed order)

// Job tables are built once per plan with addresses relative to the call's
// buffers (DPtrs), so a call only launches kernels over tables already on
// the device.
enum { kSrcX = 0, kSrcH = 1, kSrcG = 2 };     // FJob sources: x, h, dL/dy
enum { kDstY = 0, kDstGH = 1, kDstGX = 2 };   // IJob targets: y, dL/dh, dL/dx
struct DPtrs {
    const float* in[3];
    float* out[3];
    char* ws;   // workspace: spectra rows are byte offsets into it
};
// window FFT job: row at ws + dst_off = rfft(w) * scale, w[n] = src[start + n]
// for n < 2N with src = in[src] + src_off, zero outside [0, len); half == 1
// zeroes the second half ([g block, 0_N]), half == 2 the first ([0_N, h part])
struct FJob {
    long long src_off, len, start, dst_off;
    float scale;
    int src, half, pad;
};
// inverse FFT job: o = irfft(row at ws + src_off), dst = out[dst] + dst_off;
// mode 0: dst[i] = o[i], 1: dst[i] += o[i] (i < min(N, limit)); mode 2:
// dst[q] = o[N - q] * scale (q < min(N, limit))
struct IJob {
    long long src_off, dst_off, limit;
    float scale;
    int dst, mode, pad;
};

// (the 512-thread, two-butterfly instances here and in difft_kernel are held
// to 32 registers so that four CTAs fit an SM: the 512 windows of a
// 4096-sample level over a batch of 8 then run in one wave instead of two)
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT, NT * MAXB == 1024 ? 4 : 1) dfft_kernel(const FJob* __restrict__ jobs, DPtrs ptr, int N, int logN,
                                                  const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const FJob jb = jobs[blockIdx.x];
    const float* src = ptr.in[jb.src] + jb.src_off;
    float2* dst = reinterpret_cast<float2*>(ptr.ws + jb.dst_off);
    const int lo = jb.half == 2 ? N : 0, hi = jb.half == 1 ? N : 2 * N;   // live window samples [lo, hi)
    for (int n = threadIdx.x; n < N; n += NT) {
        const long long i = jb.start + 2LL * n;
        float a = 0.f, b = 0.f;
        if (2 * n >= lo && 2 * n < hi && i >= 0 && i < jb.len) a = src[i];
        if (2 * n + 1 >= lo && 2 * n + 1 < hi && i + 1 >= 0 && i + 1 < jb.len) b = src[i + 1];
        s[sidx<true>(n)] = make_float2(a, b);
    }
    load_twiddles_sw<NT>(twt, logN, W, wlog);
    __syncthreads();
    const Twiddles tw{twt, logN};
    // transform buffer and twiddles in the conflict-free placement
    fft_smem<NT, MAXB, true>(s, N, logN, tw, false);
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split<true>(s[sidx<true>(k)], s[sidx<true>(nk)], k, logN, tw, xk, xnk);
        dst[k] = make_float2(xk.x * jb.scale, xk.y * jb.scale);
        if (N - k != k) dst[N - k] = make_float2(xnk.x * jb.scale, xnk.y * jb.scale);
    }
}

template <int NT, int MAXB>
__global__ void __launch_bounds__(NT, NT * MAXB == 1024 ? 4 : 1) difft_kernel(const IJob* __restrict__ jobs, DPtrs ptr, int N, int logN,
                                                   const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const IJob jb = jobs[blockIdx.x];
    const float2* src = reinterpret_cast<const float2*>(ptr.ws + jb.src_off);
    float* dst = ptr.out[jb.dst] + jb.dst_off;
    load_twiddles_sw<NT>(twt, logN, W, wlog);
    __syncthreads();
    const Twiddles tw{twt, logN};
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        float2 zk, znk;
        irfft_merge<true>(src[k], src[N - k], k, logN, tw, zk, znk);
        s[sidx<true>(k)] = zk;
        if (k != 0 && k != N / 2) s[sidx<true>(N - k)] = znk;
    }
    __syncthreads();
    fft_smem<NT, MAXB, true>(s, N, logN, tw, true);
    // real sample i is component i & 1 of complex element i >> 1
    auto y = [&](int i) { return reinterpret_cast<const float*>(s + sidx<true>(i >> 1))[i & 1]; };
    const int n = jb.limit < N ? (int)jb.limit : N;
    for (int i = threadIdx.x; i < n; i += NT) {
        if (jb.mode == 0) dst[i] = y(i);
        else if (jb.mode == 1) dst[i] += y(i);
        else dst[i] = y(N - i) * jb.scale;
    }
}

// Y[s][b] = sum_p X[s][b-p] H[p]                       (forward, mode 0)
// Y[s][b] = sum_p (-1)^k conj(H[p]) X[s][b+p]          (adjoint, mode 1)
// X has nxb blocks per signal; Y has nyb.
__global__ void dmac_kernel(const float2* __restrict__ X, const float2* __restrict__ H, float2* __restrict__ Y, int nsig,
                            int nxb, int nyb, int P, int cs, int mode) {
    const long long total = (long long)nsig * nyb * cs;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % cs);
        const long long sb = t / cs;
        const int b = (int)(sb % nyb);
        const int sg = (int)(sb / nyb);
        float2 acc = make_float2(0.f, 0.f);
        for (int p = 0; p < P; ++p) {
            const int xb = mode == 0 ? b - p : b + p;
            if (xb < 0 || xb >= nxb) continue;
            const float2 x = X[((long long)sg * nxb + xb) * cs + k];
            float2 h = H[(long long)p * cs + k];
            if (mode == 1) h = (k & 1) ? make_float2(-h.x, h.y) : make_float2(h.x, -h.y);   // (-1)^k conj(h)
            acc = cadd(acc, cmul(x, h));
        }
        Y[t] = acc;
    }
}

// Dpart[chunk][p][k] = sum over (s, b) of chunk of conj(GP[s][b][k]) X[s][b-p][k]
__global__ void ddh_partial_kernel(const float2* __restrict__ X, const float2* __restrict__ GP,
                                   float2* __restrict__ Dpart, int nsig, int nb, int P, int cs, int nchunk) {
    const long long total = (long long)nchunk * P * cs;
    const long long nsb = (long long)nsig * nb;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % cs);
        const int p = (int)((t / cs) % P);
        const int ch = (int)(t / ((long long)cs * P));
        const long long j0 = ch * nsb / nchunk, j1 = (ch + 1) * nsb / nchunk;
        float2 acc = make_float2(0.f, 0.f);
        for (long long j = j0; j < j1; ++j) {
            const int sg = (int)(j / nb), b = (int)(j % nb);
            if (b - p < 0) continue;
            const float2 g = GP[((long long)sg * nb + b) * cs + k];
            const float2 x = X[((long long)sg * nb + (b - p)) * cs + k];
            acc = cadd(acc, cmul(cconj(g), x));
        }
        Dpart[t] = acc;
    }
}

// Sliding forms of the two FDL sums for P <= kSlideP: a thread owns one bin
// of one signal over a run of kSlideRun consecutive blocks and keeps the last
// P input spectra of that bin in registers, so each block's spectrum is
// loaded once instead of once per part.  Same sums in the same part order as
// dmac_kernel / ddh_partial_kernel.
constexpr int kSlideP = 16;
constexpr int kSlideRun = 32;

// Y[s][b] = sum_p X[s][b-p] H[p] (mode 0); Y[s][b] = sum_p (-1)^k conj(H[p]) X[s][b+p] (mode 1)
__global__ void dmac_slide_kernel(const float2* __restrict__ X, const float2* __restrict__ H, float2* __restrict__ Y,
                                  int nsig, int nxb, int nyb, int P, int cs, int mode) {
    const int nrun = (nyb + kSlideRun - 1) / kSlideRun;
    const long long total = (long long)nsig * nrun * cs;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % cs);
        const long long sr = t / cs;
        const int run = (int)(sr % nrun), sg = (int)(sr / nrun);
        float2 h[kSlideP], w[kSlideP];   // filter bin per part; window of input spectra
#pragma unroll
        for (int p = 0; p < kSlideP; ++p) {
            h[p] = make_float2(0.f, 0.f);
            w[p] = make_float2(0.f, 0.f);
            if (p < P) {
                float2 v = H[(long long)p * cs + k];
                if (mode == 1) v = (k & 1) ? make_float2(-v.x, v.y) : make_float2(v.x, -v.y);   // (-1)^k conj
                h[p] = v;
            }
        }
        const float2* Xs = X + (long long)sg * nxb * cs + k;
        float2* Ys = Y + (long long)sg * nyb * cs + k;
        const int b0 = run * kSlideRun, b1 = min(nyb, b0 + kSlideRun);
        auto xat = [&](int xb) { return (xb >= 0 && xb < nxb) ? Xs[(long long)xb * cs] : make_float2(0.f, 0.f); };
        // mode 0 walks b upwards with w[p] = X[b - p]; mode 1 walks it
        // downwards with w[p] = X[b + p].  Each step shifts the window by one
        // and loads the newest block into w[0].
        const int dir = mode == 0 ? 1 : -1;
        const int start = mode == 0 ? b0 : b1 - 1;
#pragma unroll
        for (int p = 0; p < kSlideP - 1; ++p)   // the window one step before `start`
            if (p < P - 1) w[p] = xat(start - dir * (p + 1));
        for (int i = 0, b = start; i < b1 - b0; ++i, b += dir) {
#pragma unroll
            for (int p = kSlideP - 1; p > 0; --p) w[p] = w[p - 1];
            w[0] = xat(b);
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int p = 0; p < kSlideP; ++p)
                if (p < P) acc = cadd(acc, cmul(w[p], h[p]));
            Ys[(long long)b * cs] = acc;
        }
    }
}

// Dpart[s * nrun + run][p][k] = sum over blocks b of the run of
// conj(GP[s][b][k]) X[s][b-p][k], p < P <= kSlideP (the dL/dh correlation),
// with the last P input spectra of the bin kept in registers.
__global__ void ddh_slide_kernel(const float2* __restrict__ X, const float2* __restrict__ GP,
                                 float2* __restrict__ Dpart, int nsig, int nb, int P, int cs) {
    const int nrun = (nb + kSlideRun - 1) / kSlideRun;
    const long long total = (long long)nsig * nrun * cs;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % cs);
        const long long sr = t / cs;
        const int run = (int)(sr % nrun), sg = (int)(sr / nrun);
        const float2* Xs = X + (long long)sg * nb * cs + k;
        const float2* Gs = GP + (long long)sg * nb * cs + k;
        const int b0 = run * kSlideRun, b1 = min(nb, b0 + kSlideRun);
        float2 w[kSlideP], acc[kSlideP];
#pragma unroll
        for (int p = 0; p < kSlideP; ++p) {
            acc[p] = make_float2(0.f, 0.f);
            const int xb = b0 - 1 - p;   // the window one block before b0
            w[p] = (p < P - 1 && xb >= 0) ? Xs[(long long)xb * cs] : make_float2(0.f, 0.f);
        }
        for (int b = b0; b < b1; ++b) {
#pragma unroll
            for (int p = kSlideP - 1; p > 0; --p) w[p] = w[p - 1];
            w[0] = Xs[(long long)b * cs];
            const float2 g = cconj(Gs[(long long)b * cs]);
#pragma unroll
            for (int p = 0; p < kSlideP; ++p)
                if (p < P) acc[p] = cadd(acc[p], cmul(g, w[p]));
        }
        float2* D = Dpart + (sr * P) * cs + k;
#pragma unroll
        for (int p = 0; p < kSlideP; ++p)
            if (p < P) D[(long long)p * cs] = acc[p];
    }
}

__global__ void ddh_reduce_kernel(const float2* __restrict__ Dpart, float2* __restrict__ D, int P, int cs, int nchunk) {
    const int total = P * cs;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int c = 0; c < nchunk; ++c) acc = cadd(acc, Dpart[(long long)c * total + t]);
        D[t] = acc;
    }
}

int cls_of(int N) { return N <= 1024 ? 0 : (N <= 4096 ? 1 : 2); }

// the FDL sum over parts, sliding for P <= kSlideP
int launch_mac(const float2* X, const float2* H, float2* Y, int nsig, int nxb, int nyb, int P, int cs, int mode,
               cudaStream_t st) {
    if (P <= kSlideP) {
        const long long total = (long long)nsig * ((nyb + kSlideRun - 1) / kSlideRun) * cs;
        dmac_slide_kernel<<<(int)std::min<long long>((total + 255) / 256, 152 * 16), 256, 0, st>>>(X, H, Y, nsig, nxb,
                                                                                                    nyb, P, cs, mode);
    } else {
        const long long total = (long long)nsig * nyb * cs;
        dmac_kernel<<<(int)std::min<long long>((total + 255) / 256, 152 * 16), 256, 0, st>>>(X, H, Y, nsig, nxb, nyb,
                                                                                              P, cs, mode);
    }
    return 0;
}

cudaError_t launch_fft(int N, int logN, const FJob* jobs, int njobs, const DPtrs& ptr, const float2* W,
                       cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    const size_t smem = (size_t)12 * N;
    switch (cls_of(N)) {
        case 0:   // one radix-4 butterfly per thread and stage: N / 4 threads
            if (N <= 512) dfft_kernel<128, 1><<<njobs, 128, smem, st>>>(jobs, ptr, N, logN, W, kWlog);
            else dfft_kernel<256, 1><<<njobs, 256, smem, st>>>(jobs, ptr, N, logN, W, kWlog);
            break;
        case 1: dfft_kernel<512, 2><<<njobs, 512, smem, st>>>(jobs, ptr, N, logN, W, kWlog); break;
        default: dfft_kernel<512, 8><<<njobs, 512, smem, st>>>(jobs, ptr, N, logN, W, kWlog); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_ifft(int N, int logN, const IJob* jobs, int njobs, const DPtrs& ptr, const float2* W,
                        cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    const size_t smem = (size_t)12 * N;
    switch (cls_of(N)) {
        case 0:
            if (N <= 512) difft_kernel<128, 1><<<njobs, 128, smem, st>>>(jobs, ptr, N, logN, W, kWlog);
            else difft_kernel<256, 1><<<njobs, 256, smem, st>>>(jobs, ptr, N, logN, W, kWlog);
            break;
        case 1: difft_kernel<512, 2><<<njobs, 512, smem, st>>>(jobs, ptr, N, logN, W, kWlog); break;
        default: difft_kernel<512, 8><<<njobs, 512, smem, st>>>(jobs, ptr, N, logN, W, kWlog); break;
    }
    return cudaGetLastError();
}

}  // namespace

struct pcd_plan {
    int M = 0, B = 0, ir_len = 0;
    long long T = 0;
    std::vector<int> N, P, logN, cs, nb, nbg;
    std::vector<long long> s;
    // workspace offsets (bytes)
    size_t o_W = 0, total = 0;
    std::vector<size_t> o_H, o_X, o_Y, o_Dp, o_D;
    // job tables (device, built at creation): per level and kind, byte offset
    // into d_tab and job count
    struct Tab {
        size_t off = 0;
        int n = 0;
    };
    enum Kind { kFH, kFX, kIY, kFGP, kIGH, kFGX, kIGX, kKinds };
    std::vector<std::array<Tab, kKinds>> tab;
    char* d_tab = nullptr;
    int device = -1;
    std::string err;
    long long launches = 0;
    bool attrs_set = false;   // large-FFT shared memory attributes applied
    ~pcd_plan() {
        if (d_tab) {
            int cur = -1;
            cudaGetDevice(&cur);
            if (device >= 0) cudaSetDevice(device);
            cudaFree(d_tab);
            if (cur >= 0) cudaSetDevice(cur);
        }
    }
};

namespace {

size_t take(size_t& off, size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
}

int dfail(pcd_plan* p, int code, const std::string& m) {
    if (p) p->err = m;
    return code;
}

#define DCK(call, where)                                                                                   \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return dfail(p, PC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct WS {
    char* base;
    template <class T>
    T* at(size_t off) const {
        return reinterpret_cast<T*>(base + off);
    }
};

// launch the table of one kind for level L over the call's buffers
int run_tab(pcd_plan* p, int L, int kind, const DPtrs& ptr, cudaStream_t st) {
    const pcd_plan::Tab& t = p->tab[L][kind];
    if (t.n <= 0) return PC_OK;
    const float2* W = reinterpret_cast<const float2*>(ptr.ws + p->o_W);
    const bool fwd = kind == pcd_plan::kFH || kind == pcd_plan::kFX || kind == pcd_plan::kFGP || kind == pcd_plan::kFGX;
    if (fwd)
        DCK(launch_fft(p->N[L], p->logN[L], reinterpret_cast<const FJob*>(p->d_tab + t.off), t.n, ptr, W, st),
            "window FFT");
    else
        DCK(launch_ifft(p->N[L], p->logN[L], reinterpret_cast<const IJob*>(p->d_tab + t.off), t.n, ptr, W, st),
            "inverse FFT");
    p->launches++;
    return PC_OK;
}

int filter_spectra(pcd_plan* p, const DPtrs& ptr, cudaStream_t st) {
    for (int L = 0; L < p->M; ++L) {
        int r = run_tab(p, L, pcd_plan::kFH, ptr, st);
        if (r) return r;
    }
    return PC_OK;
}

int input_spectra(pcd_plan* p, const DPtrs& ptr, cudaStream_t st) {
    for (int L = 0; L < p->M; ++L) {
        int r = run_tab(p, L, pcd_plan::kFX, ptr, st);
        if (r) return r;
    }
    return PC_OK;
}

// every job table of the plan, relative to the call's buffers (see DPtrs)
int build_tables(pcd_plan* p) {
    std::vector<char> host;
    auto add = [&](auto&& jobs) -> pcd_plan::Tab {
        pcd_plan::Tab t;
        t.off = host.size();
        t.n = (int)jobs.size();
        const size_t bytes = sizeof(jobs[0]) * jobs.size();
        host.resize(host.size() + ((bytes + 255) & ~(size_t)255));
        if (bytes) std::memcpy(host.data() + t.off, jobs.data(), bytes);
        return t;
    };
    const long long T = p->T;
    p->tab.assign(p->M, {});
    for (int L = 0; L < p->M; ++L) {
        const int N = p->N[L], P = p->P[L], nb = p->nb[L], nbg = p->nbg[L];
        const long long row = (long long)sizeof(float2) * p->cs[L];
        const long long sL = p->s[L];
        auto& tb = p->tab[L];
        std::vector<FJob> f;
        std::vector<IJob> v;
        for (int q = 0; q < P; ++q)   // H_q = rfft([0_N, h part q]) / 2N: the window starts N before the part
            f.push_back(FJob{0, p->ir_len, sL + (long long)q * N - N, (long long)p->o_H[L] + q * row,
                             1.0f / (2.0f * N), kSrcH, 2, 0});
        tb[pcd_plan::kFH] = add(f);
        f.clear();
        for (int sg = 0; sg < p->B; ++sg)   // X_b = rfft(x[(b-1)N - s_L, (b+1)N - s_L))
            for (int b = 0; b < nb; ++b)
                f.push_back(FJob{sg * T, T, (long long)(b - 1) * N - sL,
                                 (long long)p->o_X[L] + ((long long)sg * nb + b) * row, 1.0f, kSrcX, 0, 0});
        tb[pcd_plan::kFX] = add(f);
        f.clear();
        for (int sg = 0; sg < p->B; ++sg)   // y block b (level 0 stores, larger levels add)
            for (int b = 0; b < nb; ++b) {
                const long long t0 = (long long)b * N;
                v.push_back(IJob{(long long)p->o_Y[L] + ((long long)sg * nb + b) * row, sg * T + t0, T - t0, 1.0f,
                                 kDstY, L == 0 ? 0 : 1, 0});
            }
        tb[pcd_plan::kIY] = add(v);
        v.clear();
        for (int sg = 0; sg < p->B; ++sg)   // GP_b = rfft([g block b, 0_N])
            for (int b = 0; b < nb; ++b)
                f.push_back(FJob{sg * T, T, (long long)b * N, (long long)p->o_Y[L] + ((long long)sg * nb + b) * row,
                                 1.0f, kSrcG, 1, 0});
        tb[pcd_plan::kFGP] = add(f);
        f.clear();
        for (int q = 0; q < P; ++q) {   // dh[s_L + qN + t] = irfft(D_q)[N - t] / 2N
            const long long t0 = sL + (long long)q * N;
            if (t0 >= p->ir_len) break;
            v.push_back(IJob{(long long)p->o_D[L] + q * row, t0, p->ir_len - t0, 1.0f / (2.0f * N), kDstGH, 2, 0});
        }
        tb[pcd_plan::kIGH] = add(v);
        v.clear();
        for (int sg = 0; sg < p->B; ++sg)   // G'_c = rfft(g[cN + s_L, cN + s_L + 2N)), c < nb + P - 1
            for (int c = 0; c < nbg; ++c)
                f.push_back(FJob{sg * T, T, (long long)c * N + sL,
                                 (long long)p->o_Y[L] + ((long long)sg * nbg + c) * row, 1.0f, kSrcG, 0, 0});
        tb[pcd_plan::kFGX] = add(f);
        f.clear();
        for (int sg = 0; sg < p->B; ++sg)   // dx block b from the adjoint sums (kept in the X rows)
            for (int b = 0; b < nb; ++b) {
                const long long t0 = (long long)b * N;
                v.push_back(IJob{(long long)p->o_X[L] + ((long long)sg * nb + b) * row, sg * T + t0, T - t0, 1.0f,
                                 kDstGX, L == 0 ? 0 : 1, 0});
            }
        tb[pcd_plan::kIGX] = add(v);
        v.clear();
    }
    DCK(cudaGetDevice(&p->device), "cudaGetDevice");
    DCK(cudaMalloc(&p->d_tab, std::max<size_t>(host.size(), 256)), "job table allocation");
    DCK(cudaMemcpy(p->d_tab, host.data(), host.size(), cudaMemcpyHostToDevice), "job table upload");
    return PC_OK;
}

}  // namespace

extern "C" {

pcd_plan* pcd_create(int M, const int* N, int* P, int ir_len, int batch, long long length, char* msg, int msglen) {
    auto put = [&](const char* m) {
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", m);
    };
    if (M < 1 || M > kMaxDLevels || !N || !P || ir_len < 1 || batch < 1 || length < 1) {
        put("bad plan arguments");
        return nullptr;
    }
    std::vector<int> Nv(N, N + M), Pv(P, P + M);
    char m2[256];
    if (pc_check_layout(M, Nv.data(), Pv.data(), ir_len, 1, nullptr, m2, sizeof m2)) {
        put(m2);
        return nullptr;
    }
    if (Nv[M - 1] > kMaxBlockOneCta) {
        put("differentiable levels are limited to blocks of 16384 (larger blocks: pc_* engine)");
        return nullptr;
    }
    if (Nv[0] < 16) {
        put("block size of level 0 must be >= 16");
        return nullptr;
    }
    for (int i = 0; i < M; ++i) P[i] = Pv[i];
    pcd_plan* p = new (std::nothrow) pcd_plan();
    if (!p) return nullptr;
    p->M = M;
    p->B = batch;
    p->ir_len = ir_len;
    p->T = length;
    p->N = Nv;
    p->P = Pv;
    long long s = 0;
    size_t off = 0;
    p->o_W = take(off, sizeof(float2) << kWlog);
    for (int L = 0; L < M; ++L) {
        p->s.push_back(s);
        p->logN.push_back((int)std::lround(std::log2((double)Nv[L])));
        p->cs.push_back(Nv[L] + 2);
        const int nb = (int)((length + Nv[L] - 1) / Nv[L]);
        p->nb.push_back(nb);
        p->nbg.push_back(nb + Pv[L] - 1);   // adjoint windows reach P-1 blocks past the end
        s += (long long)Nv[L] * Pv[L];
    }
    for (int L = 0; L < M; ++L) {
        const size_t cs = p->cs[L];
        p->o_H.push_back(take(off, sizeof(float2) * Pv[L] * cs));
        p->o_X.push_back(take(off, sizeof(float2) * (size_t)batch * p->nb[L] * cs));
        p->o_Y.push_back(take(off, sizeof(float2) * (size_t)batch * p->nbg[L] * cs));
        const size_t nrun = (size_t)(p->nb[L] + kSlideRun - 1) / kSlideRun;
        p->o_Dp.push_back(take(off, sizeof(float2) * std::max<size_t>(kDhChunks, (size_t)batch * nrun) * Pv[L] * cs));
        p->o_D.push_back(take(off, sizeof(float2) * (size_t)Pv[L] * cs));
    }
    p->total = off;
    if (build_tables(p) != PC_OK) {
        put(p->err.c_str());
        delete p;
        return nullptr;
    }
    put("");
    return p;
}

long long pcd_workspace_bytes(const pcd_plan* p) { return p ? (long long)p->total : -1; }

int pcd_forward(pcd_plan* p, const float* d_x, const float* d_h, float* d_y, void* d_ws, void* stream) {
    if (!p || !d_x || !d_h || !d_y || !d_ws) return dfail(p, PC_ERR_ARG, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    WS w{static_cast<char*>(d_ws)};
    const DPtrs ptr{{d_x, d_h, nullptr}, {d_y, nullptr, nullptr}, w.base};
    {
        static thread_local std::vector<float2> Wh;
        if (Wh.empty()) {
            Wh.resize((size_t)1 << kWlog);
            for (size_t m = 0; m < Wh.size(); ++m) {
                const double a = -2.0 * M_PI * (double)m / (double)Wh.size();
                Wh[m] = make_float2((float)std::cos(a), (float)std::sin(a));
            }
        }
        DCK(cudaMemcpyAsync(w.at<float2>(p->o_W), Wh.data(), sizeof(float2) * Wh.size(), cudaMemcpyHostToDevice, st),
            "twiddles");
    }
    if (!p->attrs_set) {
        DCK(cudaFuncSetAttribute(dfft_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384), "attr");
        DCK(cudaFuncSetAttribute(difft_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384), "attr");
        p->attrs_set = true;
    }
    int r = filter_spectra(p, ptr, st);
    if (r) return r;
    r = input_spectra(p, ptr, st);
    if (r) return r;
    for (int L = 0; L < p->M; ++L) {
        const int cs = p->cs[L], nb = p->nb[L];
        float2* Y = w.at<float2>(p->o_Y[L]);
        r = launch_mac(w.at<float2>(p->o_X[L]), w.at<float2>(p->o_H[L]), Y, p->B, nb, nb, p->P[L], cs, 0, st);
        DCK(cudaGetLastError(), "forward MAC");
        p->launches++;
        r = run_tab(p, L, pcd_plan::kIY, ptr, st);
        if (r) return r;
    }
    return PC_OK;
}

int pcd_backward(pcd_plan* p, const float* d_x, const float* d_h, const float* d_gy, float* d_gx, float* d_gh,
                 void* d_ws, int recompute, void* stream) {
    if (!p || !d_gy || !d_ws) return dfail(p, PC_ERR_ARG, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    WS w{static_cast<char*>(d_ws)};
    const DPtrs ptr{{d_x, d_h, d_gy}, {nullptr, d_gh, d_gx}, w.base};
    int r;
    if (recompute) {   // rebuild what the forward pass left in the workspace
        if (!d_x || !d_h) return dfail(p, PC_ERR_ARG, "recompute needs x and h");
        r = filter_spectra(p, ptr, st);
        if (r) return r;
        r = input_spectra(p, ptr, st);
        if (r) return r;
    }
    for (int L = 0; L < p->M; ++L) {
        const int cs = p->cs[L], nb = p->nb[L], nbg = p->nbg[L], P = p->P[L];
        float2* Y = w.at<float2>(p->o_Y[L]);
        // dL/dh first: it needs the input spectra X, which the adjoint pass
        // below overwrites with its own result
        if (d_gh) {
            r = run_tab(p, L, pcd_plan::kFGP, ptr, st);   // GP_b = rfft([g block b, 0_N]) into Y
            if (r) return r;
            float2* Dp = w.at<float2>(p->o_Dp[L]);
            float2* D = w.at<float2>(p->o_D[L]);
            int nchunk = kDhChunks;
            if (P <= kSlideP) {
                const int nrun = (nb + kSlideRun - 1) / kSlideRun;
                nchunk = p->B * nrun;
                const long long tot = (long long)nchunk * cs;
                ddh_slide_kernel<<<(int)std::min<long long>((tot + 255) / 256, 152 * 16), 256, 0, st>>>(
                    w.at<float2>(p->o_X[L]), Y, Dp, p->B, nb, P, cs);
            } else {
                const long long tot = (long long)kDhChunks * P * cs;
                ddh_partial_kernel<<<(int)std::min<long long>((tot + 255) / 256, 152 * 16), 256, 0, st>>>(
                    w.at<float2>(p->o_X[L]), Y, Dp, p->B, nb, P, cs, kDhChunks);
            }
            ddh_reduce_kernel<<<(P * cs + 255) / 256, 256, 0, st>>>(Dp, D, P, cs, nchunk);
            DCK(cudaGetLastError(), "dL/dh reduction");
            p->launches += 2;
            r = run_tab(p, L, pcd_plan::kIGH, ptr, st);   // dh[s_L + qN + t] = irfft(D_q)[N - t] / 2N
            if (r) return r;
        }
        if (d_gx) {
            r = run_tab(p, L, pcd_plan::kFGX, ptr, st);   // G'_c into Y
            if (r) return r;
            float2* Z = w.at<float2>(p->o_X[L]);   // adjoint sums replace the input spectra
            launch_mac(Y, w.at<float2>(p->o_H[L]), Z, p->B, nbg, nb, P, cs, 1, st);
            DCK(cudaGetLastError(), "adjoint MAC");
            p->launches++;
            r = run_tab(p, L, pcd_plan::kIGX, ptr, st);
            if (r) return r;
        }
    }
    return PC_OK;
}

void pcd_destroy(pcd_plan* p) { delete p; }
const char* pcd_last_error(const pcd_plan* p) { return p ? p->err.c_str() : ""; }
long long pcd_kernel_launches(const pcd_plan* p) { return p ? p->launches : 0; }

}  // extern "C"
