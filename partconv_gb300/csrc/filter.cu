// filter.cu -- PartConvFilter on the GPU: the reference's fine-grained,
// per-level API (src/partconv.h:40-114, src/partconv.cpp:70-648 of
// ebattenberg/partconv) with its DelayBuffer / DoubleBuffer schedule
// (src/partconv.cpp:1401-1511).
//
// The host keeps the reference's index state (block counters, ring
// indices, read/write buffer selection); the buffers live on the device and
// runLevel(L) is one kernel: slide the level's 2N window onto the delay
// ring's block, real FFT into ring slot bcurr mod P, the FDL MAC over all
// parts in ascending order, inverse FFT, first N samples into the level's
// double-buffer write side.  This is the API tune.py drives
// (PartConvFilter.setup / bench); the batched engine (engine.cu) runs the
// minimum-latency schedule instead.
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

constexpr int kWlog = 17;   // twiddle table: real transforms of blocks up to 65536

// One level block of the reference schedule.  win_old: the previous delay
// block (first half of the window, updated in place); blk: this call's delay
// block; out: the level's double-buffer write side.
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) filter_level_kernel(int N, int logN, int P, int cs, unsigned bcurr,
                                                          const float2* __restrict__ H, float2* X, float* win_old,
                                                          const float* blk, float* out, const float2* __restrict__ W,
                                                          int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const int tid = threadIdx.x;
    for (int n = tid; n < N; n += NT) {
        const int i = 2 * n;
        const float a = i < N ? win_old[i] : blk[i - N];
        const float b = i + 1 < N ? win_old[i + 1] : blk[i + 1 - N];
        s[n] = make_float2(a, b);
    }
    load_twiddles<NT>(twt, logN, W, wlog);
    __syncthreads();
    // the delay block becomes the first half of the next window
    for (int i = tid; i < N; i += NT) win_old[i] = blk[i];
    const Twiddles tw{twt, logN};
    fft_smem<NT, MAXB>(s, N, logN, tw, false);
    const int slot = (int)(bcurr % (unsigned)P);
    float2* Xs = X + (size_t)slot * cs;
    const int half = N >> 1;
    for (int k = tid; k <= half; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, logN, tw, xk, xnk);
        const int bk = k, bnk = N - k;
        Xs[bk] = xk;
        if (bnk != bk) Xs[bnk] = xnk;
        // Y = sum_p X[(bcurr - p) mod P] H[p], p ascending (partconv.cpp:370-479)
        float2 yk = cmul(xk, H[bk]);
        float2 ynk = cmul(xnk, H[bnk]);
        for (int p = 1; p < P; ++p) {
            const int sl = (int)((bcurr - (unsigned)p + (unsigned)P) % (unsigned)P);
            const float2* Xp = X + (size_t)sl * cs;
            const float2* Hp = H + (size_t)p * cs;
            yk = cadd(yk, cmul(Xp[bk], Hp[bk]));
            ynk = cadd(ynk, cmul(Xp[bnk], Hp[bnk]));
        }
        float2 zk, znk;
        irfft_merge(yk, ynk, k, logN, tw, zk, znk);
        s[k] = zk;
        if (k != 0 && k != half) s[N - k] = znk;
    }
    __syncthreads();
    fft_smem<NT, MAXB>(s, N, logN, tw, true);
    const float* sf = reinterpret_cast<const float*>(s);
    for (int i = tid; i < N; i += NT) out[i] = sf[i];
}

// y = level-0 output + the selected N0-slice of every other level
__global__ void filter_output_kernel(float* y, const float* out0, const float* const* slices, int nslices, int N0) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N0; i += gridDim.x * blockDim.x) {
        float v = out0[i];
        for (int L = 0; L < nslices; ++L) v += slices[L][i];
        y[i] = v;
    }
}

// H rows: rfft([0_N, h_row]) / 2N, one CTA per row (same math as the
// engine's spectra kernel)
template <int NT, int MAXB>
__global__ void __launch_bounds__(NT) filter_spectra_kernel(const float* h, long long h_len, long long start, int N,
                                                            int logN, int cs, float2* H, const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    float2* s = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = s + N;
    const int p = blockIdx.x;
    const long long base = start + (long long)p * N;
    for (int n = threadIdx.x; n < N; n += NT) {
        const int i = 2 * n - N;
        float a = 0.f, b = 0.f;
        if (i >= 0) {
            if (base + i < h_len) a = h[base + i];
            if (base + i + 1 < h_len) b = h[base + i + 1];
        }
        s[n] = make_float2(a, b);
    }
    load_twiddles<NT>(twt, logN, W, wlog);
    __syncthreads();
    const Twiddles tw{twt, logN};
    fft_smem<NT, MAXB>(s, N, logN, tw, false);
    const float inv = 1.0f / (float)(2 * N);
    float2* dst = H + (size_t)p * cs;
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        const int nk = (k == 0) ? 0 : N - k;
        float2 xk, xnk;
        rfft_split(s[k], s[nk], k, logN, tw, xk, xnk);
        dst[k] = make_float2(xk.x * inv, xk.y * inv);
        if (N - k != k) dst[N - k] = make_float2(xnk.x * inv, xnk.y * inv);
    }
}

struct DelayRing {   // src/partconv.cpp:1401-1472
    int frameSize, framesPerBlock, numBlocks, bufferSize;
    int readBlock, writeBlock, writeFrame, readFrameDelay;
    float* d_mem = nullptr;
    void init_indices() {
        readBlock = numBlocks - 1;
        writeBlock = readFrameDelay / framesPerBlock;
        writeFrame = readFrameDelay % framesPerBlock;
    }
};

}  // namespace

struct pcf_handle {
    int verbosity = 0, fs = 44100;
    std::string err;
    bool ready = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    int M = 0;
    std::vector<int> N, P, num_N0, ind_N0;
    std::vector<unsigned> bcurr;
    int start_sync_depth = 0, end_sync_depth = 0;
    std::vector<DelayRing> db;
    std::vector<float*> ybuf[2];   // double buffers per level
    std::vector<int> rd;           // which of the two is the read side
    std::vector<float2*> H, X;
    std::vector<float*> win_old;
    float* out0 = nullptr;         // level 0's latest block (outbuffer[0])
    float* d_y = nullptr;          // output staging
    float* d_x = nullptr;          // input staging
    const float** d_slices = nullptr;
    float2* W = nullptr;
    float* pollute = nullptr;
    std::vector<void*> allocs;
    bool overlap_error = false;
    long long launches = 0;
};

namespace {

int ffail(pcf_handle* h, int code, const std::string& m) {
    h->err = m;
    return code;
}

#define FCK(call, where)                                                                               \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return ffail(h, PC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void ffree(pcf_handle* h) {
    if (h->device >= 0) cudaSetDevice(h->device);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    h->ready = false;
}

template <class T>
cudaError_t dalloc(pcf_handle* h, T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
    if (e == cudaSuccess) {
        h->allocs.push_back(*p);
        e = cudaMemsetAsync(*p, 0, sizeof(T) * std::max<size_t>(n, 1), h->stream);
    }
    return e;
}

int cls_of(int N) { return N <= 1024 ? 0 : (N <= 4096 ? 1 : (N <= kMaxBlockOneCta ? 2 : 3)); }

cudaError_t launch_level(pcf_handle* h, int L) {
    const int N = h->N[L], logN = (int)std::lround(std::log2((double)N)), P = h->P[L], cs = N + 2;
    DelayRing& d = h->db[L];
    const float* blk = d.d_mem + (size_t)d.readBlock * d.framesPerBlock * d.frameSize;
    float* out = h->ybuf[1 - h->rd[L]][L];
    const size_t smem = (size_t)12 * N;
    switch (cls_of(N)) {
        case 3:   // a cluster of CTAs (cluster_fire.cu); H and X in the cluster bin order
            h->launches += 1;
            {
                cudaError_t e = launch_cluster_filter_level(N, P, cs, h->bcurr[L], h->H[L], h->X[L], h->win_old[L],
                                                            blk, out, h->W, kWlog, h->stream);
                if (e == cudaSuccess && L == 0)
                    e = cudaMemcpyAsync(h->out0, out, sizeof(float) * N, cudaMemcpyDeviceToDevice, h->stream);
                return e;
            }
        case 0:
            filter_level_kernel<256, 1><<<1, 256, smem, h->stream>>>(N, logN, P, cs, h->bcurr[L], h->H[L], h->X[L],
                                                                     h->win_old[L], blk, out, h->W, kWlog);
            break;
        case 1:
            filter_level_kernel<512, 2><<<1, 512, smem, h->stream>>>(N, logN, P, cs, h->bcurr[L], h->H[L], h->X[L],
                                                                     h->win_old[L], blk, out, h->W, kWlog);
            break;
        default:
            filter_level_kernel<512, 8><<<1, 512, smem, h->stream>>>(N, logN, P, cs, h->bcurr[L], h->H[L], h->X[L],
                                                                     h->win_old[L], blk, out, h->W, kWlog);
            break;
    }
    h->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && L == 0) e = cudaMemcpyAsync(h->out0, out, sizeof(float) * N, cudaMemcpyDeviceToDevice, h->stream);
    return e;
}

}  // namespace

extern "C" {

pcf_handle* pcf_create(int verbosity, int sample_rate) {
    pcf_handle* h = new (std::nothrow) pcf_handle();
    if (!h) return nullptr;
    h->verbosity = verbosity;
    h->fs = sample_rate;
    return h;
}

int pcf_setup(pcf_handle* h, int M, const int* N, int* P, const float* ir, int ir_len, int relaxed_check) {
    if (!h || !N || !P) return PC_ERR_ARG;
    if (h->ready) return ffail(h, PC_ERR_STATE, "setup called twice without cleanup");
    std::vector<int> Nv(N, N + M), Pv(P, P + M);
    std::vector<float> hv;
    if (ir && ir_len > 0) {
        hv.assign(ir, ir + ir_len);
    } else {   // partconv.cpp:132-142: benching without an IR uses an all-ones IR
        long len = 0;
        for (int i = 0; i < M; ++i) len += (long)Nv[i] * Pv[i];
        hv.assign(std::max<long>(len, 1), 1.0f);
    }
    std::vector<int> delays(std::max(M, 1));
    char msg[256];
    int r = pc_check_layout(M, Nv.data(), Pv.data(), (int)hv.size(), relaxed_check, delays.data(), msg, sizeof msg);
    if (r) return ffail(h, r, msg);
    for (int i = 0; i < M; ++i) P[i] = Pv[i];
    if (Nv[0] < 16) return ffail(h, PC_ERR_LIMIT, "block size of level 0 must be >= 16");
    FCK(cudaGetDevice(&h->device), "cudaGetDevice");
    FCK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
    FCK(prepare_kernels(), "kernel attributes");
    FCK(cudaFuncSetAttribute(filter_level_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384),
        "kernel attributes");
    FCK(cudaFuncSetAttribute(filter_spectra_kernel<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 12 * 16384),
        "kernel attributes");
    h->M = M;
    h->N = Nv;
    h->P = Pv;
    h->num_N0.resize(M);
    h->ind_N0.resize(M);
    h->bcurr.assign(M, 0);
    for (int i = 0; i < M; ++i) {
        h->num_N0[i] = Nv[i] / Nv[0];
        h->ind_N0[i] = h->num_N0[i] - 1;
    }
    // twiddles
    {
        std::vector<float2> W((size_t)1 << kWlog);
        for (size_t m = 0; m < W.size(); ++m) {
            const double a = -2.0 * M_PI * (double)m / (double)W.size();
            W[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        FCK(dalloc(h, &h->W, W.size()), "alloc");
        FCK(cudaMemcpyAsync(h->W, W.data(), sizeof(float2) * W.size(), cudaMemcpyHostToDevice, h->stream), "upload");
        FCK(cudaStreamSynchronize(h->stream), "sync");
    }
    float* d_ir = nullptr;
    FCK(dalloc(h, &d_ir, hv.size()), "alloc");
    FCK(cudaMemcpyAsync(d_ir, hv.data(), sizeof(float) * hv.size(), cudaMemcpyHostToDevice, h->stream), "upload");
    h->db.resize(M);
    h->ybuf[0].resize(M);
    h->ybuf[1].resize(M);
    h->rd.assign(M, 0);
    h->H.resize(M);
    h->X.resize(M);
    h->win_old.resize(M);
    std::vector<SpectraJob> big;   // filter rows of cluster levels, one job per part
    long start = 0;
    for (int L = 0; L < M; ++L) {
        const int n = Nv[L], cs = n + 2, logN = (int)std::lround(std::log2((double)n));
        FCK(dalloc(h, &h->H[L], (size_t)Pv[L] * cs), "alloc");
        FCK(dalloc(h, &h->X[L], (size_t)Pv[L] * cs), "alloc");
        FCK(dalloc(h, &h->win_old[L], n), "alloc");
        FCK(dalloc(h, &h->ybuf[0][L], n), "alloc");
        FCK(dalloc(h, &h->ybuf[1][L], n), "alloc");
        DelayRing& d = h->db[L];
        d.frameSize = Nv[0];
        d.framesPerBlock = n / Nv[0];
        d.readFrameDelay = delays[L] - d.framesPerBlock - 1;
        // a negative read delay (layouts that pass only the relaxed check)
        // would read frames not yet written; reads then report an overlap
        const int rfd = std::max(d.readFrameDelay, 0);
        const int rem = (rfd + 1) % d.framesPerBlock;
        d.bufferSize = rfd + 1 + (d.framesPerBlock - rem);
        d.numBlocks = d.bufferSize / d.framesPerBlock + 1;
        d.bufferSize = d.numBlocks * d.framesPerBlock;
        d.readFrameDelay = rfd;
        d.init_indices();
        FCK(dalloc(h, &d.d_mem, (size_t)d.bufferSize * d.frameSize), "alloc");
        const size_t smem = (size_t)12 * n;
        switch (cls_of(n)) {
            case 3:
                for (int p = 0; p < Pv[L]; ++p) {
                    const long row = start + (long)p * n;
                    const long left = (long)hv.size() - row;
                    big.push_back(SpectraJob{d_ir + std::min<long>(row, (long)hv.size()),
                                             (int)std::max<long>(0, std::min<long>(left, n)), n, logN,
                                             h->H[L] + (size_t)p * cs});
                }
                break;
            case 0:
                filter_spectra_kernel<256, 1><<<Pv[L], 256, smem, h->stream>>>(d_ir, (long long)hv.size(), start, n, logN,
                                                                               cs, h->H[L], h->W, kWlog);
                break;
            case 1:
                filter_spectra_kernel<512, 2><<<Pv[L], 512, smem, h->stream>>>(d_ir, (long long)hv.size(), start, n, logN,
                                                                               cs, h->H[L], h->W, kWlog);
                break;
            default:
                filter_spectra_kernel<512, 8><<<Pv[L], 512, smem, h->stream>>>(d_ir, (long long)hv.size(), start, n, logN,
                                                                               cs, h->H[L], h->W, kWlog);
                break;
        }
        FCK(cudaGetLastError(), "filter spectra");
        if (cls_of(n) < 3) h->launches += 1;
        start += (long)n * Pv[L];
    }
    if (!big.empty()) {
        SpectraJob* d_jobs = nullptr;
        FCK(dalloc(h, &d_jobs, big.size()), "alloc");
        FCK(cudaMemcpyAsync(d_jobs, big.data(), sizeof(SpectraJob) * big.size(), cudaMemcpyHostToDevice, h->stream),
            "upload");
        FCK(launch_cluster_spectra((int)big.size(), d_jobs, h->W, kWlog, h->stream), "filter spectra");
        h->launches += 1;
        FCK(cudaStreamSynchronize(h->stream), "spectra sync");   // before the job table goes out of scope
    }
    FCK(dalloc(h, &h->out0, Nv[0]), "alloc");
    FCK(dalloc(h, &h->d_y, Nv[0]), "alloc");
    FCK(dalloc(h, &h->d_x, Nv[0]), "alloc");
    FCK(dalloc(h, &h->d_slices, std::max(M, 1)), "alloc");
    FCK(cudaStreamSynchronize(h->stream), "setup sync");
    h->ready = true;
    h->overlap_error = false;
    return PC_OK;
}

int pcf_sync_levels(pcf_handle* h, int relaxed) {
    if (!h || !h->ready) return PC_ERR_STATE;
    // partconv.cpp:568-603
    h->start_sync_depth = 0;
    h->end_sync_depth = 0;
    for (int L = 0; L < h->M; ++L) {
        h->ind_N0[L]++;
        if (h->ind_N0[L] == h->num_N0[L]) {
            h->ind_N0[L] = 0;
            h->start_sync_depth = L;
            if (relaxed) h->end_sync_depth = L;
        } else if (!relaxed && h->ind_N0[L] == h->num_N0[L] - 1) {
            h->end_sync_depth = L;
        }
    }
    return PC_OK;
}

int pcf_input(pcf_handle* h, const float* x) {
    if (!h || !h->ready || !x) return PC_ERR_ARG;
    cudaSetDevice(h->device);
    const int N0 = h->N[0];
    FCK(cudaMemcpyAsync(h->d_x, x, sizeof(float) * N0, cudaMemcpyHostToDevice, h->stream), "input copy");
    for (int L = 0; L < h->M; ++L) {   // partconv.cpp:605-613, DelayBuffer::write :1430-1443
        DelayRing& d = h->db[L];
        const int frame = d.writeBlock * d.framesPerBlock + d.writeFrame;
        FCK(cudaMemcpyAsync(d.d_mem + (size_t)frame * d.frameSize, h->d_x, sizeof(float) * N0, cudaMemcpyDeviceToDevice,
                            h->stream),
            "delay write");
        if (++d.writeFrame == d.framesPerBlock) {
            d.writeFrame = 0;
            if (++d.writeBlock == d.numBlocks) d.writeBlock = 0;
        }
        if (L <= h->start_sync_depth)
            if (++d.readBlock == d.numBlocks) d.readBlock = 0;
    }
    return PC_OK;
}

int pcf_run_level(pcf_handle* h, int L) {
    if (!h || !h->ready) return PC_ERR_STATE;
    if (L < 0 || L >= h->M) return ffail(h, PC_ERR_ARG, "level out of range");
    cudaSetDevice(h->device);
    DelayRing& d = h->db[L];
    if (d.readBlock == d.writeBlock) {   // partconv.cpp:1449-1455 exits here
        h->overlap_error = true;
        return ffail(h, PC_ERR_STATE, "DelayBuffer read block equals write block");
    }
    FCK(launch_level(h, L), "runLevel");
    h->bcurr[L]++;
    return PC_OK;
}

int pcf_output(pcf_handle* h, float* y, int relaxed) {
    if (!h || !h->ready || !y) return PC_ERR_ARG;
    cudaSetDevice(h->device);
    // partconv.cpp:616-648
    std::vector<const float*> sl;
    for (int L = 1; L < h->M; ++L) {
        if (L <= h->end_sync_depth) h->rd[L] = 1 - h->rd[L];
        int rb = relaxed ? h->ind_N0[L] : h->ind_N0[L] + 1;
        if (rb == h->num_N0[L]) rb = 0;
        sl.push_back(h->ybuf[h->rd[L]][L] + (size_t)h->N[0] * rb);
    }
    if (!sl.empty())
        FCK(cudaMemcpyAsync(h->d_slices, sl.data(), sizeof(float*) * sl.size(), cudaMemcpyHostToDevice, h->stream),
            "slice table");
    filter_output_kernel<<<1, 256, 0, h->stream>>>(h->d_y, h->out0, h->d_slices, (int)sl.size(), h->N[0]);
    FCK(cudaGetLastError(), "output");
    h->launches += 1;
    FCK(cudaMemcpyAsync(y, h->d_y, sizeof(float) * h->N[0], cudaMemcpyDeviceToHost, h->stream), "output copy");
    FCK(cudaStreamSynchronize(h->stream), "output sync");
    return PC_OK;
}

int pcf_reset(pcf_handle* h) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return PC_OK;
    cudaSetDevice(h->device);
    std::fill(h->bcurr.begin(), h->bcurr.end(), 0u);
    for (int L = 0; L < h->M; ++L) {   // partconv.cpp:492-506
        h->ind_N0[L] = h->num_N0[L] - 1;
        const int n = h->N[L];
        FCK(cudaMemsetAsync(h->win_old[L], 0, sizeof(float) * n, h->stream), "reset");
        FCK(cudaMemsetAsync(h->X[L], 0, sizeof(float2) * (size_t)h->P[L] * (n + 2), h->stream), "reset");
        FCK(cudaMemsetAsync(h->ybuf[0][L], 0, sizeof(float) * n, h->stream), "reset");
        FCK(cudaMemsetAsync(h->ybuf[1][L], 0, sizeof(float) * n, h->stream), "reset");
        DelayRing& d = h->db[L];
        FCK(cudaMemsetAsync(d.d_mem, 0, sizeof(float) * (size_t)d.bufferSize * d.frameSize, h->stream), "reset");
        d.init_indices();
    }
    // like the reference, reset leaves level 0's last block (outbuffer[0])
    // in place: the first output_relaxed() after a reset returns it
    FCK(cudaStreamSynchronize(h->stream), "reset sync");
    h->overlap_error = false;
    return PC_OK;
}

double pcf_bench(pcf_handle* h, int L, int trials, int pollute_every, double max_time, double* bench_data) {
    // partconv.cpp:508-566: mean time of runLevel(L), polluting caches every
    // pollute_every trials (here: a write larger than the GPU's L2)
    if (!h || !h->ready || L < 0 || L >= h->M || trials < 1) return -1.0;
    cudaSetDevice(h->device);
    const size_t pollute_n = (size_t)64 << 20;   // 256 MB
    if (pollute_every > 0 && !h->pollute) {
        if (dalloc(h, &h->pollute, pollute_n) != cudaSuccess) return -1.0;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double total = 0.0;
    int trial, cnt = 0;
    for (trial = 0; trial < trials; trial++) {
        if (pollute_every > 0 && cnt++ == pollute_every) {
            cnt = 0;
            cudaMemsetAsync(h->pollute, trial & 0xff, sizeof(float) * pollute_n, h->stream);
        }
        DelayRing& d = h->db[L];
        if (d.readBlock == d.writeBlock)   // keep the ring consistent while benching
            if (++d.readBlock == d.numBlocks) d.readBlock = 0;
        cudaEventRecord(a, h->stream);
        if (launch_level(h, L) != cudaSuccess) break;
        cudaEventRecord(b, h->stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        total += ms * 1e-3;
        h->bcurr[L] += 2;   // runLevel's increment plus the bench loop's (partconv.cpp:544-546)
        if (total > max_time) {
            trial++;
            break;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double mean = total / std::max(trial, 1);
    if (bench_data) {
        const int value = (int)(100.0 * mean / ((double)h->N[L] / h->fs));
        bench_data[2 * L] = value;
        bench_data[2 * L + 1] = value;
    }
    pcf_reset(h);
    return mean;
}

int pcf_cleanup(pcf_handle* h) {
    if (!h) return PC_ERR_ARG;
    ffree(h);
    return PC_OK;
}

void pcf_destroy(pcf_handle* h) {
    if (!h) return;
    ffree(h);
    delete h;
}

const char* pcf_last_error(const pcf_handle* h) { return h ? h->err.c_str() : ""; }

int pcf_get_parts(const pcf_handle* h, int* P) {
    if (!h || !P) return PC_ERR_ARG;
    for (int i = 0; i < h->M; ++i) P[i] = h->P[i];
    return PC_OK;
}

int pcf_overlap_error(const pcf_handle* h) { return h && h->overlap_error ? 1 : 0; }

}  // extern "C"
