// cluster_fire.cu -- level blocks of 16384 < N <= 65536 samples, computed by
// a thread-block cluster of 8 CTAs that exchange data through distributed
// shared memory (sm_90+ clusters; sm_103a here).
//
// A level of block N transforms 2N real samples: the N-point complex FFT of
// z[j] = x[2j] + i x[2j+1] plus the real split pass (as in fft_smem.cuh).
// N complex points (512 KB at N = 65536) do not fit one CTA's shared memory,
// so the transform is the four-step factorisation n = C m (C = 8 CTAs,
// m = n / 8 points each):
//   X[k1 + C k2] = sum_j2 w_m^(j2 k2) [ w_n^(j2 k1) sum_j1 x[j1 m + j2] w_C^(j1 k1) ]
// CTA r holds x[r m .. (r+1) m); a column pass computes the C-point DFTs
// over j1 (one column per thread, its C values read from and written back to
// the C CTAs' shared memory) and applies w_n^(j2 k1); each CTA then runs an
// m-point Stockham FFT in its own shared memory and holds the bins
// k = r + C k2.  The inverse runs the same steps backwards.
//
// Filter spectra, spectrum ring and partial sums of such a level are stored
// with bin k at position (k mod C) m + k / C (bin N at N), so every CTA
// streams one contiguous range of each row; the spread tasks, which work bin
// by bin, need no change.  The real split pairs bin k (CTA r) with bin N - k
// (CTA (C - r) mod C); each CTA handles half of its pairs and writes the
// partner's results into the partner's shared memory.
//
// Work of one fire (the same as fire_body in step_kernels.cu for the large
// classes): window from the input ring (the newest N0 samples from this
// call's input for a level that fires within its step), forward transform,
// X_b stored in ring slot b mod P, Y = X_b H_0 (+ X_{b-1} H_1 for a deferred
// level) + partial-sum rows, inverse transform, first N samples to the
// level's output ring.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "engine_types.h"
#include "fft_smem.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace pcg {

namespace {

constexpr int kC = kClusterCtas;            // CTAs per cluster
constexpr int kNT = 512;                    // threads per CTA
constexpr int kMaxM = kClusterMaxN / kC;    // points per CTA
constexpr int kMaxB = kMaxM / 4 / kNT;      // radix-4 butterflies per thread and stage
constexpr int kMaxPairs = (kMaxM / 2 + 1 + kNT - 1) / kNT;   // split pairs per thread

struct Geo {
    int n, logn, m, logm, rank;
    const float2* W;   // global table exp(-2 pi i t / 2^wlog)
    int wlog;
    // exp(-2 pi i e / n), 0 <= e (taken mod n)
    __device__ __forceinline__ float2 wn(long long e) const {
        return __ldg(&W[(size_t)(e & (n - 1)) << (wlog - logn)]);
    }
    // exp(-i pi k / n) = exp(-2 pi i k / 2n), 0 <= k <= n
    __device__ __forceinline__ float2 wsplit(int k) const { return __ldg(&W[(size_t)k << (wlog - logn - 1)]); }
};

// Forward column pass over this CTA's share of columns: 8-point DFTs over
// the CTAs, twiddle w_n^(j2 k1), results back in place.  Ends with a
// cluster barrier.
__device__ void column_pass_fwd(const Geo& g, float2* const* rem, cg::cluster_group& cl) {
    const int cols = g.m / kC;
    for (int c = threadIdx.x; c < cols; c += kNT) {
        const int j2 = g.rank * cols + c;
        const int p = sidx<true>(j2);
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = rem[r][p];
        dft8(v, false);
#pragma unroll
        for (int k1 = 1; k1 < 8; ++k1) v[k1] = cmul(v[k1], g.wn((long long)j2 * k1));
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) rem[k1][p] = v[k1];
    }
    cl.sync();
}

// Inverse column pass: conj(w_n^(k1 j2)) then the inverse 8-point DFT over
// k1; output index j2 + m j1 goes to CTA j1.  Ends with a cluster barrier.
__device__ void column_pass_inv(const Geo& g, float2* const* rem, cg::cluster_group& cl) {
    const int cols = g.m / kC;
    for (int c = threadIdx.x; c < cols; c += kNT) {
        const int j2 = g.rank * cols + c;
        const int p = sidx<true>(j2);
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = rem[r][p];
#pragma unroll
        for (int k1 = 1; k1 < 8; ++k1) v[k1] = cmul(v[k1], cconj(g.wn((long long)j2 * k1)));
        dft8(v, true);
#pragma unroll
        for (int j1 = 0; j1 < 8; ++j1) rem[j1][p] = v[j1];
    }
    cl.sync();
}

// The split pairs this CTA handles: pair index i (0 <= i < npairs) ->
// own position k2, partner CTA and position, and the two bins.
struct Pair {
    int k2, pr, pk2, k, nk;   // nk == k: self-paired; k == 0: bins 0 and n
};
__device__ __forceinline__ int pair_count(const Geo& g) { return g.rank == 0 ? g.m / 2 + 1 : g.m / 2; }
__device__ __forceinline__ Pair pair_at(const Geo& g, int i) {
    Pair q;
    q.k2 = i;
    q.k = g.rank + kC * i;
    if (g.rank == 0) {
        q.pr = 0;
        q.pk2 = (g.m - i) & (g.m - 1);   // k2 = 0 pairs bin 0 with bin n (no partner read)
        q.nk = (i == 0) ? g.n : g.n - q.k;
    } else {
        q.pr = kC - g.rank;
        q.pk2 = g.m - 1 - i;
        q.nk = g.n - q.k;
    }
    return q;
}

// X[k], X[n-k] from Z[k], Z[n-k] (the split of fft_smem.cuh's rfft_split
// with the twiddle from the global table); k == 0 gives X[0] and X[n].
__device__ __forceinline__ void split_pair(const Geo& g, float2 zk, float2 znk, int k, float2& xk, float2& xnk) {
    if (k == 0) {
        xk = make_float2(zk.x + zk.y, 0.0f);
        xnk = make_float2(zk.x - zk.y, 0.0f);
        return;
    }
    const float2 E = make_float2(0.5f * (zk.x + znk.x), 0.5f * (zk.y - znk.y));
    const float2 O = make_float2(0.5f * (zk.y + znk.y), -0.5f * (zk.x - znk.x));
    const float2 wO = cmul(g.wsplit(k), O);
    xk = cadd(E, wO);
    xnk = cconj(csub(E, wO));
}

// Z'[k], Z'[n-k] from Y[k], Y[n-k] (irfft_merge with the global twiddle;
// imaginary parts of Y[0] and Y[n] ignored, as FFTW's c2r does).
__device__ __forceinline__ void merge_pair(const Geo& g, float2 yk, float2 ynk, int k, float2& zk, float2& znk) {
    if (k == 0) {
        yk.y = 0.0f;
        ynk.y = 0.0f;
    }
    const float2 A = make_float2(yk.x + ynk.x, yk.y - ynk.y);
    const float2 B = make_float2(yk.x - ynk.x, yk.y + ynk.y);
    const float2 w = g.wsplit(k);
    const float2 cB = cmul(cconj(w), B);
    zk = make_float2(A.x - cB.y, A.y + cB.x);
    const float2 wcB = cmul(w, cconj(B));
    znk = make_float2(A.x - wcB.y, -A.y + wcB.x);
}

__device__ __forceinline__ int bin_pos(const Geo& g, int k) { return k == g.n ? g.n : (k & (kC - 1)) * g.m + (k >> 3); }

// Shared memory: transform buffer (m points, conflict-free placement) and
// the quarter-wave twiddles of the m-point transform.
__device__ __forceinline__ void setup_geo(Geo& g, int N, const float2* W, int wlog, float2* tw_tab) {
    g.n = N;
    g.logn = 31 - __clz(N);
    g.m = N / kC;
    g.logm = g.logn - 3;
    g.rank = (int)cg::this_cluster().block_rank();
    g.W = W;
    g.wlog = wlog;
    load_twiddles_sw<kNT>(tw_tab, g.logm, W, wlog);
}

}  // namespace

// One fire per cluster: task blockIdx.x / 8 of this launch.
__global__ void __cluster_dims__(kC, 1, 1) __launch_bounds__(kNT)
    cluster_fire_kernel(Bank bank, const Task* __restrict__ tasks, RunState rs_val, const RunState* rs_dev,
                        int step_in_batch) {
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(16) Task tk;
    __shared__ __align__(16) RunState rs;
    cg::cluster_group cl = cg::this_cluster();
    cudaTriggerProgrammaticLaunchCompletion();
    const int tid = threadIdx.x;
    const int ti = blockIdx.x / kC;
    if (tid < 12) {
        reinterpret_cast<int4*>(&tk)[tid] = __ldg(reinterpret_cast<const int4*>(tasks + ti) + tid);
    } else if (tid >= 32 && tid < 37) {
        const int j = tid - 32;
        if (rs_dev) reinterpret_cast<int4*>(&rs)[j] = __ldcg(reinterpret_cast<const int4*>(rs_dev) + j);
    }
    if (!rs_dev && tid == 64) rs = rs_val;
    float2* S = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = S + kMaxM;
    __syncthreads();
    Geo g;
    setup_geo(g, tk.N, bank.W, bank.wlog, twt);
    float2* rem[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) rem[r] = cl.map_shared_rank(S, r);

    long long c = rs.step_base + step_in_batch;
    const long long io_step = c - rs.io.step0;
    c -= tk.origin;
    const int N = tk.N, P = tk.P, cs = tk.cs, N0 = bank.N0;
    const long long q = c + 1 + tk.s_blocks;
    const long long b = q / tk.T - 1;
    const bool dfer = tk.dfer != 0;
    const long long t_end = (c + 1) * (long long)N0;   // end of the window (exclusive)
    const float* in = rs.io.in + io_step * rs.io.in_step + (long long)tk.in_ch * rs.io.in_ch;
    const long long isamp = rs.io.in_sample;

    // earlier steps' kernels have completed (input ring, spectra, partial sums)
    cudaGridDependencySynchronize();

    // ---- window: complex points j = rank m + j2 <- samples 2j, 2j + 1 ---------------
    {
        const long long w0 = t_end - 2LL * N;       // first window sample
        const long long fresh = 2LL * N - N0;       // window index of this step's first sample
        for (int j2 = tid; j2 < g.m; j2 += kNT) {
            const long long t = 2LL * (g.rank * (long long)g.m + j2);   // window index
            float2 v;
            if (!dfer && t >= fresh) {
                const long long i = t - fresh;
                v = make_float2(in[i * isamp] * tk.scale, in[(i + 1) * isamp] * tk.scale);
            } else {
                v = __ldcg(reinterpret_cast<const float2*>(tk.xring + ((w0 + t) & tk.rin_mask)));
            }
            S[sidx<true>(j2)] = v;
        }
    }
    cl.sync();
    column_pass_fwd(g, rem, cl);
    const Twiddles tw{twt, g.logm};
    fft_smem<kNT, kMaxB, true>(S, g.m, g.logm, tw, false);
    cl.sync();

    // ---- split, FDL MAC, inverse merge: Y = X_b H_0 (+ X_{b-1} H_1) + Yp ----------
    const bool two = dfer;
    const bool use_x1 = two && P >= 2;
    const bool use_yp = (two && P >= 3) || (!two && P >= 2);
    const int slot = (int)(((b % P) + P) % P);
    float2* Xs = tk.X + (size_t)slot * cs;
    const float2* X1 = tk.X + (size_t)((((b - 1) % P) + P) % P) * cs;
    const float2* Ypb = tk.Yp + (two ? (size_t)(b & 1) * cs : 0);
    const int npart = tk.k0 > 0 ? tk.k0 : 1;
    const size_t rstride = 2 * (size_t)cs;
    auto mac = [&](int pos, float2 x) {
        float2 y = cmul(x, __ldg(&tk.H[pos]));
        if (use_x1) y = cadd(y, cmul(__ldcg(&X1[pos]), __ldg(&tk.H[cs + pos])));
        if (use_yp)
            for (int qr = 0; qr < npart; ++qr) y = cadd(y, __ldcg(&Ypb[qr * rstride + pos]));
        return y;
    };
    const int np = pair_count(g);
    float2 zo[kMaxPairs][2];
#pragma unroll
    for (int i = 0; i < kMaxPairs; ++i) {
        const int pi = tid + i * kNT;
        if (pi >= np) continue;
        const Pair pq = pair_at(g, pi);
        const float2 zk = S[sidx<true>(pq.k2)];
        const bool self = (pq.nk == pq.k);
        const float2 znk = (pq.k == 0 || self) ? zk : rem[pq.pr][sidx<true>(pq.pk2)];
        float2 xk, xnk;
        split_pair(g, zk, znk, pq.k, xk, xnk);
        const int pk = bin_pos(g, pq.k), pnk = bin_pos(g, pq.nk);
        Xs[pk] = xk;
        if (!self) Xs[pnk] = xnk;
        const float2 yk = mac(pk, xk);
        const float2 ynk = self ? yk : mac(pnk, xnk);
        merge_pair(g, yk, ynk, pq.k, zo[i][0], zo[i][1]);
    }
    cl.sync();   // every CTA has read the forward spectra
#pragma unroll
    for (int i = 0; i < kMaxPairs; ++i) {
        const int pi = tid + i * kNT;
        if (pi >= np) continue;
        const Pair pq = pair_at(g, pi);
        S[sidx<true>(pq.k2)] = zo[i][0];
        if (pq.k != 0 && pq.nk != pq.k) rem[pq.pr][sidx<true>(pq.pk2)] = zo[i][1];
    }
    cl.sync();
    fft_smem<kNT, kMaxB, true>(S, g.m, g.logm, tw, true);
    cl.sync();
    column_pass_inv(g, rem, cl);

    // ---- output: complex points [0, n/2) are the block's first N samples -----------
    if (g.rank < kC / 2) {
        const long long t0 = b * (long long)N + 2LL * g.rank * g.m;
        for (int j2 = tid; j2 < g.m; j2 += kNT)
            *reinterpret_cast<float2*>(tk.yring + ((t0 + 2 * j2) & tk.rmask)) = S[sidx<true>(j2)];
    }
}

// Filter spectra of cluster levels: H = rfft([0_N, h_row]) / 2N, one row per
// cluster, stored in the cluster bin order.
__global__ void __cluster_dims__(kC, 1, 1) __launch_bounds__(kNT)
    cluster_spectra_kernel(const SpectraJob* __restrict__ jobs, const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    cg::cluster_group cl = cg::this_cluster();
    const SpectraJob jb = jobs[blockIdx.x / kC];
    float2* S = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = S + kMaxM;
    Geo g;
    setup_geo(g, jb.N, W, wlog, twt);
    float2* rem[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) rem[r] = cl.map_shared_rank(S, r);
    const int N = jb.N;
    for (int j2 = threadIdx.x; j2 < g.m; j2 += kNT) {
        const int t = 2 * (g.rank * g.m + j2) - N;   // tap index of window sample 2j
        float a = 0.f, bb = 0.f;
        if (t >= 0) {
            if (t < jb.len) a = jb.src[t];
            if (t + 1 < jb.len) bb = jb.src[t + 1];
        }
        S[sidx<true>(j2)] = make_float2(a, bb);
    }
    cl.sync();
    column_pass_fwd(g, rem, cl);
    const Twiddles tw{twt, g.logm};
    fft_smem<kNT, kMaxB, true>(S, g.m, g.logm, tw, false);
    cl.sync();
    const float inv = 1.0f / (float)(2 * N);
    const int np = pair_count(g);
    for (int pi = threadIdx.x; pi < np; pi += kNT) {
        const Pair pq = pair_at(g, pi);
        const float2 zk = S[sidx<true>(pq.k2)];
        const bool self = (pq.nk == pq.k);
        const float2 znk = (pq.k == 0 || self) ? zk : rem[pq.pr][sidx<true>(pq.pk2)];
        float2 xk, xnk;
        split_pair(g, zk, znk, pq.k, xk, xnk);
        jb.dst[bin_pos(g, pq.k)] = make_float2(xk.x * inv, xk.y * inv);
        if (!self) jb.dst[bin_pos(g, pq.nk)] = make_float2(xnk.x * inv, xnk.y * inv);
    }
    cl.sync();   // no CTA leaves while others may still read its shared memory
}

// PartConvFilter::runLevel (src/partconv.cpp:354-490) for one level with
// 16384 < N <= 65536, one cluster: window = [win_old | blk] (the previous and
// this call's delay block), forward transform into ring slot bcurr mod P,
// Y = sum_p X[(bcurr - p) mod P] H[p] with p ascending, inverse transform,
// the first N samples to out.  win_old then holds blk.  H and the ring use
// the cluster bin order.
__global__ void __cluster_dims__(kC, 1, 1) __launch_bounds__(kNT)
    cluster_filter_level_kernel(int N, int P, int cs, unsigned bcurr, const float2* __restrict__ H, float2* X,
                                float* win_old, const float* blk, float* out, const float2* W, int wlog) {
    extern __shared__ float4 dyn_smem[];
    cg::cluster_group cl = cg::this_cluster();
    const int tid = threadIdx.x;
    float2* S = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = S + kMaxM;
    Geo g;
    setup_geo(g, N, W, wlog, twt);
    float2* rem[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) rem[r] = cl.map_shared_rank(S, r);
    // complex point j = rank m + j2 <- window samples 2j, 2j + 1; CTAs of
    // rank < kC / 2 read win_old, the others blk
    const int w0 = 2 * g.rank * g.m;
    for (int j2 = tid; j2 < g.m; j2 += kNT) {
        const int t = w0 + 2 * j2;
        S[sidx<true>(j2)] = t < N ? *reinterpret_cast<const float2*>(win_old + t)
                                  : *reinterpret_cast<const float2*>(blk + (t - N));
    }
    __syncthreads();
    // each CTA overwrites only the part of win_old it has read
    if (w0 < N)
        for (int i = tid; i < 2 * g.m; i += kNT) win_old[w0 + i] = blk[w0 + i];
    cl.sync();
    column_pass_fwd(g, rem, cl);
    const Twiddles tw{twt, g.logm};
    fft_smem<kNT, kMaxB, true>(S, g.m, g.logm, tw, false);
    cl.sync();

    const unsigned uP = (unsigned)P;
    float2* Xs = X + (size_t)(bcurr % uP) * cs;
    auto mac = [&](int pos, float2 x) {
        float2 y = cmul(x, __ldg(&H[pos]));
        for (int p = 1; p < P; ++p) {
            const unsigned sl = (bcurr - (unsigned)p + uP) % uP;
            y = cadd(y, cmul(__ldcg(&X[(size_t)sl * cs + pos]), __ldg(&H[(size_t)p * cs + pos])));
        }
        return y;
    };
    const int np = pair_count(g);
    float2 zo[kMaxPairs][2];
#pragma unroll
    for (int i = 0; i < kMaxPairs; ++i) {
        const int pi = tid + i * kNT;
        if (pi >= np) continue;
        const Pair pq = pair_at(g, pi);
        const float2 zk = S[sidx<true>(pq.k2)];
        const bool self = (pq.nk == pq.k);
        const float2 znk = (pq.k == 0 || self) ? zk : rem[pq.pr][sidx<true>(pq.pk2)];
        float2 xk, xnk;
        split_pair(g, zk, znk, pq.k, xk, xnk);
        const int pk = bin_pos(g, pq.k), pnk = bin_pos(g, pq.nk);
        Xs[pk] = xk;
        if (!self) Xs[pnk] = xnk;
        const float2 yk = mac(pk, xk);
        const float2 ynk = self ? yk : mac(pnk, xnk);
        merge_pair(g, yk, ynk, pq.k, zo[i][0], zo[i][1]);
    }
    cl.sync();   // every CTA has read the forward spectra
#pragma unroll
    for (int i = 0; i < kMaxPairs; ++i) {
        const int pi = tid + i * kNT;
        if (pi >= np) continue;
        const Pair pq = pair_at(g, pi);
        S[sidx<true>(pq.k2)] = zo[i][0];
        if (pq.k != 0 && pq.nk != pq.k) rem[pq.pr][sidx<true>(pq.pk2)] = zo[i][1];
    }
    cl.sync();
    fft_smem<kNT, kMaxB, true>(S, g.m, g.logm, tw, true);
    cl.sync();
    column_pass_inv(g, rem, cl);
    // complex points [0, n/2) are the block's first N samples
    if (g.rank < kC / 2)
        for (int j2 = tid; j2 < g.m; j2 += kNT) *reinterpret_cast<float2*>(out + w0 + 2 * j2) = S[sidx<true>(j2)];
}

size_t cluster_smem_bytes() { return sizeof(float2) * (size_t)kMaxM + sizeof(float2) * (size_t)(kMaxM / 2); }

cudaError_t prepare_cluster_kernels() {
    cudaError_t e = cudaFuncSetAttribute(cluster_fire_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cluster_smem_bytes());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(cluster_filter_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)cluster_smem_bytes());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(cluster_spectra_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)cluster_smem_bytes());
}

cudaError_t launch_cluster_filter_level(int N, int P, int cs, unsigned bcurr, const float2* H, float2* X,
                                        float* win_old, const float* blk, float* out, const float2* W, int wlog,
                                        cudaStream_t st) {
    cluster_filter_level_kernel<<<kC, kNT, cluster_smem_bytes(), st>>>(N, P, cs, bcurr, H, X, win_old, blk, out, W,
                                                                       wlog);
    return cudaGetLastError();
}

cudaError_t launch_cluster_fire(int ntasks, const Bank& bank, const Task* tasks, const RunState& rs,
                                const RunState* rs_dev, int step_in_batch, cudaStream_t st, bool pdl, int prio) {
    if (ntasks <= 0) return cudaSuccess;
    static int least = 0, greatest = 0;
    static const bool have_range = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess;
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
    cfg.gridDim = dim3(ntasks * kC);
    cfg.blockDim = dim3(kNT);
    cfg.dynamicSmemBytes = cluster_smem_bytes();
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, cluster_fire_kernel, bank, tasks, rs, rs_dev, step_in_batch);
}

cudaError_t launch_cluster_spectra(int njobs, const SpectraJob* jobs, const float2* W, int wlog, cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    cluster_spectra_kernel<<<njobs * kC, kNT, cluster_smem_bytes(), st>>>(jobs, W, wlog);
    return cudaGetLastError();
}

}  // namespace pcg
