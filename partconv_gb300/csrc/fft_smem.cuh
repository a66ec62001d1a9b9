// fft_smem.cuh -- shared-memory Stockham FFT and the real-FFT split passes
// used by the level kernels.
//
// A real transform of length 2N (one FDL block window) is computed as the
// N-point complex FFT of z[n] = x[2n] + i x[2n+1] followed by the split
// post-pass (X[k] = E[k] + w^k O[k], X[N-k] = conj(E[k] - w^k O[k]),
// w = e^{-i pi / N}); the inverse runs the matching pre-pass and an
// unnormalised inverse N-point FFT, giving FFTW c2r's unnormalised output
// (the 1/nfft factor lives in the filter spectra, as in
// src/partconv.cpp:216-228 of ebattenberg/partconv).
//
// The complex FFT is the Stockham autosort formulation (Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors",
// SC 2008): radix-4 stages then one radix-2 stage when log2 N is odd.  Each
// stage stages its butterflies' inputs in registers, so one N-element
// shared buffer suffices (a barrier separates the reads from the writes).
//
// Twiddles come from a quarter-wave table in shared memory,
// tw[m] = exp(-2 pi i m / 2N) for 0 <= m < N/2, filled once per CTA from a
// global table computed in double on the host; other angles follow by
// quarter-turn symmetry.  The radix-4 stages in the conflict-free placement
// (the large transforms) read only w^k and form w^2k and w^3k by complex
// products (about one float32 rounding more per factor).
#pragma once
#include <cuda_runtime.h>

namespace pcg {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Placement of quarter-wave table entry m (< 2^15) in its conflict-free
// form: the low four bits XORed with the three nibbles above them, so 16
// threads reading entries k 2^s (k consecutive, any s), or 16 consecutive
// entries, hit distinct 8-byte bank pairs.
__device__ __forceinline__ int twsw(int m) { return m ^ (((m >> 4) ^ (m >> 8) ^ (m >> 12)) & 15); }

// Quarter-wave twiddle table of a 2N-point circle in shared memory.
struct Twiddles {
    const float2* tab;   // N/2 entries (entry m at tab[twsw(m)] when read with SW)
    int logN;            // log2 N

    // exp(-+2 pi i a / 2^lg), 0 <= a < 2^lg, 2^lg <= 2N
    template <bool SW = false>
    __device__ __forceinline__ float2 get(int a, int lg, bool inv) const {
        const int a2 = a << (logN + 1 - lg);           // index on the 2N circle
        const int q = a2 >> (logN - 1);                // quadrant
        const int m = a2 & ((1 << (logN - 1)) - 1);
        const float2 t = tab[SW ? twsw(m) : m];
        // quadrant q rotates by (-i)^q: odd q swaps (x, y) -> (y, -x), q >= 2 negates
        // (selects rather than a switch, so a warp does not diverge)
        const bool odd = (q & 1) != 0;
        const float sg = (q & 2) ? -1.0f : 1.0f;
        float2 w = make_float2(sg * (odd ? t.y : t.x), sg * (odd ? -t.x : t.y));
        return inv ? cconj(w) : w;
    }

    // get() for a first-quadrant angle, 0 <= a < 2^(lg-2): one table read,
    // no quadrant arithmetic
    template <bool SW = false>
    __device__ __forceinline__ float2 get_q0(int a, int lg, bool inv) const {
        const int m = a << (logN + 1 - lg);
        const float2 t = tab[SW ? twsw(m) : m];
        return inv ? cconj(t) : t;
    }
};

// Fill the quarter-wave table for an N-point complex FFT (2N-point real
// transform) from the global table W of 2^wlog entries (2^wlog >= 2N).
template <int NT>
__device__ __forceinline__ void load_twiddles(float2* tab, int logN, const float2* __restrict__ W, int wlog) {
    const int n = 1 << (logN - 1);   // angles [0, pi/2): get() never needs index N/2
    const int sh = wlog - (logN + 1);
    for (int m = threadIdx.x; m < n; m += NT) tab[m] = __ldg(&W[m << sh]);
}

// load_twiddles for a table read in the conflict-free placement (Twiddles::get<true>)
template <int NT>
__device__ __forceinline__ void load_twiddles_sw(float2* tab, int logN, const float2* __restrict__ W, int wlog) {
    const int n = 1 << (logN - 1);
    const int sh = wlog - (logN + 1);
    for (int m = threadIdx.x; m < n; m += NT) tab[twsw(m)] = __ldg(&W[m << sh]);
}

// Shared-memory placement of complex element i of a transform buffer.  With
// SW the low four bits of i are XORed with 5 * ((i >> 4) & 3): a bijection
// on every block of 64 elements under which the strided writes of the first
// stages (elements 4j + r, and 16m + k + 4r, of consecutive threads j) and
// every aligned run of 16 elements hit 16 distinct 8-byte bank pairs, so a
// half-warp's 64-bit accesses have no bank conflicts.  Every access to a
// buffer must use the same placement.
template <bool SW>
__device__ __forceinline__ int sidx(int i) {
    return SW ? (i ^ (((i >> 4) & 3) * 5)) : i;
}

// One radix-4 Stockham stage (Ns = product of previous radices).
template <int NT, int MAXB, bool SW = false>
__device__ __forceinline__ void stage_r4(float2* s, int N, int Ns, int lgNs, const Twiddles& tw, bool inv) {
    const int nb = N >> 2;
    float2 v[MAXB][4];
#pragma unroll
    for (int i = 0; i < MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
#pragma unroll
            for (int r = 0; r < 4; ++r) v[i][r] = s[sidx<SW>(j + r * nb)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
            const int k = j & (Ns - 1);
            if (Ns > 1) {
                const int lg = lgNs + 2;
                if constexpr (SW) {
                    // the large transforms: w^k from the table, w^2k and w^3k
                    // by products (the index arithmetic of the two other
                    // reads costs more than the multiplies)
                    const float2 w1 = tw.get_q0<SW>(k, lg, inv);
                    const float2 w2 = cmul(w1, w1);
                    v[i][1] = cmul(v[i][1], w1);
                    v[i][2] = cmul(v[i][2], w2);
                    v[i][3] = cmul(v[i][3], cmul(w2, w1));
                } else {
                    v[i][1] = cmul(v[i][1], tw.get<SW>(k, lg, inv));
                    v[i][2] = cmul(v[i][2], tw.get<SW>(2 * k, lg, inv));
                    v[i][3] = cmul(v[i][3], tw.get<SW>(3 * k, lg, inv));
                }
            }
            const float2 a0 = cadd(v[i][0], v[i][2]);
            const float2 a1 = csub(v[i][0], v[i][2]);
            const float2 a2 = cadd(v[i][1], v[i][3]);
            const float2 d = csub(v[i][1], v[i][3]);
            // forward: (v1 - v3) * (-i); inverse: (v1 - v3) * (+i)
            const float2 a3 = inv ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
            const int base = ((j - k) << 2) + k;
            s[sidx<SW>(base)] = cadd(a0, a2);
            s[sidx<SW>(base + Ns)] = cadd(a1, a3);
            s[sidx<SW>(base + 2 * Ns)] = csub(a0, a2);
            s[sidx<SW>(base + 3 * Ns)] = csub(a1, a3);
        }
    }
    __syncthreads();
}

// Final radix-2 Stockham stage.
template <int NT, int MAXB, bool SW = false>
__device__ __forceinline__ void stage_r2(float2* s, int N, int Ns, int lgNs, const Twiddles& tw, bool inv) {
    const int nb = N >> 1;
    float2 v[2 * MAXB][2];
#pragma unroll
    for (int i = 0; i < 2 * MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
            v[i][0] = s[sidx<SW>(j)];
            v[i][1] = s[sidx<SW>(j + nb)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 2 * MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
            const int k = j & (Ns - 1);
            float2 b = v[i][1];
            if (Ns > 1) b = cmul(b, tw.get<SW>(k, lgNs + 1, inv));
            const int base = ((j - k) << 1) + k;
            s[sidx<SW>(base)] = cadd(v[i][0], b);
            s[sidx<SW>(base + Ns)] = csub(v[i][0], b);
        }
    }
    __syncthreads();
}

// In-place complex FFT of N = 2^logN points in shared memory (unnormalised),
// element i at s[sidx<SW>(i)].  Requires N / 4 <= NT * MAXB and 16 <= N.
// Callers __syncthreads() after writing the data; the function ends with a
// barrier.
template <int NT, int MAXB, bool SW = false>
__device__ void fft_smem(float2* s, int N, int logN, const Twiddles& tw, bool inv) {
    int Ns = 1, lgNs = 0;
    for (; lgNs + 2 <= logN; lgNs += 2, Ns <<= 2) stage_r4<NT, MAXB, SW>(s, N, Ns, lgNs, tw, inv);
    if (lgNs < logN) stage_r2<NT, MAXB, SW>(s, N, Ns, lgNs, tw, inv);
}

// Radix-4 and radix-2 Stockham stages from src to dst (a second buffer): one
// barrier per stage instead of two, and the same arithmetic as the in-place
// stages in the plain placement (SW = false), so results are bit-identical
// to those.
template <int NT, int MAXB>
__device__ __forceinline__ void stage_r4_pp(const float2* src, float2* dst, int N, int Ns, int lgNs,
                                            const Twiddles& tw, bool inv) {
    const int nb = N >> 2;
#pragma unroll
    for (int i = 0; i < MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
            float2 v[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) v[r] = src[j + r * nb];
            const int k = j & (Ns - 1);
            if (Ns > 1) {
                const int lg = lgNs + 2;
                v[1] = cmul(v[1], tw.get(k, lg, inv));
                v[2] = cmul(v[2], tw.get(2 * k, lg, inv));
                v[3] = cmul(v[3], tw.get(3 * k, lg, inv));
            }
            const float2 a0 = cadd(v[0], v[2]);
            const float2 a1 = csub(v[0], v[2]);
            const float2 a2 = cadd(v[1], v[3]);
            const float2 d = csub(v[1], v[3]);
            const float2 a3 = inv ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
            const int base = ((j - k) << 2) + k;
            dst[base] = cadd(a0, a2);
            dst[base + Ns] = cadd(a1, a3);
            dst[base + 2 * Ns] = csub(a0, a2);
            dst[base + 3 * Ns] = csub(a1, a3);
        }
    }
    __syncthreads();
}

template <int NT, int MAXB>
__device__ __forceinline__ void stage_r2_pp(const float2* src, float2* dst, int N, int Ns, int lgNs,
                                            const Twiddles& tw, bool inv) {
    const int nb = N >> 1;
#pragma unroll
    for (int i = 0; i < 2 * MAXB; ++i) {
        const int j = threadIdx.x + i * NT;
        if (j < nb) {
            const float2 v0 = src[j];
            float2 b = src[j + nb];
            const int k = j & (Ns - 1);
            if (Ns > 1) b = cmul(b, tw.get(k, lgNs + 1, inv));
            const int base = ((j - k) << 1) + k;
            dst[base] = cadd(v0, b);
            dst[base + Ns] = csub(v0, b);
        }
    }
    __syncthreads();
}

// fft_smem with a scratch buffer tmp of N points: stages alternate between
// s and tmp (the first one runs in place when the stage count is odd), so
// the result ends in s.  Same preconditions and results as fft_smem.
template <int NT, int MAXB>
__device__ void fft_smem_pp(float2* s, float2* tmp, int N, int logN, const Twiddles& tw, bool inv) {
    const int n4 = logN >> 1, n2 = logN & 1;
    int Ns = 1, lgNs = 0, st = 0;
    float2* a = s;
    float2* b = tmp;
    if ((n4 + n2) & 1) {   // odd stage count: one in-place stage first
        stage_r4<NT, MAXB>(s, N, Ns, lgNs, tw, inv);
        lgNs += 2;
        Ns <<= 2;
        st = 1;
    }
    for (; st < n4; ++st, lgNs += 2, Ns <<= 2) {
        stage_r4_pp<NT, MAXB>(a, b, N, Ns, lgNs, tw, inv);
        float2* t = a;
        a = b;
        b = t;
    }
    if (n2) stage_r2_pp<NT, MAXB>(a, b, N, Ns, lgNs, tw, inv);
}

// fft_smem_pp for a compile-time size N = 2^LOGN: the same stages in the same
// order (identical results), unrolled with constant shifts and strides.
template <int NT, int MAXB, int LOGN>
__device__ __forceinline__ void fft_smem_pp_c(float2* s, float2* tmp, const float2* twtab, bool inv) {
    constexpr int N = 1 << LOGN, n4 = LOGN >> 1, n2 = LOGN & 1;
    constexpr bool odd = ((n4 + n2) & 1) != 0;
    const Twiddles tw{twtab, LOGN};
    float2* a = s;
    float2* b = tmp;
    if (odd) stage_r4<NT, MAXB>(s, N, 1, 0, tw, inv);   // odd stage count: one in-place stage first
#pragma unroll
    for (int st = odd ? 1 : 0; st < n4; ++st) {
        stage_r4_pp<NT, MAXB>(a, b, N, 1 << (2 * st), 2 * st, tw, inv);
        float2* t = a;
        a = b;
        b = t;
    }
    if (n2) stage_r2_pp<NT, MAXB>(a, b, N, 1 << (2 * n4), 2 * n4, tw, inv);
}

// Batched Stockham stages: K transforms of N points, transform t at
// src + t N (dst + t N); the stage's K N / 4 (radix 4) or K N / 2 (radix 2)
// butterflies are dealt round-robin over the CTA, so a CTA with more
// threads than one transform has butterflies keeps all of them busy.  Same
// arithmetic per butterfly as the single-transform stages.
template <int NT, int MAXB>
__device__ __forceinline__ void stage_r4_batch(const float2* src, float2* dst, int K, int N, int logN, int Ns,
                                               int lgNs, const Twiddles& tw, bool inv) {
    const int nb = N >> 2;
    const int total = K * nb;
#pragma unroll
    for (int i = 0; i < MAXB; ++i) {
        const int jj = threadIdx.x + i * NT;
        if (jj < total) {
            const int t = jj >> (logN - 2);
            const int j = jj & (nb - 1);
            const float2* a = src + t * N;
            float2* o = dst + t * N;
            float2 v[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) v[r] = a[j + r * nb];
            const int k = j & (Ns - 1);
            if (Ns > 1) {
                const int lg = lgNs + 2;
                v[1] = cmul(v[1], tw.get(k, lg, inv));
                v[2] = cmul(v[2], tw.get(2 * k, lg, inv));
                v[3] = cmul(v[3], tw.get(3 * k, lg, inv));
            }
            const float2 a0 = cadd(v[0], v[2]);
            const float2 a1 = csub(v[0], v[2]);
            const float2 a2 = cadd(v[1], v[3]);
            const float2 d = csub(v[1], v[3]);
            const float2 a3 = inv ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
            const int base = ((j - k) << 2) + k;
            o[base] = cadd(a0, a2);
            o[base + Ns] = cadd(a1, a3);
            o[base + 2 * Ns] = csub(a0, a2);
            o[base + 3 * Ns] = csub(a1, a3);
        }
    }
    __syncthreads();
}

template <int NT, int MAXB>
__device__ __forceinline__ void stage_r2_batch(const float2* src, float2* dst, int K, int N, int logN, int Ns,
                                               int lgNs, const Twiddles& tw, bool inv) {
    const int nb = N >> 1;
    const int total = K * nb;
#pragma unroll
    for (int i = 0; i < 2 * MAXB; ++i) {
        const int jj = threadIdx.x + i * NT;
        if (jj < total) {
            const int t = jj >> (logN - 1);
            const int j = jj & (nb - 1);
            const float2* a = src + t * N;
            float2* o = dst + t * N;
            const float2 v0 = a[j];
            float2 b = a[j + nb];
            const int k = j & (Ns - 1);
            if (Ns > 1) b = cmul(b, tw.get(k, lgNs + 1, inv));
            const int base = ((j - k) << 1) + k;
            o[base] = cadd(v0, b);
            o[base + Ns] = csub(v0, b);
        }
    }
    __syncthreads();
}

// K transforms of N points from buffer a into stages alternating between a
// and b (both K N points); returns the buffer that holds the result.
// Requires K N / 4 <= NT MAXB and 16 <= N.  Callers __syncthreads() after
// writing the data; the function ends with a barrier.
template <int NT, int MAXB>
__device__ __noinline__ float2* fft_smem_batch(float2* a, float2* b, int K, int N, int logN, const Twiddles& tw, bool inv) {
    int Ns = 1, lgNs = 0;
    for (; lgNs + 2 <= logN; lgNs += 2, Ns <<= 2) {
        stage_r4_batch<NT, MAXB>(a, b, K, N, logN, Ns, lgNs, tw, inv);
        float2* t = a;
        a = b;
        b = t;
    }
    if (lgNs < logN) {
        stage_r2_batch<NT, MAXB>(a, b, K, N, logN, Ns, lgNs, tw, inv);
        a = b;
    }
    return a;
}

// fft_smem_batch for a compile-time size N = 2^LOGN: the stage loop unrolls
// and every shift, mask and twiddle stride is a constant.
template <int NT, int MAXB, int LOGN>
__device__ __noinline__ float2* fft_smem_batch_c(float2* a, float2* b, int K, const float2* twtab, bool inv) {
    constexpr int N = 1 << LOGN;
    const Twiddles tw{twtab, LOGN};
#pragma unroll
    for (int lgNs = 0; lgNs + 2 <= LOGN; lgNs += 2) {
        stage_r4_batch<NT, MAXB>(a, b, K, N, LOGN, 1 << lgNs, lgNs, tw, inv);
        float2* t = a;
        a = b;
        b = t;
    }
    if (LOGN & 1) {
        stage_r2_batch<NT, MAXB>(a, b, K, N, LOGN, 1 << (LOGN - 1), LOGN - 1, tw, inv);
        a = b;
    }
    return a;
}

// Split post-pass for the pair (k, N-k), 0 <= k <= N/2, on Z = FFT_N(z).
// Returns X[k] in xk and X[N-k] in xnk (for k == 0: X[0] and X[N]).
template <bool SW = false>
__device__ __forceinline__ void rfft_split(float2 zk, float2 znk, int k, int logN, const Twiddles& tw, float2& xk,
                                           float2& xnk) {
    if (k == 0) {
        xk = make_float2(zk.x + zk.y, 0.0f);
        xnk = make_float2(zk.x - zk.y, 0.0f);
        return;
    }
    const float2 E = make_float2(0.5f * (zk.x + znk.x), 0.5f * (zk.y - znk.y));
    const float2 O = make_float2(0.5f * (zk.y + znk.y), -0.5f * (zk.x - znk.x));
    const float2 w = tw.get<SW>(k, logN + 1, false);   // e^{-i pi k / N}
    const float2 wO = cmul(w, O);
    xk = cadd(E, wO);
    xnk = cconj(csub(E, wO));
}

// Inverse pre-pass for the pair (k, N-k) from Y[k] (yk) and Y[N-k] (ynk);
// for k == 0 yk = Y[0], ynk = Y[N] and only zk (= Z'[0]) is meaningful.
// Imaginary parts of Y[0] and Y[N] are ignored, as FFTW's c2r does.
template <bool SW = false>
__device__ __forceinline__ void irfft_merge(float2 yk, float2 ynk, int k, int logN, const Twiddles& tw, float2& zk,
                                            float2& znk) {
    if (k == 0) {
        yk.y = 0.0f;
        ynk.y = 0.0f;
    }
    const float2 A = make_float2(yk.x + ynk.x, yk.y - ynk.y);   // Y[k] + conj(Y[N-k])
    const float2 B = make_float2(yk.x - ynk.x, yk.y + ynk.y);   // Y[k] - conj(Y[N-k])
    const float2 w = tw.get<SW>(k, logN + 1, false);
    const float2 cB = cmul(cconj(w), B);                          // conj(w^k) B
    zk = make_float2(A.x - cB.y, A.y + cB.x);                     // A + i conj(w^k) B
    const float2 wcB = cmul(w, cconj(B));                         // w^k conj(B)
    znk = make_float2(A.x - wcB.y, -A.y + wcB.x);                 // conj(A) + i w^k conj(B)
}

// 8-point DFT in registers (used by the cluster transforms and the warp
// transform of the level-0 inverse)
constexpr float kSqrtHalf8 = 0.70710678118654752440f;
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }   // a * (-i)
__device__ __forceinline__ float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }   // a * (+i)

// 8-point DFT in registers, decimation in frequency (unnormalised; inverse =
// conjugate rotations).  Output in natural order.
__device__ __forceinline__ void dft8(float2 v[8], bool inv) {
    // stage 1: pairs (i, i + 4), rotation w8^i of the differences
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 a = cadd(v[i], v[i + 4]);
        float2 d = csub(v[i], v[i + 4]);
        if (i == 1) d = inv ? make_float2(kSqrtHalf8 * (d.x - d.y), kSqrtHalf8 * (d.x + d.y))
                            : make_float2(kSqrtHalf8 * (d.x + d.y), kSqrtHalf8 * (d.y - d.x));
        if (i == 2) d = inv ? mul_pi(d) : mul_mi(d);
        if (i == 3) d = inv ? make_float2(-kSqrtHalf8 * (d.x + d.y), kSqrtHalf8 * (d.x - d.y))
                            : make_float2(kSqrtHalf8 * (d.y - d.x), -kSqrtHalf8 * (d.x + d.y));
        v[i] = a;
        v[i + 4] = d;
    }
    // stage 2: in each half, pairs (i, i + 2), rotation w4^i
#pragma unroll
    for (int h = 0; h < 8; h += 4) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float2 a = cadd(v[h + i], v[h + i + 2]);
            float2 d = csub(v[h + i], v[h + i + 2]);
            if (i == 1) d = inv ? mul_pi(d) : mul_mi(d);
            v[h + i] = a;
            v[h + i + 2] = d;
        }
    }
    // stage 3: pairs (i, i + 1)
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const float2 a = cadd(v[i], v[i + 1]);
        const float2 d = csub(v[i], v[i + 1]);
        v[i] = a;
        v[i + 1] = d;
    }
    // bit-reversed -> natural: swap 1<->4, 3<->6
    float2 t = v[1];
    v[1] = v[4];
    v[4] = t;
    t = v[3];
    v[3] = v[6];
    v[6] = t;
}

}  // namespace pcg
