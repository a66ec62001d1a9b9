// orc_fft.h -- the oracle's float32 FFT (test infrastructure only).
//
// Shared by the CPU restatement (pc_oracle.cpp) and by the FFTW stand-in
// (fftw_shim/) that lets the reference's own partconv.cpp run here, so both
// CPU paths transform with the same arithmetic.  The real transform of
// length 2n is the n-point complex FFT of the even/odd packed sequence plus
// the standard split post-pass; the inverse is FFTW's unnormalised c2r
// (imaginary parts of the DC and Nyquist bins ignored).
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

namespace orc {

inline bool is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

inline int ilog2(int x) {
    int p = 0;
    while ((1 << p) < x) ++p;
    return p;
}

// ---------------------------------------------------------------------------
// Float32 FFT (radix-2, decimation in time, bit-reversed input permutation).
// Twiddles are computed in double and rounded once to float.
// ---------------------------------------------------------------------------
struct ComplexFFT {
    int n = 0, logn = 0;
    std::vector<float> wr, wi;   // e^{-2 pi i k / n}, k < n/2
    std::vector<int> rev;

    void init(int n_) {
        n = n_;
        logn = ilog2(n);
        wr.resize(std::max(1, n / 2));
        wi.resize(std::max(1, n / 2));
        for (int k = 0; k < n / 2; ++k) {
            double a = -2.0 * M_PI * (double)k / (double)n;
            wr[k] = (float)std::cos(a);
            wi[k] = (float)std::sin(a);
        }
        rev.resize(n);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < logn; ++b)
                if (i & (1 << b)) r |= 1 << (logn - 1 - b);
            rev[i] = r;
        }
    }

    // in place on split real/imag arrays; inverse = conjugate twiddles,
    // unnormalised.
    void run(float* re, float* im, bool inverse) const {
        for (int i = 0; i < n; ++i) {
            int j = rev[i];
            if (j > i) {
                std::swap(re[i], re[j]);
                std::swap(im[i], im[j]);
            }
        }
        const float sgn = inverse ? -1.0f : 1.0f;
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1;
            const int step = n / len;
            for (int i = 0; i < n; i += len) {
                for (int j = 0; j < half; ++j) {
                    const float c = wr[j * step];
                    const float s = sgn * wi[j * step];
                    const int a = i + j, b = i + j + half;
                    const float vr = re[b] * c - im[b] * s;
                    const float vi = re[b] * s + im[b] * c;
                    re[b] = re[a] - vr;
                    im[b] = im[a] - vi;
                    re[a] = re[a] + vr;
                    im[a] = im[a] + vi;
                }
            }
        }
    }
};

// Real FFT of length nfft = 2n: n+1 bins, interleaved (re, im).
struct RealFFT {
    int nfft = 0, n = 0;
    ComplexFFT cf;
    std::vector<float> pr, pi;   // e^{-i pi k / n}, k <= n
    mutable std::vector<float> br, bi;

    void init(int nfft_) {
        nfft = nfft_;
        n = nfft / 2;
        cf.init(n);
        pr.resize(n + 1);
        pi.resize(n + 1);
        for (int k = 0; k <= n; ++k) {
            double a = -M_PI * (double)k / (double)n;
            pr[k] = (float)std::cos(a);
            pi[k] = (float)std::sin(a);
        }
        br.resize(n);
        bi.resize(n);
    }

    void forward(const float* x, float* X) const {
        for (int k = 0; k < n; ++k) {
            br[k] = x[2 * k];
            bi[k] = x[2 * k + 1];
        }
        cf.run(br.data(), bi.data(), false);
        X[0] = br[0] + bi[0];
        X[1] = 0.0f;
        X[2 * n] = br[0] - bi[0];
        X[2 * n + 1] = 0.0f;
        for (int k = 1; k < n; ++k) {
            const float zr = br[k], zi = bi[k];
            const float mr = br[n - k], mi = -bi[n - k];   // conj(Z[n-k])
            const float er = 0.5f * (zr + mr), ei = 0.5f * (zi + mi);
            // O = -i/2 (Z - conj Z[n-k])
            const float dr = zr - mr, di = zi - mi;
            const float orr = 0.5f * di, oi = -0.5f * dr;
            const float wr_ = pr[k], wi_ = pi[k];
            X[2 * k] = er + (wr_ * orr - wi_ * oi);
            X[2 * k + 1] = ei + (wr_ * oi + wi_ * orr);
        }
    }

    // unnormalised c2r: y[m] = sum_{k<2n} Y[k] e^{+2 pi i k m / 2n}
    void inverse(const float* Y, float* y) const {
        for (int k = 0; k < n; ++k) {
            float ykr = Y[2 * k], yki = Y[2 * k + 1];
            float ynr = Y[2 * (n - k)], yni = Y[2 * (n - k) + 1];
            if (k == 0) { yki = 0.0f; yni = 0.0f; }
            const float ar = ykr + ynr, ai = yki - yni;   // Y[k] + conj(Y[n-k])
            const float bR = ykr - ynr, bI = yki + yni;   // Y[k] - conj(Y[n-k])
            // conj(w^k) * B, then times i
            const float cr = pr[k], ci = -pi[k];
            const float tr = cr * bR - ci * bI, ti = cr * bI + ci * bR;
            br[k] = ar - ti;
            bi[k] = ai + tr;
        }
        cf.run(br.data(), bi.data(), true);
        for (int m = 0; m < n; ++m) {
            y[2 * m] = br[m];
            y[2 * m + 1] = bi[m];
        }
    }
};

}  // namespace orc
