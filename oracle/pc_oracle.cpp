// pc_oracle.cpp -- CPU restatement of partconv's multi-level partitioned
// FFT convolution.
//
// TEST INFRASTRUCTURE ONLY.  This file is what the GPU path is compared
// against, and the timed CPU baseline.  Only tests, the smoke check and the benchmark's
// CPU-baseline leg load it; the product library never links or calls it.
//
// What is restated (file:line refer to ebattenberg/partconv):
//   * layout validation and IR partitioning      src/partconv.cpp:70-230
//     (strict slack check :148-166, last-level part count :169-181,
//      relaxed MATLAB check matlab/MFDL_part_conv.m:25-37)
//   * PartConvFilter::runLevel                    src/partconv.cpp:354-490
//     (slot arithmetic :362,:372,:487; p-ascending MAC :370-479)
//   * sync_levels / sync_levels_relaxed / input / output / output_relaxed
//                                                 src/partconv.cpp:568-648
//   * DelayBuffer, DoubleBuffer                   src/partconv.cpp:1401-1511
//   * PartConvMulti::run and the Relaxed variant  src/partconvMulti.cpp:815-928,
//                                                 :1017-1134 (deinterleave+scale
//                                                 :839-847, mix :911-921)
//   * the minimum-latency schedule for layouts that pass only the relaxed
//     check (each level block computed in the callback in which its input
//     completes; the structure of matlab/MFDL_part_conv.m:131-243).
//
// FFTW (fftw-3.2.2 per src/wisdom.wis:1; not vendored) is replaced by the
// oracle's own float32 radix-2 FFT (orc_fft.h).  The real transform of length 2N is the
// N-point complex FFT of the even/odd packed sequence plus the standard
// split post-pass; the inverse is FFTW's unnormalised c2r (imaginary parts of
// the DC and Nyquist bins ignored).  Build with -ffp-contract=off so the MAC
// rounds like the reference's SSE3 multiply/addsub sequence (no fused ops).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "orc_fft.h"

namespace orc {

// ---------------------------------------------------------------------------
// Layout validation.  src/partconv.cpp:87-181 (strict) and
// matlab/MFDL_part_conv.m:25-37 (relaxed).  Returns 0 on success.
// P[M-1] is recomputed from the IR length as the reference does.
// ---------------------------------------------------------------------------
static int check_layout(int M, const int* N, int* P, int ir_len, bool relaxed,
                        int* delays, std::string& msg) {
    char buf[256];
    if (M < 1) { msg = "at least one partitioning level is required"; return 1; }
    for (int i = 0; i < M; ++i) {
        if (!is_pow2(N[i])) {
            snprintf(buf, sizeof buf, "block size of level %d must be a power of 2 (N[%d] = %d)", i, i, N[i]);
            msg = buf;
            return 1;
        }
    }
    for (int i = 1; i < M; ++i) {
        if (N[i] <= N[i - 1]) {
            snprintf(buf, sizeof buf, "N[%d]=%d <= N[%d]=%d", i, N[i], i - 1, N[i - 1]);
            msg = buf;
            return 1;
        }
    }
    for (int i = 0; i < M - 1; ++i) {
        if (P[i] < 1) {
            snprintf(buf, sizeof buf, "level %d needs at least one partition", i);
            msg = buf;
            return 1;
        }
    }
    long position = 2L * N[0];
    long s = 0;
    for (int i = 0; i < M - 1; ++i) {
        if (delays) delays[i] = (int)(position / N[0]);
        position += (long)N[i] * P[i];
        s += (long)N[i] * P[i];
        bool ok = relaxed ? (s >= N[i + 1]) : (position >= 2L * N[i + 1]);
        if (!ok) {
            snprintf(buf, sizeof buf, "sufficient delay not allowed for block size of level %d", i + 2);
            msg = buf;
            return 1;
        }
    }
    if (delays) delays[M - 1] = (int)(position / N[0]);
    long rem = (long)ir_len - s;
    // The reference refuses only rem < 0 (src/partconv.cpp:169-170).  With
    // rem == 0 it sets P[M-1] = 0 and its runLevel then computes
    // bcurr % num_parts (partconv.cpp:362), a division by zero; here the
    // layout is refused instead, with the reference's message.
    if (rem <= 0) {
        snprintf(buf, sizeof buf, "last partitioning level (%d) not required", M);
        msg = buf;
        return 1;
    }
    P[M - 1] = (int)((rem + N[M - 1] - 1) / N[M - 1]);
    return 0;
}

// Filter spectra for one level: row p = [0_N, h_L[pN..(p+1)N)], rfft / nfft.
// src/partconv.cpp:185-230, src/buffers.cpp:194-217.
static void level_spectra(const RealFFT& fft, const float* hpad, long start, int N, int P,
                          std::vector<float>& H) {
    const int C = N + 1;
    H.assign((size_t)P * C * 2, 0.0f);
    std::vector<float> row(2 * N);
    const float scale = (float)(2 * N);
    for (int p = 0; p < P; ++p) {
        std::fill(row.begin(), row.end(), 0.0f);
        std::memcpy(&row[N], hpad + start + (long)p * N, sizeof(float) * N);
        fft.forward(row.data(), &H[(size_t)p * C * 2]);
        for (int j = 0; j < 2 * C; ++j) H[(size_t)p * C * 2 + j] /= scale;
    }
}

// Y += X * H over C bins, reference operation order (partconv.cpp:379-479).
static inline void cmac(float* Y, const float* X, const float* Hp, int C) {
    for (int k = 0; k < C; ++k) {
        const float a = X[2 * k], b = X[2 * k + 1];
        const float c = Hp[2 * k], d = Hp[2 * k + 1];
        Y[2 * k] += (a * c) - (b * d);
        Y[2 * k + 1] += (a * d) + (b * c);
    }
}

// ---------------------------------------------------------------------------
// DelayBuffer / DoubleBuffer (src/partconv.cpp:1401-1511).
// ---------------------------------------------------------------------------
struct DelayBuffer {
    int frameSize, framesPerBlock, numBlocks, bufferSize;
    int readBlock, writeBlock, writeFrame, readFrameDelay;
    std::vector<float> mem;
    bool overlap_error = false;

    DelayBuffer(int fs, int fpb, int delay) : frameSize(fs), framesPerBlock(fpb) {
        readFrameDelay = delay - framesPerBlock - 1;
        int rem = (readFrameDelay + 1) % framesPerBlock;
        bufferSize = readFrameDelay + 1 + (framesPerBlock - rem);
        numBlocks = bufferSize / framesPerBlock + 1;
        bufferSize = numBlocks * framesPerBlock;
        mem.assign((size_t)bufferSize * frameSize, 0.0f);
        reset_idx();
    }
    void reset_idx() {
        readBlock = numBlocks - 1;
        writeBlock = readFrameDelay / framesPerBlock;
        writeFrame = readFrameDelay % framesPerBlock;
    }
    void write(const float* x) {
        int frame = writeBlock * framesPerBlock + writeFrame;
        std::memcpy(&mem[(size_t)frame * frameSize], x, sizeof(float) * frameSize);
        if (++writeFrame == framesPerBlock) {
            writeFrame = 0;
            if (++writeBlock == numBlocks) writeBlock = 0;
        }
    }
    // the reference exits the process when the read block is the write block
    // (partconv.cpp:1449-1455); here the error is recorded instead.
    void read(float* y) {
        if (readBlock == writeBlock) overlap_error = true;
        int frame = readBlock * framesPerBlock;
        std::memcpy(y, &mem[(size_t)frame * frameSize], sizeof(float) * frameSize * framesPerBlock);
    }
    void prepNextRead() {
        if (++readBlock == numBlocks) readBlock = 0;
    }
    void reset() {
        std::fill(mem.begin(), mem.end(), 0.0f);
        reset_idx();
    }
};

struct DoubleBuffer {
    std::vector<float> a, b;
    float* rd;
    float* wr;
    explicit DoubleBuffer(int n) : a(n, 0.0f), b(n, 0.0f) { rd = a.data(); wr = b.data(); }
    void swap() { std::swap(rd, wr); }
    void reset() {
        std::fill(a.begin(), a.end(), 0.0f);
        std::fill(b.begin(), b.end(), 0.0f);
    }
};

// Common interface for one partitioned convolver of one IR.
struct Convolver {
    virtual ~Convolver() {}
    int M = 0, N0 = 0;
    std::vector<int> N, P;
    // strict-schedule callback (zero added latency)
    virtual void process(const float* in, float* out) = 0;
    // PartConvMultiRelaxed-schedule callback (one base block of latency)
    virtual void process_relaxed(const float* in, float* out) = 0;
    virtual void reset() = 0;
    virtual bool error() const { return false; }
};

// ---------------------------------------------------------------------------
// PartConvFilter restatement (strict layouts).  src/partconv.cpp:70-648.
// ---------------------------------------------------------------------------
struct Filter : Convolver {
    std::vector<int> nfft, cfft, num_N0, ind_N0;
    std::vector<unsigned> bcurr;
    int start_sync_depth = 0, end_sync_depth = 0;
    std::vector<RealFFT> fft;
    std::vector<std::vector<float>> H, Xfft, inbuffer, outbuffer, Yfft;
    std::vector<std::unique_ptr<DelayBuffer>> Xbuf;
    std::vector<std::unique_ptr<DoubleBuffer>> Ybuf;

    int setup(int M_, const int* N_, const int* P_, const float* h, int len, bool relaxed_check,
              std::string& msg) {
        M = M_;
        N.assign(N_, N_ + M);
        P.assign(P_, P_ + M);
        std::vector<int> delays(M);
        if (check_layout(M, N.data(), P.data(), len, relaxed_check, delays.data(), msg)) return 1;
        N0 = N[0];
        nfft.resize(M); cfft.resize(M); num_N0.resize(M); ind_N0.resize(M); bcurr.assign(M, 0);
        for (int i = 0; i < M; ++i) {
            nfft[i] = 2 * N[i];
            cfft[i] = N[i] + 1;
            num_N0[i] = N[i] / N[0];
            ind_N0[i] = num_N0[i] - 1;
        }
        long total = 0;
        for (int i = 0; i < M; ++i) total += (long)N[i] * P[i];
        std::vector<float> hpad(total, 0.0f);
        if (h) std::memcpy(hpad.data(), h, sizeof(float) * std::min<long>(len, total));
        else std::fill(hpad.begin(), hpad.begin() + std::min<long>(len, total), 1.0f);
        fft.resize(M);
        H.resize(M); Xfft.resize(M); inbuffer.resize(M); outbuffer.resize(M); Yfft.resize(M);
        long start = 0;
        for (int L = 0; L < M; ++L) {
            fft[L].init(nfft[L]);
            level_spectra(fft[L], hpad.data(), start, N[L], P[L], H[L]);
            start += (long)N[L] * P[L];
            Xfft[L].assign((size_t)P[L] * cfft[L] * 2, 0.0f);
            inbuffer[L].assign(nfft[L], 0.0f);
            outbuffer[L].assign(nfft[L], 0.0f);
            Yfft[L].assign((size_t)cfft[L] * 2, 0.0f);
            Xbuf.emplace_back(new DelayBuffer(N[0], N[L] / N[0], delays[L]));
            Ybuf.emplace_back(new DoubleBuffer(N[L]));
        }
        return 0;
    }

    int runLevel(int L) {
        const int n = N[L], C = cfft[L], Pl = P[L];
        std::memcpy(&inbuffer[L][0], &inbuffer[L][n], sizeof(float) * n);
        Xbuf[L]->read(&inbuffer[L][n]);
        int slot = (int)(bcurr[L] % (unsigned)Pl);
        fft[L].forward(inbuffer[L].data(), &Xfft[L][(size_t)slot * C * 2]);
        std::fill(Yfft[L].begin(), Yfft[L].end(), 0.0f);
        for (int p = 0; p < Pl; ++p) {
            slot = (int)((bcurr[L] - p + Pl) % (unsigned)Pl);
            cmac(Yfft[L].data(), &Xfft[L][(size_t)slot * C * 2], &H[L][(size_t)p * C * 2], C);
        }
        fft[L].inverse(Yfft[L].data(), outbuffer[L].data());
        std::memcpy(Ybuf[L]->wr, outbuffer[L].data(), sizeof(float) * n);
        bcurr[L]++;
        return 0;
    }

    void sync_levels() {
        start_sync_depth = 0;
        end_sync_depth = 0;
        for (int L = 0; L < M; ++L) {
            ind_N0[L]++;
            if (ind_N0[L] == num_N0[L]) {
                ind_N0[L] = 0;
                start_sync_depth = L;
            } else if (ind_N0[L] == num_N0[L] - 1) {
                end_sync_depth = L;
            }
        }
    }
    void sync_levels_relaxed() {
        start_sync_depth = 0;
        end_sync_depth = 0;
        for (int L = 0; L < M; ++L) {
            ind_N0[L]++;
            if (ind_N0[L] == num_N0[L]) {
                ind_N0[L] = 0;
                start_sync_depth = L;
                end_sync_depth = L;
            }
        }
    }
    void input(const float* x) {
        for (int L = 0; L < M; ++L) {
            Xbuf[L]->write(x);
            if (L <= start_sync_depth) Xbuf[L]->prepNextRead();
        }
    }
    void output(float* y) {
        std::memcpy(y, outbuffer[0].data(), sizeof(float) * N[0]);
        for (int L = 1; L < M; ++L) {
            if (L <= end_sync_depth) Ybuf[L]->swap();
            int rb = ind_N0[L] + 1;
            if (rb == num_N0[L]) rb = 0;
            const float* ptr = Ybuf[L]->rd + (size_t)N[0] * rb;
            for (int i = 0; i < N[0]; ++i) y[i] += ptr[i];
        }
    }
    void output_relaxed(float* y) {
        std::memcpy(y, outbuffer[0].data(), sizeof(float) * N[0]);
        for (int L = 1; L < M; ++L) {
            if (L <= end_sync_depth) Ybuf[L]->swap();
            int rb = ind_N0[L];
            if (rb == num_N0[L]) rb = 0;
            const float* ptr = Ybuf[L]->rd + (size_t)N[0] * rb;
            for (int i = 0; i < N[0]; ++i) y[i] += ptr[i];
        }
    }
    void reset() override {
        std::fill(bcurr.begin(), bcurr.end(), 0u);
        for (int L = 0; L < M; ++L) {
            ind_N0[L] = num_N0[L] - 1;
            std::fill(inbuffer[L].begin(), inbuffer[L].end(), 0.0f);
            std::fill(Xfft[L].begin(), Xfft[L].end(), 0.0f);
            Xbuf[L]->reset();
            Ybuf[L]->reset();
        }
    }
    bool error() const override {
        for (auto& d : Xbuf)
            if (d->overlap_error) return true;
        return false;
    }
    // PartConvMulti::run per-PC sequence (partconvMulti.cpp:849-909): the
    // level workers woken at start_sync_depth run right after input().
    void process(const float* in, float* out) override {
        sync_levels();
        input(in);
        for (int L = 0; L <= start_sync_depth; ++L) runLevel(L);
        output(out);
    }
    // PartConvMultiRelaxed::run per-PC sequence (partconvMulti.cpp:1040-1111).
    void process_relaxed(const float* in, float* out) override {
        sync_levels_relaxed();
        output_relaxed(out);
        input(in);
        for (int L = 0; L <= start_sync_depth; ++L) runLevel(L);
    }
};

// ---------------------------------------------------------------------------
// Minimum-latency schedule (relaxed layouts, s_L >= N_L for L >= 1).
// Level L covers taps [s_L, s_L + N_L P_L).  Its block b (output samples
// [b N_L, (b+1) N_L)) needs input up to sample (b+1) N_L - s_L - 1, so it is
// computed in the callback c with (c + 1) N0 + s_L = (b + 1) N_L: the window
// is always the newest 2 N_L input samples.  Outputs wait in a per-level
// ring until emitted; the sum runs over levels in ascending order like
// PartConvFilter::output (partconv.cpp:616-631).
// ---------------------------------------------------------------------------
struct MinLatFilter : Convolver {
    std::vector<long> s;
    std::vector<int> T, R;
    int only = -1;   // >= 0: run and emit that level alone (one worker per level)
    std::vector<RealFFT> fft;
    std::vector<std::vector<float>> H, X, Y, yring;
    std::vector<float> xring, win, blk, prev_out;
    int Rin = 0;
    long c = 0;

    int setup(int M_, const int* N_, const int* P_, const float* h, int len, std::string& msg) {
        M = M_;
        N.assign(N_, N_ + M);
        P.assign(P_, P_ + M);
        if (check_layout(M, N.data(), P.data(), len, true, nullptr, msg)) return 1;
        N0 = N[0];
        s.assign(M, 0);
        for (int L = 1; L < M; ++L) s[L] = s[L - 1] + (long)N[L - 1] * P[L - 1];
        long total = s[M - 1] + (long)N[M - 1] * P[M - 1];
        std::vector<float> hpad(total, 0.0f);
        if (h) std::memcpy(hpad.data(), h, sizeof(float) * std::min<long>(len, total));
        else std::fill(hpad.begin(), hpad.begin() + std::min<long>(len, total), 1.0f);
        fft.resize(M); H.resize(M); X.resize(M); Y.resize(M); yring.resize(M);
        T.resize(M); R.resize(M);
        for (int L = 0; L < M; ++L) {
            fft[L].init(2 * N[L]);
            level_spectra(fft[L], hpad.data(), s[L], N[L], P[L], H[L]);
            X[L].assign((size_t)P[L] * (N[L] + 1) * 2, 0.0f);
            Y[L].assign((size_t)(N[L] + 1) * 2, 0.0f);
            T[L] = N[L] / N0;
            long need = s[L] + N0;
            int r = N[L];
            while (r < need) r <<= 1;
            R[L] = r;
            yring[L].assign(r, 0.0f);
        }
        Rin = 1;
        while (Rin < 2 * N[M - 1]) Rin <<= 1;
        xring.assign(Rin, 0.0f);
        win.resize(2 * N[M - 1]);
        blk.resize(2 * N[M - 1]);
        prev_out.assign(N0, 0.0f);
        c = 0;
        return 0;
    }

    void run_block(int L, long b) {
        const int n = N[L], C = n + 1, Pl = P[L];
        const long end = (c + 1) * (long)N0;    // newest sample + 1
        for (int i = 0; i < 2 * n; ++i) win[i] = xring[(size_t)((end - 2 * n + i) & (Rin - 1))];
        const int slot = (int)(b % Pl);
        fft[L].forward(win.data(), &X[L][(size_t)slot * C * 2]);
        std::fill(Y[L].begin(), Y[L].end(), 0.0f);
        for (int p = 0; p < Pl; ++p) {
            long bb = b - p;
            int sl = (int)(((bb % Pl) + Pl) % Pl);
            cmac(Y[L].data(), &X[L][(size_t)sl * C * 2], &H[L][(size_t)p * C * 2], C);
        }
        fft[L].inverse(Y[L].data(), blk.data());
        const long t0 = b * (long)n;
        for (int i = 0; i < n; ++i) yring[L][(size_t)((t0 + i) & (R[L] - 1))] = blk[i];
    }

    void step(const float* in, float* out) {
        const long t = c * (long)N0;
        for (int i = 0; i < N0; ++i) xring[(size_t)((t + i) & (Rin - 1))] = in[i];
        for (int L = 0; L < M; ++L) {
            if (only >= 0 && L != only) continue;
            long q = c + 1 + s[L] / N0;
            if (q % T[L] == 0) run_block(L, q / T[L] - 1);
        }
        if (only >= 0) {
            for (int i = 0; i < N0; ++i) out[i] = yring[only][(size_t)((t + i) & (R[only] - 1))];
        } else {
            for (int i = 0; i < N0; ++i) out[i] = yring[0][(size_t)((t + i) & (R[0] - 1))];
            for (int L = 1; L < M; ++L)
                for (int i = 0; i < N0; ++i) out[i] += yring[L][(size_t)((t + i) & (R[L] - 1))];
        }
        ++c;
    }
    void process(const float* in, float* out) override { step(in, out); }
    void process_relaxed(const float* in, float* out) override {
        std::memcpy(out, prev_out.data(), sizeof(float) * N0);
        step(in, prev_out.data());
    }
    void reset() override {
        for (int L = 0; L < M; ++L) {
            std::fill(X[L].begin(), X[L].end(), 0.0f);
            std::fill(yring[L].begin(), yring[L].end(), 0.0f);
        }
        std::fill(xring.begin(), xring.end(), 0.0f);
        std::fill(prev_out.begin(), prev_out.end(), 0.0f);
        c = 0;
    }
};

// ---------------------------------------------------------------------------
// PartConvMulti restatement (src/partconvMulti.cpp:815-928, :1017-1134).
// ---------------------------------------------------------------------------
struct Multi {
    int buffer_size = 0, n_in = 0, n_out = 0, relaxed = 0;
    std::vector<std::unique_ptr<Convolver>> pc;
    std::vector<int> in_ch, out_ch, mute;
    std::vector<float> scale;
    std::vector<float> in_mix, out_mix;

    int run(float* out, const float* in, int frames) {
        if (frames != buffer_size) return 1;
        const int npc = (int)pc.size();
        std::memset(out, 0, sizeof(float) * (size_t)n_out * frames);
        for (int i = 0; i < npc; ++i) {
            const int ch = in_ch[i];
            const float sc = scale[i];
            for (int j = 0; j < frames; ++j) in_mix[j] = in[ch + j * n_in] * sc;
            if (relaxed) pc[i]->process_relaxed(in_mix.data(), out_mix.data());
            else pc[i]->process(in_mix.data(), out_mix.data());
            if (!mute[i]) {
                const int oc = out_ch[i];
                for (int j = 0; j < frames; ++j) out[oc + j * n_out] += out_mix[j];
            }
        }
        for (auto& p : pc)
            if (p->error()) return 2;
        return 0;
    }
};

}  // namespace orc

using namespace orc;

static void put_msg(char* dst, int len, const std::string& s) {
    if (dst && len > 0) {
        std::snprintf(dst, (size_t)len, "%s", s.c_str());
    }
}

extern "C" {

// layout check: returns 0 and fills P[M-1] and delays (base blocks) on success
int orc_layout_check(int M, const int* N, int* P, int ir_len, int relaxed, int* delays,
                     char* msg, int msglen) {
    std::string m;
    int r = check_layout(M, N, P, ir_len, relaxed != 0, delays, m);
    put_msg(msg, msglen, m);
    return r;
}

// schedule: 0 = strict restatement when the layout passes the strict check,
// otherwise minimum-latency; 1 = strict restatement only; 2 = minimum-latency.
void* orc_multi_create(int buffer_size, int n_in, int n_out, int num_pcs, const int* M,
                       const int* N_flat, const int* P_flat, const float* const* irs,
                       const int* ir_lens, const int* in_ch, const int* out_ch,
                       const float* scale, const int* mute, int relaxed_variant, int schedule,
                       char* msg, int msglen) {
    auto* m = new Multi();
    m->buffer_size = buffer_size;
    m->n_in = n_in;
    m->n_out = n_out;
    m->relaxed = relaxed_variant;
    int off = 0;
    for (int i = 0; i < num_pcs; ++i) {
        std::string err;
        std::unique_ptr<Convolver> cv;
        std::vector<int> Pt(P_flat + off, P_flat + off + M[i]);
        bool strict_ok = false;
        if (schedule != 2) {
            std::string e2;
            std::vector<int> Pc = Pt;
            strict_ok = check_layout(M[i], N_flat + off, Pc.data(), ir_lens[i], false, nullptr, e2) == 0;
            if (!strict_ok && schedule == 1) {
                put_msg(msg, msglen, "PC " + std::to_string(i) + ": " + e2);
                delete m;
                return nullptr;
            }
        }
        if (strict_ok) {
            auto* f = new Filter();
            if (f->setup(M[i], N_flat + off, Pt.data(), irs[i], ir_lens[i], false, err)) {
                delete f;
                put_msg(msg, msglen, "PC " + std::to_string(i) + ": " + err);
                delete m;
                return nullptr;
            }
            cv.reset(f);
        } else {
            auto* f = new MinLatFilter();
            if (f->setup(M[i], N_flat + off, Pt.data(), irs[i], ir_lens[i], err)) {
                delete f;
                put_msg(msg, msglen, "PC " + std::to_string(i) + ": " + err);
                delete m;
                return nullptr;
            }
            cv.reset(f);
        }
        if (cv->N0 != buffer_size) {
            put_msg(msg, msglen, "PC " + std::to_string(i) + ": first block size must equal buffer_size");
            delete m;
            return nullptr;
        }
        m->pc.push_back(std::move(cv));
        off += M[i];
    }
    m->in_ch.assign(in_ch, in_ch + num_pcs);
    m->out_ch.assign(out_ch, out_ch + num_pcs);
    m->scale.assign(scale, scale + num_pcs);
    m->mute.assign(mute, mute + num_pcs);
    m->in_mix.assign(buffer_size, 0.0f);
    m->out_mix.assign(buffer_size, 0.0f);
    put_msg(msg, msglen, "");
    return m;
}

// frames may be any multiple of buffer_size: runs frames/buffer_size callbacks
int orc_multi_run(void* h, float* out, const float* in, long frames) {
    auto* m = (Multi*)h;
    if (frames % m->buffer_size) return 1;
    long nb = frames / m->buffer_size;
    for (long b = 0; b < nb; ++b) {
        int r = m->run(out + b * m->buffer_size * (long)m->n_out, in + b * m->buffer_size * (long)m->n_in,
                       m->buffer_size);
        if (r) return r;
    }
    return 0;
}

void orc_multi_reset(void* h) {
    for (auto& p : ((Multi*)h)->pc) p->reset();
}

void orc_multi_destroy(void* h) { delete (Multi*)h; }

// ---- PartConvFilter fine-grained API (strict or relaxed validation) ----
void* orc_filter_create(int M, const int* N, const int* P, const float* ir, int ir_len,
                        int relaxed_check, char* msg, int msglen) {
    auto* f = new Filter();
    std::string err;
    if (f->setup(M, N, P, ir, ir_len, relaxed_check != 0, err)) {
        put_msg(msg, msglen, err);
        delete f;
        return nullptr;
    }
    put_msg(msg, msglen, "");
    return f;
}
void orc_filter_sync_levels(void* h) { ((Filter*)h)->sync_levels(); }
void orc_filter_sync_levels_relaxed(void* h) { ((Filter*)h)->sync_levels_relaxed(); }
void orc_filter_input(void* h, const float* x) { ((Filter*)h)->input(x); }
void orc_filter_output(void* h, float* y) { ((Filter*)h)->output(y); }
void orc_filter_output_relaxed(void* h, float* y) { ((Filter*)h)->output_relaxed(y); }
int orc_filter_run_level(void* h, int L) { return ((Filter*)h)->runLevel(L); }
void orc_filter_reset(void* h) { ((Filter*)h)->reset(); }
int orc_filter_error(void* h) { return ((Filter*)h)->error() ? 1 : 0; }
void orc_filter_parts(void* h, int* P) {
    auto* f = (Filter*)h;
    for (int i = 0; i < f->M; ++i) P[i] = f->P[i];
}
// copy level L's filter spectra (P x (N+1) complex, interleaved)
void orc_filter_spectra(void* h, int L, float* out) {
    auto* f = (Filter*)h;
    std::memcpy(out, f->H[L].data(), sizeof(float) * f->H[L].size());
}
void orc_filter_destroy(void* h) { delete (Filter*)h; }

// ---- transforms ----
int orc_rfft(int nfft, const float* x, float* X) {
    if (!is_pow2(nfft) || nfft < 2) return 1;
    RealFFT f;
    f.init(nfft);
    f.forward(x, X);
    return 0;
}
int orc_irfft(int nfft, const float* X, float* y) {
    if (!is_pow2(nfft) || nfft < 2) return 1;
    RealFFT f;
    f.init(nfft);
    f.inverse(X, y);
    return 0;
}

// ---- FP64 direct convolution at chosen output indices (all if idx == NULL) ----
void orc_conv_direct_f64(const float* x, long nx, const float* h, long nh, const long* idx,
                         long nidx, double* y, int threads) {
    if (threads < 1) threads = 1;
    auto work = [&](int t) {
        for (long j = t; j < nidx; j += threads) {
            long n = idx ? idx[j] : j;
            double acc = 0.0;
            long k0 = std::max(0L, n - nx + 1), k1 = std::min(nh - 1, n);
            for (long k = k0; k <= k1; ++k) acc += (double)h[k] * (double)x[n - k];
            y[j] = acc;
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(work, t);
    for (auto& t : th) t.join();
}

// ---- throughput runner: independent mono streams spread over threads ----
// Each stream s has its own layout (M[s] levels; N/P flattened) and IR.
// in: [S][frames] planar; out: [S][frames].  Streams are handed to threads
// dynamically; returns wall seconds, or a negative value on a setup error.
double orc_run_streams(int S, const int* M, const int* N_flat, const int* P_flat,
                       const float* const* irs, const int* ir_lens, const float* in, float* out,
                       long frames, int buffer_size, int threads, char* msg, int msglen) {
    std::vector<std::unique_ptr<MinLatFilter>> f(S);
    int off = 0;
    for (int s = 0; s < S; ++s) {
        f[s].reset(new MinLatFilter());
        std::vector<int> Pt(P_flat + off, P_flat + off + M[s]);
        std::string err;
        if (f[s]->setup(M[s], N_flat + off, Pt.data(), irs[s], ir_lens[s], err) ||
            f[s]->N0 != buffer_size) {
            put_msg(msg, msglen, "stream " + std::to_string(s) + ": " + (err.empty() ? "bad N0" : err));
            return -1.0;
        }
        off += M[s];
    }
    if (threads < 1) threads = 1;
    std::atomic<int> next(0);
    const long nb = frames / buffer_size;
    auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            int s = next.fetch_add(1);
            if (s >= S) break;
            for (long b = 0; b < nb; ++b)
                f[s]->step(in + (long)s * frames + b * buffer_size, out + (long)s * frames + b * buffer_size);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Reference-shaped CPU throughput: one worker thread per level, as the
// reference runs each level on its own thread (src/partconvMulti.cpp:473-694).
// Each worker convolves the whole signal with its level's part of the IR;
// the level outputs are then summed in level order, the order of the
// sequential restatement, so the result is bit-identical to it.  Returns
// wall seconds (-1 on a bad layout).
double orc_run_leveled(int M, const int* N, const int* P, const float* ir, int ir_len, const float* in,
                       float* out, long frames, char* msg, int msglen) {
    std::vector<std::unique_ptr<MinLatFilter>> f(M);
    for (int L = 0; L < M; ++L) {
        f[L].reset(new MinLatFilter());
        std::vector<int> Pt(P, P + M);
        std::string err;
        if (f[L]->setup(M, N, Pt.data(), ir, ir_len, err)) {
            put_msg(msg, msglen, err);
            return -1.0;
        }
        f[L]->only = L;
    }
    const int N0 = N[0];
    const long nb = frames / N0;
    std::vector<std::vector<float>> y(M, std::vector<float>((size_t)nb * N0));
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int L = 0; L < M; ++L)
        th.emplace_back([&, L]() {
            for (long b = 0; b < nb; ++b) f[L]->step(in + b * N0, y[L].data() + b * N0);
        });
    for (auto& t : th) t.join();
    for (long i = 0; i < nb * N0; ++i) {
        float v = y[0][i];
        for (int L = 1; L < M; ++L) v += y[L][i];
        out[i] = v;
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
