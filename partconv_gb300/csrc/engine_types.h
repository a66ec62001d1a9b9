// engine_types.h -- device-resident descriptors shared by the host engine
// and the step kernels.
//
// Data layout in HBM (one arena per handle, 256-byte aligned carve-outs):
//   per PC:    input ring xring[Rin]           (time domain, Rin = pow2 >= 2 N_max)
//   per level: H[P][cs]  filter spectra        (float2, cs = N + 2 row stride)
//              X[P][cs]  input-spectrum ring   (slot b mod P holds block b)
//              Yp[cs]    partial sum over parts p >= 1 for the next block
//              yring[R]  output ring            (levels >= 1; R = pow2 >= s_L + N0)
//   per PC:    pcout[N0] level sum (only when an output mixes several PCs)
//   global:    twiddle table W[2^wlog], per-phase task tables, mix counters.
// Rows are (N + 2) complex values so every row starts 16-byte aligned and
// the MAC can move two bins per float4.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
struct float2_ { float x, y; };
#endif

namespace pcg {

#ifdef __CUDACC__
using cfloat2 = float2;
#else
using cfloat2 = float2_;
#endif

// One partition level of one PC.
struct DevLevel {
    int N;          // block size N_L
    int logN;       // log2 N_L
    int P;          // number of parts P_L
    int T;          // N_L / N0: base steps per level block
    int s_blocks;   // s_L / N0: taps before this level, in base blocks
    int cs;         // row stride in complex values (N_L + 2)
    int rmask;      // output ring size - 1 (levels >= 1)
    int pc;         // owning PC
    cfloat2* H;     // [P][cs]
    cfloat2* X;     // [P][cs]
    cfloat2* Yp;    // [cs]
    float* yring;   // [rmask + 1]
};

// One partitioned convolver (one pc.config line).
struct DevPC {
    int M;           // levels
    int lv0;         // index of level 0 in the level array
    int in_ch;
    int out_ch;
    int mute;
    int mix_mode;    // 0: muted (no write), 1: sole writer of out_ch, 2: mixed via pcout
    int zero_outs;   // number of PC-less output channels this PC zero-fills
    int zero_off;    // offset of those channels in the zero list
    float scale;
    int rin_mask;    // input ring size - 1
    float* xring;
    float* pcout;    // [N0] (mix_mode 2)
};

// Where step c's input/output live: base + (c - step0) * step_stride +
// sample * sample_stride + channel * ch_stride.
struct IOView {
    const float* in;
    float* out;
    long long step0;
    long long in_step, in_sample, in_ch;
    long long out_step, out_sample, out_ch;
};

// Per-run state read by every step kernel.
struct RunState {
    long long step_base;   // global step of the first launch in this batch
    IOView io;
};

// A fire task: compute one level block (FFT -> MAC -> IFFT) of one level.
struct FireTask {
    int level;   // index into the level array
};

// A spread task: partial MAC over parts p >= 1 for bins [k0, k1).
struct SpreadTask {
    int level;
    int k0, k1;
};

// Static tables the step kernels read.
struct Bank {
    const DevPC* pcs;
    const DevLevel* lv;
    const cfloat2* W;      // twiddles, 2^wlog entries
    int wlog;
    int N0;
    int H;                 // hyperperiod in steps (power of two)
    int n_out;
    // per output channel mixing lists (mix_mode 2): out_off[o]..out_off[o+1]
    const int* out_off;
    const int* out_pcs;
    int* mix_cnt;          // per output channel arrival counters (zero between steps)
    const int* zero_list;  // output channels with no unmuted PC
};

}  // namespace pcg
