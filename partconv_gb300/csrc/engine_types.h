// engine_types.h -- device-resident descriptors shared by the host engine
// and the step kernels.
//
// Data layout in HBM (one arena per handle, 256-byte aligned carve-outs):
//   per PC:    input ring xring[Rin]           (time domain, Rin = pow2 >= 2 N_max)
//   per level: H[P][cs]  filter spectra        (float2, cs = N + 2 row stride)
//              X[P][cs]  input-spectrum ring   (slot b mod P holds block b)
//              Yp[rows][2][cs] partial sums of the FDL MAC for the next block
//                        (level 0 with K base blocks per step: [rows][2K][cs])
//              yring[R]  output ring            (levels >= 1; R = pow2 >= s_L + N0)
//   per PC:    pcout[N0] level sum (only when an output mixes several PCs)
//   global:    twiddle table W[2^wlog], per-phase task tables, mix counters.
// Rows are (N + 2) complex values so every row starts 16-byte aligned and
// the MAC can move two bins per float4.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pcg {

constexpr int kEmitLevels = 4;   // level-0 tasks carry the output rings of up to 4 more levels

// One partition level of one PC (host copy and device table).
struct DevLevel {
    int N;          // block size N_L
    int logN;       // log2 N_L
    int P;          // number of parts P_L
    int T;          // N_L / N0: base steps per level block
    int s_blocks;   // s_L / N0: taps before this level, in base blocks
    int cs;         // row stride in complex values (N_L + 2)
    int rmask;      // output ring size - 1 (levels >= 1)
    int pc;         // owning PC
    int npart;      // partial-sum rows (a spread task covers at most the handle's parts per task)
    float2* H;      // [P][cs]
    float2* X;      // [P][cs]
    float2* Yp;     // [npart][2][cs]: row q, block parity ([npart][2K][cs], block mod 2K, for
                    // level 0 with K base blocks per step)
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

// A unit of work of one base step, self-contained so a CTA needs one load
// to start.  kind 0 (fire): compute one level block -- window, FFT, MAC,
// inverse FFT, output (level 0 also emits the step's output); k0 holds the
// number of partial-sum rows to add (0 means 1).  kind 1 (spread): partial
// FDL MAC over bins [k0, k1) and parts [p_lo, in_ch) (in_ch 0: up to P) of
// a level's next block, written to partial-sum row out_ch; a spread task
// keeps its bins per task (the tile width) in M (0: the default).
struct Task {
    int kind, N, logN, P;
    int T, s_blocks, cs, rmask;
    int k0, k1, M, in_ch;
    int out_ch, mix_mode, zero_outs, zero_off;
    int rin_mask, lv_index, p_lo, active;   // p_lo: first part summed by a spread task
                                            // (K-block level-0 fire: the parts it sums itself)
    float scale;
    int dfer;           // 1: the level's fire runs off the step chain (deferred), see engine.cu
    // step at which this PC's time starts (serving pools); in a static bank
    // with several base blocks per step, minus the offset of the task's base
    // step within the launch's step (a task sees c = launch step - origin)
    long long origin;
    float2* H;
    float2* X;
    float2* Yp;
    float* yring;
    float* xring;
    float* pcout;
    float* eyring[kEmitLevels];   // level-0 fire: output rings of levels 1..4
    int emask[kEmitLevels];
};
static_assert(sizeof(Task) == 192, "Task record is loaded as 12 x 16 bytes");

// One CTA of a serving pool's step: descriptor slot and sub-task (0: the
// level's fire, s >= 1: the s-th bin tile of its spread slice).
struct PoolCta {
    int slot;
    int sub;
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
    long long step_base;   // global step of step_in_batch == 0
    IOView io;
};
static_assert(sizeof(RunState) == 80, "RunState is loaded as 5 x 16 bytes");

// Static tables the step kernels read.
struct Bank {
    const DevPC* pcs;
    const DevLevel* lv;
    const float2* W;       // twiddles, 2^wlog entries
    int wlog;
    int N0;
    int n_out;
    int kb;                // base blocks per step (level-0 sub-blocks of one fire); 0 or 1: one
    int kq;                // with kb > 1: most parts a level-0 fire sums itself (shared-memory size)
    int tb;                // bins per spread task of the handle's step kernels (0: the default)
    // per output channel mixing lists (mix_mode 2): out_off[o]..out_off[o+1]
    const int* out_off;
    const int* out_pcs;
    int* mix_cnt;          // per output channel arrival counters (zero between steps)
    const int* zero_list;  // output channels with no unmuted PC
};

}  // namespace pcg
