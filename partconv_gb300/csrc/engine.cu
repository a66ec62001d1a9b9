// engine.cu -- host side of the GB300 partitioned-convolution engine and its
// C ABI (include/partconv_gb300.h).
//
// Replaces PartConvMulti (src/partconvMulti.h:52-148,
// src/partconvMulti.cpp:23-1134 of ebattenberg/partconv): per-PC layout
// validation and IR partitioning (src/partconv.cpp:70-230), device-resident
// FDL state, and the per-callback schedule.  The reference's pthread level
// workers become a static per-phase task table: the level schedule repeats
// every H = max_L N_L / N0 base steps, so for each phase and kernel class the
// host lists the level blocks that fire and the MAC slices spread over the
// steps between a level's blocks.  A base step is one launch per kernel
// class that has work in that phase (level 0 fires every step, so its class
// always runs); batches of steps replay a captured CUDA graph whose nodes
// have their phase baked in.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/partconv_gb300.h"
#include "engine_types.h"
#include "io.h"
#include "kernels.h"

using namespace pcg;

namespace {

constexpr int kWlog = 17;          // twiddle table 2^17 entries: real FFTs up to 2 * 65536
constexpr int kMinGraphSteps = 128;   // base steps per captured graph (a multiple of the hyperperiod)
constexpr int kMinN0 = 16;
constexpr int kClasses = kNumClasses;

bool is_pow2(long x) { return x > 0 && (x & (x - 1)) == 0; }
int ilog2(long x) {
    int p = 0;
    while ((1L << p) < x) ++p;
    return p;
}

int check_layout_impl(int M, const int* N, int* P, int ir_len, bool relaxed, int* delays, std::string& msg) {
    char buf[256];
    if (M < 1) {
        msg = "at least one partitioning level is required";
        return PC_ERR_LAYOUT;
    }
    if (M > PC_MAX_LEVELS) {
        snprintf(buf, sizeof buf, "%d levels exceed the limit of %d", M, PC_MAX_LEVELS);
        msg = buf;
        return PC_ERR_LIMIT;
    }
    for (int i = 0; i < M; ++i) {
        if (!is_pow2(N[i])) {
            snprintf(buf, sizeof buf, "block size of level %d must be a power of 2 (N[%d] = %d)", i, i, N[i]);
            msg = buf;
            return PC_ERR_LAYOUT;
        }
    }
    for (int i = 1; i < M; ++i) {
        if (N[i] <= N[i - 1]) {
            snprintf(buf, sizeof buf, "N[%d]=%d <= N[%d]=%d", i, N[i], i - 1, N[i - 1]);
            msg = buf;
            return PC_ERR_LAYOUT;
        }
    }
    if (N[M - 1] > PC_MAX_BLOCK) {
        snprintf(buf, sizeof buf, "block size %d exceeds the limit of %d", N[M - 1], PC_MAX_BLOCK);
        msg = buf;
        return PC_ERR_LIMIT;
    }
    for (int i = 0; i < M - 1; ++i) {
        if (P[i] < 1) {
            snprintf(buf, sizeof buf, "level %d needs at least one partition", i);
            msg = buf;
            return PC_ERR_LAYOUT;
        }
    }
    long position = 2L * N[0], s = 0;
    for (int i = 0; i < M - 1; ++i) {
        if (delays) delays[i] = (int)(position / N[0]);
        position += (long)N[i] * P[i];
        s += (long)N[i] * P[i];
        const bool ok = relaxed ? (s >= N[i + 1]) : (position >= 2L * N[i + 1]);
        if (!ok) {
            snprintf(buf, sizeof buf, "sufficient delay not allowed for block size of level %d", i + 2);
            msg = buf;
            return PC_ERR_LAYOUT;
        }
    }
    if (delays) delays[M - 1] = (int)(position / N[0]);
    const long rem = (long)ir_len - s;
    // The reference refuses only rem < 0 (src/partconv.cpp:169-170).  With
    // rem == 0 it sets P[M-1] = 0 and its runLevel then computes
    // bcurr % num_parts (partconv.cpp:362), a division by zero; here the
    // layout is refused instead, with the reference's message.
    if (rem <= 0) {
        snprintf(buf, sizeof buf, "last partitioning level (%d) not required", M);
        msg = buf;
        return PC_ERR_LAYOUT;
    }
    P[M - 1] = (int)((rem + N[M - 1] - 1) / N[M - 1]);
    msg.clear();
    return PC_OK;
}

struct PCSpec {
    std::vector<int> N, P;
    std::vector<float> ir;
    int in_ch = 0, out_ch = 0, mute = 0;
    float scale = 1.0f;
};

// bump allocator over one device arena (256-byte aligned pieces)
struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    }
};

}  // namespace

struct pc_handle {
    int verbosity = 0;
    std::string err;
    bool ready = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaStream_t side[kClasses] = {};    // graph-capture branches
    cudaStream_t aside[kClasses] = {};   // deferred fires (graph capture)
    cudaStream_t cin = nullptr, cout = nullptr;   // pc_process copy pipeline

    int fs = 0, N0 = 0, n_in = 0, n_out = 0;
    int relaxed = 0;
    std::vector<PCSpec> specs;

    // device arena
    char* arena = nullptr;
    size_t arena_bytes = 0;
    size_t state_off = 0, state_bytes = 0;   // zeroed by reset

    std::vector<DevPC> h_pcs;
    std::vector<DevLevel> h_lv;
    std::vector<int> lv_cls;   // kernel class of each level's fires (spectra layout follows it)
    Bank bank{};
    int H = 1;        // hyperperiod (base steps)
    int G = 64;       // base steps per captured graph (multiple of H and KB)
    int req_kb = 1;   // base blocks per step requested (pc_set_step_blocks)
    int req_tile_bins = 0, req_tile_parts = 0;   // spread tile shape requested (pc_set_tiles; 0: default)
    int TB = 0, TP = 0;                          // spread tile shape in use: bins and parts per task
    int KB = 1;       // base blocks per step in use: a launch computes KB level-0 blocks
    int Hs = 1;       // task-table phases: steps (of KB base blocks) per hyperperiod
    int maxN = 0;
    int l0_class = 0;

    // per (class, phase) task lists: d_tasks + off[cls][phase], count cnt[cls][phase]
    Task* d_tasks = nullptr;
    std::vector<int> off[kClasses], cnt[kClasses];
    std::vector<double> alg_bytes[kClasses];
    // Deferred fires (levels >= 1 whose output is due more than one step
    // after their block completes; with several base blocks per step, every
    // level >= 1): launched after the step that completed the block, on a
    // low-priority stream, and joined `due` steps later.
    struct DGroup {
        int cls, phase, due, off, cnt;
        double bytes;
    };
    std::vector<DGroup> dgroups;
    std::vector<std::vector<int>> dg_of_phase;   // phase -> indices into dgroups
    // spread tasks of levels >= 1 with several base blocks per step: their own
    // launch per step on `sside`, beside the step chain; only the levels'
    // deferred fires wait for them
    cudaStream_t sside = nullptr;
    std::vector<int> sp_off, sp_cnt;
    std::vector<double> sp_bytes;
    int class_maxN[kClasses] = {};
    RunState* d_rs = nullptr;

    // run() staging and Relaxed carry (planar [n_out][N0])
    float* d_in1 = nullptr;
    float* d_out1 = nullptr;
    float* h_in1 = nullptr;    // pinned host staging of one block (pc_run)
    float* h_out1 = nullptr;
    float* d_carry = nullptr;

    // growable device buffers for pc_process
    float* d_big_in = nullptr;
    float* d_big_out = nullptr;
    size_t big_in_cap = 0, big_out_cap = 0;
    float* d_rtmp = nullptr;
    size_t rtmp_cap = 0;

    cudaGraphExec_t gexec = nullptr;
    long long graph_kernels = 0;   // kernel nodes per replay

    long long frame_num = 0;
    long long launches = 0;
};

namespace {

int fail(pc_handle* h, int code, const std::string& m) {
    if (h) h->err = m;
    return code;
}

int cuda_fail(pc_handle* h, cudaError_t e, const char* where) {
    return fail(h, PC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call, where)                                        \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, where); \
    } while (0)

void free_device(pc_handle* h) {
    if (h->device >= 0) cudaSetDevice(h->device);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    if (h->arena) cudaFree(h->arena);
    if (h->h_in1) cudaFreeHost(h->h_in1);
    if (h->h_out1) cudaFreeHost(h->h_out1);
    h->h_in1 = h->h_out1 = nullptr;
    h->arena = nullptr;
    if (h->d_big_in) cudaFree(h->d_big_in);
    if (h->d_big_out) cudaFree(h->d_big_out);
    if (h->d_rtmp) cudaFree(h->d_rtmp);
    h->d_big_in = h->d_big_out = h->d_rtmp = nullptr;
    h->big_in_cap = h->big_out_cap = h->rtmp_cap = 0;
    for (auto& s : h->side) {
        if (s) cudaStreamDestroy(s);
        s = nullptr;
    }
    for (auto& s : h->aside) {
        if (s) cudaStreamDestroy(s);
        s = nullptr;
    }
    if (h->sside) cudaStreamDestroy(h->sside);
    h->sside = nullptr;
    if (h->cin) cudaStreamDestroy(h->cin);
    if (h->cout) cudaStreamDestroy(h->cout);
    h->cin = h->cout = nullptr;
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    h->ready = false;
}

// task-table phase of the step that starts at base step `step`
int phase_of(const pc_handle* h, long long step) { return (int)((step / h->KB) & (long long)(h->Hs - 1)); }

long long floordiv(long long a, long long b) {
    long long q = a / b;
    return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

// One base step by direct launches (classes with work in this phase).
// first: the preceding work in the stream is not one of this handle's step
// kernels, so the launch must not overlap it.
int launch_step_direct(pc_handle* h, const RunState& rs, cudaStream_t st, bool first) {
    const int ph = phase_of(h, rs.step_base);
    if (h->sp_cnt[ph] > 0) {   // levels' spread tasks first, in stream order
        CK(launch_side_spreads(h->sp_cnt[ph], h->d_tasks + h->sp_off[ph], rs, nullptr, 0, st), "spread launch");
        h->launches += 1;
    }
    for (int k = 0; k < kClasses; ++k) {
        const int cls = (h->l0_class + k) % kClasses;   // level-0 class first
        const int n = h->cnt[cls][ph];
        if (n <= 0) continue;
        CK(launch_step_class(cls, n, h->class_maxN[cls], h->bank, h->d_tasks + h->off[cls][ph], rs, nullptr, 0, st,
                             !first),
           "step launch");
        first = false;
        h->launches += 1;
    }
    // deferred fires of blocks completed by this step, in stream order (a
    // direct step does not overlap them with later steps)
    for (int gi : h->dg_of_phase[ph]) {
        const pc_handle::DGroup& gr = h->dgroups[gi];
        CK(launch_step_class(gr.cls, gr.cnt, h->class_maxN[gr.cls], h->bank, h->d_tasks + gr.off, rs, nullptr, 0, st,
                             !first),
           "deferred fire launch");
        first = false;
        h->launches += 1;
    }
    return PC_OK;
}

// Capture G steps starting at a step with phase 0.  Classes other than the
// level-0 class run on side branches joined at the end of their step.
int build_graph(pc_handle* h) {
    cudaGraph_t g = nullptr;
    std::vector<cudaEvent_t> evs;
    auto mk = [&]() {
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        evs.push_back(e);
        return e;
    };
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(h, e, "begin capture");
    RunState dummy{};
    long long kernels = 0;
    struct Pending {
        int due_step;
        cudaEvent_t done;
    };
    std::vector<Pending> pending;   // deferred fires in flight
    cudaEvent_t sp_last = nullptr;  // completion of the newest side spread launch
    for (int s = 0; s < h->G && e == cudaSuccess; s += h->KB) {   // s: first base step of the step
        const int ph = phase_of(h, s);
        // deferred fires whose output this step emits join the chain here
        for (size_t i = 0; i < pending.size() && e == cudaSuccess;) {
            if (pending[i].due_step <= s) {
                e = cudaStreamWaitEvent(h->stream, pending[i].done, 0);
                pending.erase(pending.begin() + i);
            } else {
                ++i;
            }
        }
        // levels' spread tasks (several base blocks per step): their own branch,
        // waited for only by the levels' deferred fires and the graph's end
        if (h->sp_cnt[ph] > 0 && e == cudaSuccess) {
            cudaEvent_t fork = mk();
            e = cudaEventRecord(fork, h->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->sside, fork, 0);
            if (e == cudaSuccess)
                e = launch_side_spreads(h->sp_cnt[ph], h->d_tasks + h->sp_off[ph], dummy, h->d_rs, s, h->sside);
            cudaEvent_t done = mk();
            if (e == cudaSuccess) e = cudaEventRecord(done, h->sside);
            sp_last = done;
            ++kernels;
        }
        std::vector<cudaEvent_t> joins;
        for (int cls = 0; cls < kClasses && e == cudaSuccess; ++cls) {
            if (cls == h->l0_class || h->cnt[cls][ph] <= 0) continue;
            cudaEvent_t fork = mk();
            e = cudaEventRecord(fork, h->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side[cls], fork, 0);
            if (e == cudaSuccess)
                e = launch_step_class(cls, h->cnt[cls][ph], h->class_maxN[cls], h->bank,
                                      h->d_tasks + h->off[cls][ph], dummy, h->d_rs, s, h->side[cls], false);
            cudaEvent_t join = mk();
            if (e == cudaSuccess) e = cudaEventRecord(join, h->side[cls]);
            joins.push_back(join);
            ++kernels;
        }
        const int c0 = h->l0_class;
        if (e == cudaSuccess)
            e = launch_step_class(c0, h->cnt[c0][ph], h->class_maxN[c0], h->bank, h->d_tasks + h->off[c0][ph], dummy,
                                  h->d_rs, s, h->stream, s > 0, 1);
        ++kernels;
        for (auto j : joins)
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, j, 0);
        // fires of blocks this step completed: forked after the step, low
        // priority, joined before the step that first emits their output
        for (int gi : h->dg_of_phase[ph]) {
            if (e != cudaSuccess) break;
            const pc_handle::DGroup& gr = h->dgroups[gi];
            cudaEvent_t fork = mk();
            e = cudaEventRecord(fork, h->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->aside[gr.cls], fork, 0);
            if (e == cudaSuccess && sp_last) e = cudaStreamWaitEvent(h->aside[gr.cls], sp_last, 0);
            // a large deferred fire takes a whole SM (shared memory), so it
            // never shares one with the step chain's kernels
            if (e == cudaSuccess)
                e = launch_step_class(gr.cls, gr.cnt, h->class_maxN[gr.cls], h->bank, h->d_tasks + gr.off, dummy,
                                      h->d_rs, s, h->aside[gr.cls], false, -1, gr.cls != h->l0_class);
            cudaEvent_t done = mk();
            if (e == cudaSuccess) e = cudaEventRecord(done, h->aside[gr.cls]);
            pending.push_back({s + gr.due * h->KB, done});
            ++kernels;
        }
    }
    // the graph ends with every deferred fire joined (a replay must not
    // overlap the next one's state update)
    for (auto& pd : pending)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, pd.done, 0);
    if (sp_last && e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, sp_last, 0);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    for (auto ev : evs) cudaEventDestroy(ev);
    if (e == cudaSuccess) e = e2;
    // with several base blocks per step the graph runs its nodes at their own
    // priorities (chain high, deferred fires low): 61.3k against 60.3k
    // audio-s/s on 32 streams; with one block per step that slowed the chain
    // (58.0k against 59.6k), so it keeps the stream's priority
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&h->gexec, g, h->KB > 1 ? cudaGraphInstantiateFlagUseNodePriority : 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph capture");
    h->graph_kernels = kernels;
    return PC_OK;
}

int do_setup(pc_handle* h, int fs, int buffer_size, int n_in, int n_out, std::vector<PCSpec>&& specs) {
    if (h->ready) return fail(h, PC_ERR_STATE, "setup called twice without cleanup");
    if (buffer_size < kMinN0 || !is_pow2(buffer_size))
        return fail(h, PC_ERR_ARG, "buffer_size must be a power of two >= 16");
    if (n_in < 1 || n_out < 1 || specs.empty()) return fail(h, PC_ERR_ARG, "need >= 1 input, output and PC");
    for (size_t i = 0; i < specs.size(); ++i) {
        PCSpec& p = specs[i];
        if (p.in_ch < 0 || p.in_ch >= n_in || p.out_ch < 0 || p.out_ch >= n_out)
            return fail(h, PC_ERR_ARG, "PC " + std::to_string(i) + ": channel index out of range");
        if (p.N.empty() || p.N[0] != buffer_size)
            return fail(h, PC_ERR_LAYOUT, "PC " + std::to_string(i) + ": first block size must equal buffer_size");
        std::string msg;
        int r = check_layout_impl((int)p.N.size(), p.N.data(), p.P.data(), (int)p.ir.size(), true, nullptr, msg);
        if (r) return fail(h, r, "PC " + std::to_string(i) + ": " + msg);
    }

    int dev = 0;
    CK(cudaGetDevice(&dev), "cudaGetDevice");
    h->device = dev;
    int prio_least = 0, prio_greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest), "priority range");
    CK(cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_greatest), "stream create");
    for (auto& s : h->side) CK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio_greatest), "stream create");
    for (auto& s : h->aside) CK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio_least), "stream create");
    CK(cudaStreamCreateWithPriority(&h->sside, cudaStreamNonBlocking, prio_least), "stream create");
    CK(prepare_kernels(), "kernel attributes");

    h->fs = fs;
    h->N0 = buffer_size;
    h->n_in = n_in;
    h->n_out = n_out;
    h->specs = std::move(specs);
    const int N0 = buffer_size;
    const int npc = (int)h->specs.size();

    int nlv = 0, maxN = 0, Hh = 1;
    for (auto& p : h->specs) {
        nlv += (int)p.N.size();
        maxN = std::max(maxN, p.N.back());
        Hh = std::max(Hh, p.N.back() / N0);
    }
    h->H = Hh;
    h->G = std::max(Hh, kMinGraphSteps);
    h->maxN = maxN;
    h->l0_class = fire_class_of(N0);
    // base blocks per step: at most what the level-0 kernel supports, and
    // every level >= 1 must span a whole number of steps
    int KB = std::min(h->req_kb, max_step_blocks(N0));
    for (auto& p : h->specs)
        for (size_t L = 1; L < p.N.size(); ++L)
            while (KB > 1 && (p.N[L] / N0) % KB) KB >>= 1;
    h->KB = KB;
    h->Hs = std::max(1, Hh / KB);
    // spread tile shape: bins and parts per spread task
    const int TB = h->req_tile_bins > 0 ? h->req_tile_bins : spread_task_bins();
    const int TP = h->req_tile_parts > 0 ? h->req_tile_parts : spread_task_parts();
    h->TB = TB;
    h->TP = TP;
    // parts a K-block level-0 fire sums itself; spread rows take the rest
    const int QC = KB > 1 ? multi_fire_parts(N0, KB) : 2;
    h->G = std::max(h->G, KB);

    // ---- arena layout --------------------------------------------------------------
    Carve cv;
    const size_t off_W = cv.take(sizeof(float2) << kWlog);
    const size_t off_pcs = cv.take(sizeof(DevPC) * npc);
    const size_t off_lv = cv.take(sizeof(DevLevel) * nlv);
    std::vector<size_t> off_H(nlv);
    {
        int li = 0;
        for (auto& p : h->specs)
            for (size_t L = 0; L < p.N.size(); ++L, ++li)
                off_H[li] = cv.take(sizeof(float2) * (size_t)p.P[L] * (p.N[L] + 2));
    }
    std::vector<std::vector<int>> out_list(n_out);
    for (int i = 0; i < npc; ++i)
        if (!h->specs[i].mute) out_list[h->specs[i].out_ch].push_back(i);
    std::vector<int> out_off(n_out + 1, 0), out_pcs, zero_list;
    for (int o = 0; o < n_out; ++o) {
        out_off[o + 1] = out_off[o] + (int)out_list[o].size();
        for (int q : out_list[o]) out_pcs.push_back(q);
        if (out_list[o].empty()) zero_list.push_back(o);
    }
    const size_t off_out_off = cv.take(sizeof(int) * (n_out + 1));
    const size_t off_out_pcs = cv.take(sizeof(int) * std::max<size_t>(1, out_pcs.size()));
    const size_t off_zero = cv.take(sizeof(int) * std::max<size_t>(1, zero_list.size()));
    const size_t off_rs = cv.take(sizeof(RunState));
    const size_t off_in1 = cv.take(sizeof(float) * (size_t)N0 * n_in);
    const size_t off_out1 = cv.take(sizeof(float) * (size_t)N0 * n_out);
    // task table size is known only after enumeration; it goes last in the static part
    const size_t off_tasks_placeholder = cv.off;
    (void)off_tasks_placeholder;

    // state (zeroed by reset), laid out after the task table below
    struct StateOffsets {
        std::vector<size_t> xring, pcout, X, Yp, yr;
        size_t mix = 0, carry = 0;
    } so;
    // Deferral window of each level (0: fires within its step).  Level L's
    // first output sample of a block is due slack = (s_L - N_L)/N0 steps
    // after the step that completes the block; the fire is deferred by
    // w = min(slack, T - 2) steps so that it is joined before the level's
    // next block completes (the spreads of the block after next read its
    // spectrum).  Its window stays in the input ring meanwhile.
    //
    // With KB > 1 base blocks per step every level >= 1 is deferred: its
    // block completes inside some step S, its fire is launched after S and
    // joined w' + 1 steps later, w' = min(floor(slack / KB), N_L / (KB N0) - 1).
    // The first output sample is due at the start of step S + floor(slack /
    // KB) + 1 (outputs of a level block start on a multiple of N_L, a
    // multiple of KB N0), and the cap keeps the fire ahead of the spreads of
    // the block after next.
    // dfl: the level runs in the deferred form (parts >= 2 from double-buffered rows).
    std::vector<int> rin(npc), rl(nlv), dwin(nlv, 0), dfl(nlv, 0);
    {
        int li = 0;
        for (int i = 0; i < npc; ++i) {
            const PCSpec& p = h->specs[i];
            long need = std::max(2L * p.N.back(), (long)(KB + 1) * N0);
            long sacc = 0;
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                const long T = p.N[L] / N0, sb = sacc / N0;
                if (L > 0 && KB > 1) {
                    const long w = std::min((sb - T) / KB, T / KB - 1);
                    dwin[li] = (int)w;
                    dfl[li] = 1;
                    need = std::max(need, 2L * p.N[L] + (w + 1) * (long)KB * N0);
                } else if (L > 0 && T >= 4) {
                    const long w = std::min(sb - T, T - 2);
                    if (w >= 1) {
                        dwin[li] = (int)w;
                        dfl[li] = 1;
                        need = std::max(need, 2L * p.N[L] + (w + 1) * (long)N0);
                    }
                }
                sacc += (long)p.N[L] * p.P[L];
            }
            long r = 1;
            while (r < need) r <<= 1;
            rin[i] = (int)r;
        }
    }
    {
        int li = 0;
        for (auto& p : h->specs) {
            long s = 0;
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                long r = p.N[L];
                while (r < s + (long)KB * N0) r <<= 1;
                rl[li] = (int)r;
                s += (long)p.N[L] * p.P[L];
            }
        }
    }
    // Kernel class per level.  A fire within its step sits on the step chain,
    // where its latency counts: levels of 8192 and 16384 samples then run on
    // a cluster (class 3) when few of them share a handle, so that all their
    // clusters fit the GPU at once; otherwise (and for deferred fires, which
    // overlap later steps) one CTA per fire.
    h->lv_cls.assign(nlv, 0);
    {
        int li = 0, instep_big = 0;
        for (auto& p : h->specs)
            for (size_t L = 0; L < p.N.size(); ++L, ++li)
                if (L > 0 && KB == 1 && dfl[li] == 0 && p.N[L] >= kClusterInStepMinN && p.N[L] <= kMaxBlockOneCta)
                    ++instep_big;
        const bool few = instep_big * kClusterCtas <= kClusterInStepMaxCtas;
        li = 0;
        for (auto& p : h->specs)
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                h->lv_cls[li] = fire_class_of(p.N[L]);
                if (few && L > 0 && KB == 1 && dfl[li] == 0 && p.N[L] >= kClusterInStepMinN) h->lv_cls[li] = 3;
            }
    }

    // ---- descriptors (host) ----------------------------------------------------------
    h->h_pcs.assign(npc, DevPC{});
    h->h_lv.assign(nlv, DevLevel{});
    {
        int li = 0;
        for (int i = 0; i < npc; ++i) {
            PCSpec& p = h->specs[i];
            DevPC& d = h->h_pcs[i];
            d.M = (int)p.N.size();
            d.lv0 = li;
            d.in_ch = p.in_ch;
            d.out_ch = p.out_ch;
            d.mute = p.mute;
            d.mix_mode = p.mute ? 0 : (out_list[p.out_ch].size() == 1 ? 1 : 2);
            d.zero_outs = (i == 0) ? (int)zero_list.size() : 0;
            d.zero_off = 0;
            d.scale = p.scale;
            d.rin_mask = rin[i] - 1;
            long s = 0;
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                DevLevel& l = h->h_lv[li];
                l.N = p.N[L];
                l.logN = ilog2(p.N[L]);
                l.P = p.P[L];
                l.T = p.N[L] / N0;
                l.s_blocks = (int)(s / N0);
                l.cs = p.N[L] + 2;
                l.rmask = rl[li] - 1;
                l.pc = i;
                {   // spread tasks sum parts >= 2 KB (level 0), >= 2 (deferred levels) or >= 1
                    const int p_lo = L == 0 ? (KB > 1 ? std::min(p.P[L], QC) : 2) : (dfl[li] ? 2 : 1);
                    const int np = p.P[L] - p_lo;
                    l.npart = np > 0 ? (np + TP - 1) / TP : 1;
                }
                s += (long)p.N[L] * p.P[L];
            }
        }
    }

    // ---- per (class, phase) task lists ------------------------------------------------
    // Tasks point into the arena, so they are built after the state offsets
    // are known; first count them to size the table.
    const int NP = h->Hs;   // phases
    std::vector<std::vector<std::vector<Task>>> lists(kClasses, std::vector<std::vector<Task>>(NP));
    std::map<std::tuple<int, int, int>, std::vector<Task>> dlists;   // (phase, due, class) -> deferred fires
    std::map<std::tuple<int, int, int>, double> dbytes;
    std::vector<std::vector<Task>> sp_lists(NP);   // side spread tasks per phase (KB > 1)
    h->sp_bytes.assign(NP, 0.0);
    for (int cls = 0; cls < kClasses; ++cls) h->alg_bytes[cls].assign(NP, 0.0);
    // order: larger fires first (longest CTAs start first), then level-0
    // fires, then spread tasks, also larger levels first (their slices read
    // the most; measured 1 % faster on 32 streams of three levels than level
    // 0 first)
    std::vector<int> order(nlv);
    for (int i = 0; i < nlv; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h->h_lv[a].N > h->h_lv[b].N; });
    for (int g = 0; g < NP && KB == 1; ++g) {
        for (int li : order) {
            const DevLevel& l = h->h_lv[li];
            if ((g + 1 + l.s_blocks) % l.T) continue;
            const DevPC& d = h->h_pcs[l.pc];
            Task t{};
            t.kind = 0;
            t.N = l.N;
            t.logN = l.logN;
            t.P = l.P;
            t.T = l.T;
            t.s_blocks = l.s_blocks;
            t.cs = l.cs;
            t.rmask = l.rmask;
            t.M = d.M;
            t.in_ch = d.in_ch;
            t.out_ch = d.out_ch;
            t.mix_mode = d.mix_mode;
            t.zero_outs = (l.T == 1) ? d.zero_outs : 0;
            t.zero_off = d.zero_off;
            t.rin_mask = d.rin_mask;
            t.lv_index = li;
            t.scale = d.scale;
            const int cls = h->lv_cls[li];
            // bytes a fire must move: H0 row read, new X row written, the
            // partial-sum row read (level 0 and deferred levels also X_{b-1}
            // and H_1 rows), the 2N-sample window read, N samples written;
            // level 0 also reads the other levels' due slices and appends N0
            // input samples
            const double C = l.N + 1.0;
            double b = 8.0 * C * 2.0 + 12.0 * l.N;
            if (l.T == 1 || dwin[li] > 0) {
                b += 8.0 * C * (l.P >= 2 ? 2.0 : 0.0) + (l.P >= 3 ? 8.0 * C * l.npart : 0.0);
                if (l.T == 1) b += 4.0 * N0 * (d.M - 1) + 4.0 * N0;
            } else if (l.P >= 2) {
                b += 8.0 * C * l.npart;
            }
            t.k0 = l.npart;   // partial-sum rows the fire adds
            if (dwin[li] > 0) {
                t.dfer = 1;
                dlists[std::make_tuple(g, dwin[li] + 1, cls)].push_back(t);
                dbytes[std::make_tuple(g, dwin[li] + 1, cls)] += b;
                continue;
            }
            lists[cls][g].push_back(t);
            h->alg_bytes[cls][g] += b;
        }
        const int sc = h->l0_class;
        for (int li : order) {
            const DevLevel& l = h->h_lv[li];
            int lo, hi, p_lo;
            if (l.T == 1) {
                if (l.P < 3) continue;
                lo = 0;
                hi = l.cs;
                p_lo = 2;
            } else if (dwin[li] > 0) {
                // parts >= 2 of the next deferred fire, in T slices over all
                // phases (the fire's own step builds the last slice)
                if (l.P < 3) continue;
                const int phi = (g + 1 + l.s_blocks) % l.T;
                const int j = (phi + l.T - 1) % l.T, nch = l.T;
                lo = (int)(((long)j * l.cs / nch) & ~1L);
                hi = (j == nch - 1) ? l.cs : (int)(((long)(j + 1) * l.cs / nch) & ~1L);
                p_lo = 2;
            } else {
                if (l.P < 2) continue;
                const int phi = (g + 1 + l.s_blocks) % l.T;
                if (phi == 0) continue;
                const int j = phi - 1, nch = l.T - 1;
                lo = (int)(((long)j * l.cs / nch) & ~1L);
                hi = (j == nch - 1) ? l.cs : (int)(((long)(j + 1) * l.cs / nch) & ~1L);
                p_lo = 1;
            }
            for (int k0 = lo; k0 < hi; k0 += TB)
                for (int r = 0; r < l.npart; ++r) {   // parts [p_lo + TP r, p_lo + TP (r + 1)) into row r
                    Task t{};
                    t.kind = 1;
                    t.N = l.N;
                    t.P = l.P;
                    t.T = l.T;
                    t.s_blocks = l.s_blocks;
                    t.cs = l.cs;
                    t.M = TB;   // bins per task
                    t.k0 = k0;
                    t.k1 = std::min(hi, k0 + TB);
                    t.p_lo = p_lo + r * TP;
                    t.in_ch = std::min(l.P, p_lo + (r + 1) * TP);
                    t.out_ch = r;
                    t.lv_index = li;
                    t.dfer = dwin[li] > 0;
                    lists[sc][g].push_back(t);
                }
            h->alg_bytes[sc][g] += (16.0 * (l.P - p_lo) + 8.0 * l.npart) * (hi - lo);
        }
    }
    // Several base blocks per step (KB > 1): step S covers base steps
    // S KB .. S KB + KB - 1 and has phase S mod NP (every level's pattern
    // repeats every N_L / (KB N0) steps, which divides NP).  A task sees the
    // base step c = S KB - origin.
    for (int g = 0; g < NP && KB > 1; ++g) {
        const long long S = g, c0 = S * KB;
        auto fire_task = [&](int li) {
            const DevLevel& l = h->h_lv[li];
            const DevPC& d = h->h_pcs[l.pc];
            Task t{};
            t.kind = 0;
            t.N = l.N;
            t.logN = l.logN;
            t.P = l.P;
            t.T = l.T;
            t.s_blocks = l.s_blocks;
            t.cs = l.cs;
            t.rmask = l.rmask;
            t.M = d.M;
            t.in_ch = d.in_ch;
            t.out_ch = d.out_ch;
            t.mix_mode = d.mix_mode;
            t.zero_outs = (l.T == 1) ? d.zero_outs : 0;
            t.zero_off = d.zero_off;
            t.rin_mask = d.rin_mask;
            t.lv_index = li;
            t.scale = d.scale;
            return t;
        };
        for (int li : order) {
            const DevLevel& l = h->h_lv[li];
            const DevPC& d = h->h_pcs[l.pc];
            const double C = l.N + 1.0;
            const int cls = h->lv_cls[li];
            if (l.T == 1) {   // level 0: KB blocks, parts < 2 KB in the fire
                Task t = fire_task(li);
                const int Q = std::min(l.P, QC);
                const int rows = l.P > Q ? l.npart : 0;
                t.k0 = rows;
                t.p_lo = Q;
                // per block: H_0 read and the new X row written, Q - 1 older
                // (H, X) row pairs, the partial-sum rows, 2N window samples read
                // and N written, the other levels' due slices, the ring append
                const double b = 16.0 * C * Q + 8.0 * C * rows + 12.0 * l.N + 4.0 * N0 * (d.M - 1) + 4.0 * N0;
                lists[cls][g].push_back(t);
                h->alg_bytes[cls][g] += KB * b;
                continue;
            }
            // the level's block that completes within this step, if any
            const long long r = (c0 + 1 + l.s_blocks) % l.T;
            const long long cb = c0 + (r == 0 ? 0 : l.T - r);
            if (cb >= c0 + KB) continue;
            Task t = fire_task(li);
            t.k0 = l.npart;
            t.dfer = 1;
            t.origin = -(cb - c0);
            const double b =
                16.0 * C + 12.0 * l.N + 8.0 * C * (l.P >= 2 ? 2.0 : 0.0) + (l.P >= 3 ? 8.0 * C * l.npart : 0.0);
            dlists[std::make_tuple(g, dwin[li] + 1, cls)].push_back(t);
            dbytes[std::make_tuple(g, dwin[li] + 1, cls)] += b;
        }
        const int sc = h->l0_class;
        for (int li = 0; li < nlv; ++li) {
            const DevLevel& l = h->h_lv[li];
            // level 0's K-block spreads (spread_multi) keep the default tile width
            const int tb = l.T == 1 ? spread_task_bins() : TB;
            auto add_spreads = [&](int lo, int hi, int p_lo, long long origin, std::vector<Task>& dst, double& bytes,
                                   double blocks) {
                for (int k0 = lo; k0 < hi; k0 += tb)
                    for (int q = 0; q < l.npart; ++q) {   // parts [p_lo + TP q, p_lo + TP (q + 1)) into row q
                        Task t{};
                        t.kind = 1;
                        t.N = l.N;
                        t.P = l.P;
                        t.T = l.T;
                        t.s_blocks = l.s_blocks;
                        t.cs = l.cs;
                        t.M = tb;   // bins per task
                        t.k0 = k0;
                        t.k1 = std::min(hi, k0 + tb);
                        t.p_lo = p_lo + q * TP;
                        t.in_ch = std::min(l.P, p_lo + (q + 1) * TP);
                        t.out_ch = q;
                        t.lv_index = li;
                        t.dfer = l.T > 1;
                        t.origin = origin;
                        dst.push_back(t);
                    }
                bytes += blocks * (16.0 * (l.P - p_lo) + 8.0 * l.npart) * (hi - lo);
            };
            if (l.T == 1) {   // parts >= Q of the next step's blocks S KB + KB .. S KB + 2 KB - 1
                if (l.P <= QC) continue;
                add_spreads(0, l.cs, QC, -(long long)(KB - 1), lists[sc][g], h->alg_bytes[sc][g], KB);
                continue;
            }
            if (l.P < 3) continue;
            // parts >= 2 of the first block completing at or after this step's
            // start, in N_L / (KB N0) slices over the steps after the step in
            // which its predecessor completed
            const long long bt = (c0 + l.s_blocks) / l.T;
            const long long sprev = floordiv(bt * l.T - l.s_blocks - 1, KB);
            const int nch = l.T / KB;
            const long long j = S - 1 - sprev;
            if (j < 0 || j >= nch) {
                free_device(h);
                return fail(h, PC_ERR_STATE, "internal: spread slice out of range");
            }
            const int lo = (int)((j * l.cs / nch) & ~1LL);
            const int hi = (j == nch - 1) ? l.cs : (int)(((j + 1) * l.cs / nch) & ~1LL);
            add_spreads(lo, hi, 2, 1, sp_lists[g], h->sp_bytes[g], 1.0);
        }
    }
    size_t ntasks = 0;
    for (int cls = 0; cls < kClasses; ++cls) {
        h->off[cls].assign(NP + 1, 0);
        h->cnt[cls].assign(NP, 0);
        for (int g = 0; g < NP; ++g) {
            h->off[cls][g] = (int)ntasks;
            h->cnt[cls][g] = (int)lists[cls][g].size();
            ntasks += lists[cls][g].size();
        }
        h->off[cls][NP] = (int)ntasks;
    }
    h->dgroups.clear();
    h->dg_of_phase.assign(NP, {});
    for (auto& kv : dlists) {
        pc_handle::DGroup gr;
        gr.phase = std::get<0>(kv.first);
        gr.due = std::get<1>(kv.first);
        gr.cls = std::get<2>(kv.first);
        gr.off = (int)ntasks;
        gr.cnt = (int)kv.second.size();
        gr.bytes = dbytes[kv.first];
        h->dg_of_phase[gr.phase].push_back((int)h->dgroups.size());
        h->dgroups.push_back(gr);
        ntasks += kv.second.size();
    }
    h->sp_off.assign(NP, 0);
    h->sp_cnt.assign(NP, 0);
    for (int g = 0; g < NP; ++g) {
        h->sp_off[g] = (int)ntasks;
        h->sp_cnt[g] = (int)sp_lists[g].size();
        ntasks += sp_lists[g].size();
    }
    const size_t off_tasks = cv.take(sizeof(Task) * std::max<size_t>(1, ntasks));

    // state region
    const size_t state_begin = cv.take(0);
    so.xring.resize(npc);
    so.pcout.resize(npc);
    for (int i = 0; i < npc; ++i) {
        so.xring[i] = cv.take(sizeof(float) * rin[i]);
        so.pcout[i] = cv.take(sizeof(float) * N0 * KB);
    }
    so.X.resize(nlv);
    so.Yp.resize(nlv);
    so.yr.resize(nlv);
    for (int li = 0; li < nlv; ++li) {
        const DevLevel& l = h->h_lv[li];
        so.X[li] = cv.take(sizeof(float2) * (size_t)l.P * l.cs);
        so.Yp[li] = cv.take(sizeof(float2) * 2 * (l.T == 1 ? KB : 1) * (size_t)l.npart * l.cs);
        so.yr[li] = cv.take(sizeof(float) * (size_t)(l.rmask + 1));
    }
    so.mix = cv.take(sizeof(int) * n_out);
    so.carry = cv.take(sizeof(float) * (size_t)N0 * n_out);
    const size_t state_end = cv.take(0);

    h->arena_bytes = cv.off;
    cudaError_t e = cudaMalloc(&h->arena, h->arena_bytes);
    if (e != cudaSuccess) {
        free_device(h);
        return fail(h, PC_ERR_NOMEM, std::string("device allocation of ") + std::to_string(h->arena_bytes) +
                                         " bytes failed: " + cudaGetErrorString(e));
    }
    char* A = h->arena;
    h->state_off = state_begin;
    h->state_bytes = state_end - state_begin;
    CK(cudaMemsetAsync(A + state_begin, 0, h->state_bytes, h->stream), "memset state");

    // pointers into the arena
    for (int i = 0; i < npc; ++i) {
        h->h_pcs[i].xring = reinterpret_cast<float*>(A + so.xring[i]);
        h->h_pcs[i].pcout = reinterpret_cast<float*>(A + so.pcout[i]);
    }
    for (int li = 0; li < nlv; ++li) {
        DevLevel& l = h->h_lv[li];
        l.H = reinterpret_cast<float2*>(A + off_H[li]);
        l.X = reinterpret_cast<float2*>(A + so.X[li]);
        l.Yp = reinterpret_cast<float2*>(A + so.Yp[li]);
        l.yring = reinterpret_cast<float*>(A + so.yr[li]);
    }
    std::vector<Task> all_tasks;
    all_tasks.reserve(ntasks);
    std::vector<const std::vector<Task>*> in_order;
    for (int cls = 0; cls < kClasses; ++cls)
        for (int g = 0; g < NP; ++g) in_order.push_back(&lists[cls][g]);
    for (auto& kv : dlists) in_order.push_back(&kv.second);
    for (int g = 0; g < NP; ++g) in_order.push_back(&sp_lists[g]);
    for (const auto* lst : in_order)
            for (Task t : *lst) {
                const DevLevel& l = h->h_lv[t.lv_index];
                const DevPC& d = h->h_pcs[l.pc];
                t.H = l.H;
                t.X = l.X;
                t.Yp = l.Yp;
                t.yring = l.yring;
                t.xring = d.xring;
                t.pcout = d.pcout;
                if (t.kind == 0 && t.T == 1)
                    for (int L = 1; L <= kEmitLevels && L < d.M; ++L) {
                        t.eyring[L - 1] = h->h_lv[d.lv0 + L].yring;
                        t.emask[L - 1] = h->h_lv[d.lv0 + L].rmask;
                    }
                all_tasks.push_back(t);
            }
    h->d_tasks = reinterpret_cast<Task*>(A + off_tasks);
    if (!all_tasks.empty())
        CK(cudaMemcpyAsync(h->d_tasks, all_tasks.data(), sizeof(Task) * all_tasks.size(), cudaMemcpyHostToDevice,
                           h->stream),
           "upload tasks");
    for (int cls = 0; cls < kClasses; ++cls) h->class_maxN[cls] = 0;
    for (int li = 0; li < nlv; ++li) {
        const int cls = h->lv_cls[li];
        h->class_maxN[cls] = std::max(h->class_maxN[cls], h->h_lv[li].N);
    }
    // the level-0 class also runs spread tasks; its smem must fit its fires
    if (h->class_maxN[h->l0_class] == 0) h->class_maxN[h->l0_class] = N0;

    // twiddles, computed in double
    {
        std::vector<float2> W((size_t)1 << kWlog);
        for (size_t m = 0; m < W.size(); ++m) {
            const double a = -2.0 * M_PI * (double)m / (double)W.size();
            W[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        CK(cudaMemcpyAsync(A + off_W, W.data(), sizeof(float2) * W.size(), cudaMemcpyHostToDevice, h->stream),
           "upload twiddles");
        CK(cudaStreamSynchronize(h->stream), "sync");
    }
    CK(cudaMemcpyAsync(A + off_pcs, h->h_pcs.data(), sizeof(DevPC) * npc, cudaMemcpyHostToDevice, h->stream),
       "upload PCs");
    CK(cudaMemcpyAsync(A + off_lv, h->h_lv.data(), sizeof(DevLevel) * nlv, cudaMemcpyHostToDevice, h->stream),
       "upload levels");
    CK(cudaMemcpyAsync(A + off_out_off, out_off.data(), sizeof(int) * out_off.size(), cudaMemcpyHostToDevice,
                       h->stream),
       "upload mix");
    if (!out_pcs.empty())
        CK(cudaMemcpyAsync(A + off_out_pcs, out_pcs.data(), sizeof(int) * out_pcs.size(), cudaMemcpyHostToDevice,
                           h->stream),
           "upload mix");
    if (!zero_list.empty())
        CK(cudaMemcpyAsync(A + off_zero, zero_list.data(), sizeof(int) * zero_list.size(), cudaMemcpyHostToDevice,
                           h->stream),
           "upload zero list");
    h->d_rs = reinterpret_cast<RunState*>(A + off_rs);
    h->d_in1 = reinterpret_cast<float*>(A + off_in1);
    h->d_out1 = reinterpret_cast<float*>(A + off_out1);
    // pinned staging: a callback's block crosses PCIe/C2C as a true async
    // copy instead of a driver-staged pageable one
    CK(cudaHostAlloc(reinterpret_cast<void**>(&h->h_in1), sizeof(float) * (size_t)N0 * n_in, cudaHostAllocDefault),
       "pinned staging");
    CK(cudaHostAlloc(reinterpret_cast<void**>(&h->h_out1), sizeof(float) * (size_t)N0 * n_out, cudaHostAllocDefault),
       "pinned staging");
    h->d_carry = reinterpret_cast<float*>(A + so.carry);

    h->bank.pcs = reinterpret_cast<const DevPC*>(A + off_pcs);
    h->bank.lv = reinterpret_cast<const DevLevel*>(A + off_lv);
    h->bank.W = reinterpret_cast<const float2*>(A + off_W);
    h->bank.wlog = kWlog;
    h->bank.N0 = N0;
    h->bank.kb = KB;
    h->bank.tb = TB;
    h->bank.kq = 0;
    for (auto& p : h->specs) h->bank.kq = std::max(h->bank.kq, std::min(p.P[0], QC));
    h->bank.n_out = n_out;
    h->bank.out_off = reinterpret_cast<const int*>(A + off_out_off);
    h->bank.out_pcs = reinterpret_cast<const int*>(A + off_out_pcs);
    h->bank.mix_cnt = reinterpret_cast<int*>(A + so.mix);
    h->bank.zero_list = reinterpret_cast<const int*>(A + off_zero);

    // ---- filter spectra: one CTA per (PC, level, part) row -------------------------------
    {
        std::vector<float*> d_irs(npc, nullptr);
        std::vector<std::vector<SpectraJob>> jobs(kClasses);
        int rc = PC_OK;
        for (int i = 0; i < npc && rc == PC_OK; ++i) {
            PCSpec& p = h->specs[i];
            e = cudaMalloc(&d_irs[i], sizeof(float) * std::max<size_t>(1, p.ir.size()));
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_irs[i], p.ir.data(), sizeof(float) * p.ir.size(), cudaMemcpyHostToDevice,
                                    h->stream);
            if (e != cudaSuccess) {
                rc = fail(h, PC_ERR_NOMEM, std::string("IR upload failed: ") + cudaGetErrorString(e));
                break;
            }
            long s = 0;
            for (size_t L = 0; L < p.N.size(); ++L) {
                const DevLevel& l = h->h_lv[h->h_pcs[i].lv0 + L];
                for (int q = 0; q < l.P; ++q) {
                    const long start = s + (long)q * l.N;
                    SpectraJob jb;
                    jb.src = d_irs[i] + std::min<long>(start, (long)p.ir.size());
                    jb.len = (int)std::max<long>(0, std::min<long>(l.N, (long)p.ir.size() - start));
                    jb.N = l.N;
                    jb.logN = l.logN;
                    jb.dst = l.H + (size_t)q * l.cs;
                    jobs[h->lv_cls[h->h_pcs[i].lv0 + L]].push_back(jb);
                }
                s += (long)l.N * l.P;
            }
        }
        std::vector<SpectraJob*> d_jobs(kClasses, nullptr);
        for (int cls = 0; cls < kClasses && rc == PC_OK; ++cls) {
            if (jobs[cls].empty()) continue;
            int mN = 0;
            for (auto& j : jobs[cls]) mN = std::max(mN, j.N);
            e = cudaMalloc(&d_jobs[cls], sizeof(SpectraJob) * jobs[cls].size());
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_jobs[cls], jobs[cls].data(), sizeof(SpectraJob) * jobs[cls].size(),
                                    cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess)
                e = launch_spectra(cls, (int)jobs[cls].size(), mN, d_jobs[cls], h->bank.W, kWlog, h->stream);
            if (e != cudaSuccess) rc = cuda_fail(h, e, "filter spectra");
            else h->launches += 1;
        }
        cudaError_t se = cudaStreamSynchronize(h->stream);
        for (auto q : d_irs)
            if (q) cudaFree(q);
        for (auto q : d_jobs)
            if (q) cudaFree(q);
        if (rc == PC_OK && se != cudaSuccess) rc = cuda_fail(h, se, "filter spectra");
        if (rc) {
            std::string m = h->err;
            free_device(h);
            h->err = m;
            return rc;
        }
    }

    int r = build_graph(h);
    if (r) {
        std::string m = h->err;
        free_device(h);
        h->err = m;
        return r;
    }
    h->frame_num = 0;
    h->ready = true;
    if (h->verbosity > 0) {
        printf("partconv_gb300: %d PCs, N0 = %d, hyperperiod %d steps, %zu tasks, %.1f MB device\n", npc, N0, Hh,
               ntasks, h->arena_bytes / 1e6);
        for (int i = 0; i < npc; ++i) {
            printf("  PC %d: ", i);
            for (size_t L = 0; L < h->specs[i].N.size(); ++L)
                printf("%dx%d%s", h->specs[i].N[L], h->specs[i].P[L], L + 1 < h->specs[i].N.size() ? ", " : "\n");
        }
    }
    return PC_OK;
}

// ch_stride: frames between channel rows of a planar buffer (0: frames)
IOView make_view(const pc_handle* h, const float* in, float* out, long long frames, int layout, long long step0,
                 long long ch_stride = 0) {
    if (ch_stride <= 0) ch_stride = frames;
    IOView v;
    v.in = in;
    v.out = out;
    v.step0 = step0;
    if (layout == PC_PLANAR) {
        v.in_step = h->N0;
        v.in_sample = 1;
        v.in_ch = ch_stride;
        v.out_step = h->N0;
        v.out_sample = 1;
        v.out_ch = ch_stride;
    } else {
        v.in_step = (long long)h->N0 * h->n_in;
        v.in_sample = h->n_in;
        v.in_ch = 1;
        v.out_step = (long long)h->N0 * h->n_out;
        v.out_sample = h->n_out;
        v.out_ch = 1;
    }
    return v;
}

// Run nsteps base steps starting at h->frame_num through the view: direct
// launches up to the next graph boundary, graph replays, direct remainder.
int run_steps(pc_handle* h, const IOView& view, long long nsteps, cudaStream_t st) {
    long long done = 0;
    RunState rs;
    rs.io = view;
    bool first = true;   // the stream's preceding work is not a step kernel
    auto direct = [&](long long upto) -> int {
        for (; done < upto; done += h->KB) {
            rs.step_base = h->frame_num + done;
            int r = launch_step_direct(h, rs, st, first);
            if (r) return r;
            first = false;
        }
        return PC_OK;
    };
    const long long G = h->G;
    const long long misalign = (G - (h->frame_num % G)) % G;
    int r = direct(std::min(nsteps, misalign));
    if (r) return r;
    while (nsteps - done >= G && h->gexec) {
        rs.step_base = h->frame_num + done;
        CK(launch_set_state(h->d_rs, rs, st), "state launch");
        CK(cudaGraphLaunch(h->gexec, st), "graph launch");
        h->launches += 1 + h->graph_kernels;
        done += G;
        first = true;
    }
    r = direct(nsteps);
    if (r) return r;
    h->frame_num += nsteps;
    return PC_OK;
}

__global__ void relaxed_shift_kernel(float* out, const float* res, const float* carry, long long frames, int N0,
                                     int n_out, long long os, long long oc) {
    // out[t] = t < N0 ? carry[t] : res[t - N0] (per channel); views share strides
    const long long total = frames * n_out;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i / n_out;
        const int ch = (int)(i - t * n_out);
        float v = (t < N0) ? carry[(long long)ch * N0 + t] : res[(t - N0) * os + ch * oc];
        out[t * os + ch * oc] = v;
    }
}

__global__ void relaxed_carry_kernel(float* carry, const float* res, long long frames, int N0, int n_out,
                                     long long os, long long oc) {
    const int total = N0 * n_out;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int t = i / n_out, ch = i - (i / n_out) * n_out;
        carry[(long long)ch * N0 + t] = res[(frames - N0 + t) * os + ch * oc];
    }
}

int process_device_impl(pc_handle* h, float* d_out, const float* d_in, long long frames, int layout,
                        cudaStream_t st) {
    if (!h->ready) return fail(h, PC_ERR_STATE, "process before setup");
    if (!d_out || !d_in || frames <= 0 || frames % ((long long)h->N0 * h->KB))
        return fail(h, PC_ERR_ARG, h->KB > 1 ? "frames must be a positive multiple of buffer_size x step blocks (" +
                                                   std::to_string(h->KB) + ")"
                                             : std::string("frames must be a positive multiple of buffer_size"));
    if (layout != PC_INTERLEAVED && layout != PC_PLANAR) return fail(h, PC_ERR_ARG, "unknown layout");
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    const long long nsteps = frames / h->N0;
    float* target = d_out;
    if (h->relaxed) {
        const size_t need = (size_t)frames * h->n_out;
        if (need > h->rtmp_cap) {
            if (h->d_rtmp) cudaFree(h->d_rtmp);
            h->d_rtmp = nullptr;
            h->rtmp_cap = 0;
            CK(cudaMalloc(&h->d_rtmp, sizeof(float) * need), "relaxed buffer");
            h->rtmp_cap = need;
        }
        target = h->d_rtmp;
    }
    IOView v = make_view(h, d_in, target, frames, layout, h->frame_num);
    int r = run_steps(h, v, nsteps, st);
    if (r) return r;
    if (h->relaxed) {
        const long long os = v.out_sample, oc = v.out_ch;
        relaxed_shift_kernel<<<256, 256, 0, st>>>(d_out, h->d_rtmp, h->d_carry, frames, h->N0, h->n_out, os, oc);
        relaxed_carry_kernel<<<32, 256, 0, st>>>(h->d_carry, h->d_rtmp, frames, h->N0, h->n_out, os, oc);
        CK(cudaGetLastError(), "relaxed shift");
        h->launches += 2;
    }
    return PC_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
// errors of calls that have no handle (thread-local)
static thread_local std::string g_global_err;
const char* pcg_global_error() { return g_global_err.c_str(); }
void pcg_set_global_error(const std::string& m) { g_global_err = m; }


extern "C" {

int pc_check_layout(int M, const int* N, int* P, int ir_len, int relaxed, int* delays, char* msg, int msglen) {
    std::string m;
    if (!N || !P) {
        m = "null layout arrays";
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", m.c_str());
        return PC_ERR_ARG;
    }
    int r = check_layout_impl(M, N, P, ir_len, relaxed != 0, delays, m);
    if (msg && msglen > 0) snprintf(msg, msglen, "%s", m.c_str());
    return r;
}

pc_handle* pc_create(int verbosity) {
    pc_handle* h = new (std::nothrow) pc_handle();
    if (!h) {
        pcg_set_global_error("out of host memory");
        return nullptr;
    }
    h->verbosity = verbosity;
    return h;
}

int pc_setup_layout(pc_handle* h, int fs, int buffer_size, int n_in, int n_out, int num_pcs,
                    const int* num_levels, const int* block_sizes, const int* num_parts, const float* const* irs,
                    const int* ir_lens, const int* in_ch, const int* out_ch, const float* scale, const int* mute) {
    if (!h) return PC_ERR_ARG;
    if (num_pcs < 1 || !num_levels || !block_sizes || !num_parts || !irs || !ir_lens || !in_ch || !out_ch)
        return fail(h, PC_ERR_ARG, "null or empty setup arrays");
    std::vector<PCSpec> specs(num_pcs);
    int off = 0;
    for (int i = 0; i < num_pcs; ++i) {
        const int M = num_levels[i];
        if (M < 1 || M > PC_MAX_LEVELS) return fail(h, PC_ERR_LIMIT, "PC " + std::to_string(i) + ": bad level count");
        specs[i].N.assign(block_sizes + off, block_sizes + off + M);
        specs[i].P.assign(num_parts + off, num_parts + off + M);
        off += M;
        if (ir_lens[i] < 1 || !irs[i]) return fail(h, PC_ERR_ARG, "PC " + std::to_string(i) + ": empty IR");
        specs[i].ir.assign(irs[i], irs[i] + ir_lens[i]);
        specs[i].in_ch = in_ch[i];
        specs[i].out_ch = out_ch[i];
        specs[i].scale = scale ? scale[i] : 1.0f;
        specs[i].mute = mute ? mute[i] : 0;
    }
    return do_setup(h, fs, buffer_size, n_in, n_out, std::move(specs));
}

int pc_setup_config(pc_handle* h, const char* config_file, int max_threads_per_level, int max_level0_threads,
                    double min_work) {
    (void)max_threads_per_level;
    (void)max_level0_threads;
    (void)min_work;
    if (!h) return PC_ERR_ARG;
    if (!config_file) return fail(h, PC_ERR_ARG, "null config path");
    std::ifstream f(config_file);
    if (!f) return fail(h, PC_ERR_CONFIG, std::string("Unable to open config file ") + config_file);
    std::stringstream ss;
    ss << f.rdbuf();
    ConfigFile cfg;
    std::string err;
    if (parse_config(ss.str(), cfg, err)) return fail(h, PC_ERR_CONFIG, err);
    std::string dir(config_file);
    size_t slash = dir.find_last_of('/');
    dir = (slash == std::string::npos) ? std::string(".") : dir.substr(0, slash);
    std::vector<PCSpec> specs;
    for (auto& c : cfg.pcs) {
        PCSpec p;
        p.N = c.N;
        p.P = c.P;
        p.in_ch = c.in_ch;
        p.out_ch = c.out_ch;
        p.scale = c.scale;
        p.mute = c.mute;
        std::string path = c.file;
        std::ifstream probe(path);
        if (!probe && !path.empty() && path[0] != '/') path = dir + "/" + c.file;
        if (read_wav_channel0(path, p.ir, nullptr, err)) return fail(h, PC_ERR_IO, "unable to open file: " + err);
        if (p.ir.empty()) return fail(h, PC_ERR_IO, "empty impulse response: " + path);
        specs.push_back(std::move(p));
    }
    return do_setup(h, cfg.fs, cfg.buffer_size, cfg.n_in, cfg.n_out, std::move(specs));
}

int pc_set_step_blocks(pc_handle* h, int k) {
    if (!h) return PC_ERR_ARG;
    if (h->ready) return fail(h, PC_ERR_STATE, "step blocks must be set before setup");
    if (k < 1 || k > 8 || (k & (k - 1))) return fail(h, PC_ERR_ARG, "step blocks must be 1, 2, 4 or 8");
    h->req_kb = k;
    return PC_OK;
}

int pc_set_tiles(pc_handle* h, int spread_bins, int spread_parts) {
    if (!h) return PC_ERR_ARG;
    if (h->ready) return fail(h, PC_ERR_STATE, "tile shapes must be set before setup");
    if (spread_bins != 0 && !spread_bins_ok(spread_bins))
        return fail(h, PC_ERR_ARG, "bins per spread task must be 64, 128, 256 or 512 (or 0)");
    if (spread_parts < 0 || spread_parts > 64) return fail(h, PC_ERR_ARG, "parts per spread task must be in [1, 64] (or 0)");
    h->req_tile_bins = spread_bins;
    h->req_tile_parts = spread_parts;
    return PC_OK;
}

int pc_set_relaxed(pc_handle* h, int relaxed) {
    if (!h) return PC_ERR_ARG;
    h->relaxed = relaxed ? 1 : 0;
    if (h->ready) return pc_reset(h);
    return PC_OK;
}

int pc_run(pc_handle* h, float* output, const float* input, int frame_count) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return fail(h, PC_ERR_STATE, "run before setup");
    if (!output || !input) return fail(h, PC_ERR_ARG, "null buffer");
    if (frame_count != h->N0)
        return fail(h, PC_ERR_ARG,
                    "frameCount (" + std::to_string(frame_count) + ") != buffer_size (" + std::to_string(h->N0) + ")");
    if (h->KB > 1)
        return fail(h, PC_ERR_STATE, "run() processes one block; this handle computes " + std::to_string(h->KB) +
                                         " blocks per step (use process)");
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t in_b = sizeof(float) * (size_t)h->N0 * h->n_in, out_b = sizeof(float) * (size_t)h->N0 * h->n_out;
    std::memcpy(h->h_in1, input, in_b);
    CK(cudaMemcpyAsync(h->d_in1, h->h_in1, in_b, cudaMemcpyHostToDevice, h->stream), "input copy");
    int r = process_device_impl(h, h->d_out1, h->d_in1, h->N0, PC_INTERLEAVED, h->stream);
    if (r) return r;
    CK(cudaMemcpyAsync(h->h_out1, h->d_out1, out_b, cudaMemcpyDeviceToHost, h->stream), "output copy");
    CK(cudaStreamSynchronize(h->stream), "run sync");
    std::memcpy(output, h->h_out1, out_b);
    return PC_OK;
}

int pc_process(pc_handle* h, float* output, const float* input, long long frames, int layout) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return fail(h, PC_ERR_STATE, "process before setup");
    if (!output || !input || frames <= 0 || frames % ((long long)h->N0 * h->KB))
        return fail(h, PC_ERR_ARG, "frames must be a positive multiple of buffer_size x step blocks");
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t nin = (size_t)frames * h->n_in, nout = (size_t)frames * h->n_out;
    if (nin > h->big_in_cap) {
        if (h->d_big_in) cudaFree(h->d_big_in);
        h->d_big_in = nullptr;
        h->big_in_cap = 0;
        CK(cudaMalloc(&h->d_big_in, sizeof(float) * nin), "input buffer");
        h->big_in_cap = nin;
    }
    if (nout > h->big_out_cap) {
        if (h->d_big_out) cudaFree(h->d_big_out);
        h->d_big_out = nullptr;
        h->big_out_cap = 0;
        CK(cudaMalloc(&h->d_big_out, sizeof(float) * nout), "output buffer");
        h->big_out_cap = nout;
    }
    // Long calls run as a pipeline of chunks: the input copy of chunk i + 1
    // and the output copy of chunk i - 1 (own streams) overlap the steps of
    // chunk i (the handle's stream); the steps of one call stay in order.
    const long long chunk = (long long)std::max(h->G, 128) * h->N0;   // a multiple of KB N0
    if (!h->relaxed && frames >= 2 * chunk) {
        if (!h->cin) CK(cudaStreamCreateWithFlags(&h->cin, cudaStreamNonBlocking), "stream create");
        if (!h->cout) CK(cudaStreamCreateWithFlags(&h->cout, cudaStreamNonBlocking), "stream create");
        const bool planar = layout == PC_PLANAR;
        const long long nch = (frames + chunk - 1) / chunk;
        std::vector<cudaEvent_t> evs;
        auto mkev = [&](cudaEvent_t* e) {
            cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
            if (r == cudaSuccess) evs.push_back(*e);
            return r;
        };
        int rc = PC_OK;
        for (long long i = 0; i < nch && rc == PC_OK; ++i) {
            const long long c0 = i * chunk, n = std::min(chunk, frames - c0);
            cudaEvent_t ein, edone;
            cudaError_t e = mkev(&ein);
            if (e == cudaSuccess) e = mkev(&edone);
            if (e == cudaSuccess)
                e = planar ? cudaMemcpy2DAsync(h->d_big_in + c0, sizeof(float) * frames, input + c0, sizeof(float) * frames,
                                               sizeof(float) * n, h->n_in, cudaMemcpyHostToDevice, h->cin)
                           : cudaMemcpyAsync(h->d_big_in + c0 * h->n_in, input + c0 * h->n_in,
                                             sizeof(float) * n * h->n_in, cudaMemcpyHostToDevice, h->cin);
            if (e == cudaSuccess) e = cudaEventRecord(ein, h->cin);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, ein, 0);
            if (e != cudaSuccess) {
                rc = cuda_fail(h, e, "input copy");
                break;
            }
            const float* din = h->d_big_in + (planar ? c0 : c0 * h->n_in);
            float* dout = h->d_big_out + (planar ? c0 : c0 * h->n_out);
            IOView v = make_view(h, din, dout, n, layout, h->frame_num, frames);
            rc = run_steps(h, v, n / h->N0, h->stream);
            if (rc) break;
            e = cudaEventRecord(edone, h->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->cout, edone, 0);
            if (e == cudaSuccess)
                e = planar ? cudaMemcpy2DAsync(output + c0, sizeof(float) * frames, h->d_big_out + c0, sizeof(float) * frames,
                                               sizeof(float) * n, h->n_out, cudaMemcpyDeviceToHost, h->cout)
                           : cudaMemcpyAsync(output + c0 * h->n_out, h->d_big_out + c0 * h->n_out,
                                             sizeof(float) * n * h->n_out, cudaMemcpyDeviceToHost, h->cout);
            if (e != cudaSuccess) rc = cuda_fail(h, e, "output copy");
        }
        cudaError_t e1 = cudaStreamSynchronize(h->cout);
        cudaError_t e2 = cudaStreamSynchronize(h->stream);
        for (auto ev : evs) cudaEventDestroy(ev);
        if (rc) return rc;
        if (e1 != cudaSuccess) return cuda_fail(h, e1, "process sync");
        if (e2 != cudaSuccess) return cuda_fail(h, e2, "process sync");
        return PC_OK;
    }
    CK(cudaMemcpyAsync(h->d_big_in, input, sizeof(float) * nin, cudaMemcpyHostToDevice, h->stream), "input copy");
    int r = process_device_impl(h, h->d_big_out, h->d_big_in, frames, layout, h->stream);
    if (r) return r;
    CK(cudaMemcpyAsync(output, h->d_big_out, sizeof(float) * nout, cudaMemcpyDeviceToHost, h->stream),
       "output copy");
    CK(cudaStreamSynchronize(h->stream), "process sync");
    return PC_OK;
}

int pc_process_device(pc_handle* h, float* d_output, const float* d_input, long long frames, int layout,
                      void* stream) {
    if (!h) return PC_ERR_ARG;
    return process_device_impl(h, d_output, d_input, frames, layout, (cudaStream_t)stream);
}

int pc_reset(pc_handle* h) {
    if (!h) return PC_ERR_ARG;
    h->frame_num = 0;
    if (!h->ready) return PC_OK;
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    CK(cudaMemsetAsync(h->arena + h->state_off, 0, h->state_bytes, h->stream), "reset");
    CK(cudaStreamSynchronize(h->stream), "reset sync");
    return PC_OK;
}

int pc_cleanup(pc_handle* h) {
    if (!h) return PC_ERR_ARG;
    free_device(h);
    h->specs.clear();
    h->frame_num = 0;
    return PC_OK;
}

void pc_destroy(pc_handle* h) {
    if (!h) return;
    free_device(h);
    delete h;
}

const char* pc_last_error(const pc_handle* h) { return h ? h->err.c_str() : pcg_global_error(); }

int pc_get_info(const pc_handle* h, pc_info* info) {
    if (!h || !info) return PC_ERR_ARG;
    info->fs = h->fs;
    info->buffer_size = h->N0;
    info->num_input_channels = h->n_in;
    info->num_output_channels = h->n_out;
    info->num_pcs = (int)h->specs.size();
    info->max_block_size = h->maxN;
    info->relaxed = h->relaxed;
    info->hyperperiod = h->H;
    info->step_blocks = h->KB;
    info->spread_bins = h->TB;
    info->spread_parts = h->TP;
    info->frame_num = h->frame_num;
    info->device_bytes =
        (long long)h->arena_bytes + (long long)sizeof(float) * (h->big_in_cap + h->big_out_cap + h->rtmp_cap);
    return PC_OK;
}

int pc_get_layout(const pc_handle* h, int pc, int* num_levels, int* block_sizes, int* num_parts) {
    if (!h || pc < 0 || pc >= (int)h->specs.size()) return PC_ERR_ARG;
    const PCSpec& p = h->specs[pc];
    if (num_levels) *num_levels = (int)p.N.size();
    for (size_t L = 0; L < p.N.size(); ++L) {
        if (block_sizes) block_sizes[L] = p.N[L];
        if (num_parts) num_parts[L] = p.P[L];
    }
    return PC_OK;
}

long long pc_kernel_launches(const pc_handle* h) { return h ? h->launches : 0; }

int pc_profile_kernels(pc_handle* h, long long nsteps, pc_kernel_stats* out, int max_kinds, int* n_kinds) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return fail(h, PC_ERR_STATE, "profile before setup");
    if (nsteps < 1 || !out || max_kinds < 1) return fail(h, PC_ERR_ARG, "bad profile arguments");
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    constexpr int kKinds = kClasses + 1;   // + the side spread launches
    static const char* names[kKinds] = {"step_small", "step_mid", "step_large", "step_huge", "spread_side"};
    struct Rec {
        int cls;
        int phase;
        int dgroup;   // -1: the class's per-phase list
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    // every step reads the staging input block and writes the staging output
    IOView v = make_view(h, h->d_in1, h->d_out1, h->N0, PC_INTERLEAVED, 0);
    v.in_step = 0;
    v.out_step = 0;
    RunState rs;
    rs.io = v;
    int rc = PC_OK;
    nsteps = (nsteps + h->KB - 1) / h->KB * h->KB;   // whole steps of KB base blocks
    for (long long s = 0; s < nsteps && rc == PC_OK; s += h->KB) {
        rs.step_base = h->frame_num + s;
        const int ph = phase_of(h, rs.step_base);
        if (h->sp_cnt[ph] > 0) {
            Rec r{kClasses, ph, -1, nullptr, nullptr};
            cudaEventCreate(&r.a);
            cudaEventCreate(&r.b);
            cudaEventRecord(r.a, h->stream);
            cudaError_t e = launch_side_spreads(h->sp_cnt[ph], h->d_tasks + h->sp_off[ph], rs, nullptr, 0, h->stream);
            cudaEventRecord(r.b, h->stream);
            recs.push_back(r);
            h->launches += 1;
            if (e != cudaSuccess) rc = cuda_fail(h, e, "profile launch");
        }
        for (int k = 0; k < kClasses && rc == PC_OK; ++k) {
            const int cls = (h->l0_class + k) % kClasses;
            const int n = h->cnt[cls][ph];
            if (n <= 0) continue;
            Rec r{cls, ph, -1, nullptr, nullptr};
            cudaEventCreate(&r.a);
            cudaEventCreate(&r.b);
            cudaEventRecord(r.a, h->stream);
            cudaError_t e = launch_step_class(cls, n, h->class_maxN[cls], h->bank, h->d_tasks + h->off[cls][ph], rs,
                                              nullptr, 0, h->stream, false);
            cudaEventRecord(r.b, h->stream);
            recs.push_back(r);
            h->launches += 1;
            if (e != cudaSuccess) rc = cuda_fail(h, e, "profile launch");
        }
        for (int gi : h->dg_of_phase[ph]) {
            if (rc != PC_OK) break;
            const pc_handle::DGroup& gr = h->dgroups[gi];
            Rec r{gr.cls, ph, gi, nullptr, nullptr};
            cudaEventCreate(&r.a);
            cudaEventCreate(&r.b);
            cudaEventRecord(r.a, h->stream);
            cudaError_t e = launch_step_class(gr.cls, gr.cnt, h->class_maxN[gr.cls], h->bank, h->d_tasks + gr.off, rs,
                                              nullptr, 0, h->stream, false);
            cudaEventRecord(r.b, h->stream);
            recs.push_back(r);
            h->launches += 1;
            if (e != cudaSuccess) rc = cuda_fail(h, e, "profile launch");
        }
    }
    h->frame_num += nsteps;
    cudaError_t se = cudaStreamSynchronize(h->stream);
    double ms[kKinds] = {0, 0, 0, 0}, bytes[kKinds] = {0, 0, 0, 0};
    long long cnt[kKinds] = {0, 0, 0, 0};
    for (auto& r : recs) {
        float t = 0.f;
        if (se == cudaSuccess && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
            ms[r.cls] += t;
            bytes[r.cls] += r.cls == kClasses ? h->sp_bytes[r.phase]
                                              : (r.dgroup < 0 ? h->alg_bytes[r.cls][r.phase] : h->dgroups[r.dgroup].bytes);
            cnt[r.cls] += 1;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    if (rc) return rc;
    if (se != cudaSuccess) return cuda_fail(h, se, "profile sync");
    int n = 0;
    for (int k = 0; k < kKinds && n < max_kinds; ++k) {
        const int cls = k < kClasses ? (h->l0_class + k) % kClasses : kClasses;
        if (cnt[cls] == 0) continue;
        std::snprintf(out[n].name, sizeof out[n].name, "%s", names[cls]);
        out[n].launches = cnt[cls];
        out[n].total_ms = ms[cls];
        out[n].alg_bytes = bytes[cls];
        ++n;
    }
    if (n_kinds) *n_kinds = n;
    return PC_OK;
}

}  // extern "C"
