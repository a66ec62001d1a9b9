// engine.cu -- host side of the GB300 partitioned-convolution engine and its
// C ABI (include/partconv_gb300.h).
//
// Replaces PartConvMulti (src/partconvMulti.h:52-148,
// src/partconvMulti.cpp:23-1134 of ebattenberg/partconv): per-PC layout
// validation and IR partitioning (src/partconv.cpp:70-230), device-resident
// FDL state, and the per-callback schedule.  The reference's pthread level
// workers become a static per-phase task table: the level schedule repeats
// every H = max_L N_L / N0 base steps, so for each phase the host lists the
// level blocks that fire and the MAC slices that are spread over the steps
// between a level's blocks.  Each base step is one launch per kernel class;
// batches of steps are replayed from a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
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

constexpr int kWlog = 15;          // twiddle table 2^15 entries: real FFTs up to 2 * 16384
constexpr int kGraphSteps = 64;    // base steps per captured graph
constexpr int kMinN0 = 16;

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

    int fs = 0, N0 = 0, n_in = 0, n_out = 0;
    int relaxed = 0;
    std::vector<PCSpec> specs;

    // device arena
    char* arena = nullptr;
    size_t arena_bytes = 0;
    size_t state_off = 0, state_bytes = 0;   // zeroed by reset

    std::vector<DevPC> h_pcs;
    std::vector<DevLevel> h_lv;
    Bank bank{};
    int H = 1;
    int maxN = 0;

    // per-phase tables (device) and launch shapes
    FireTask* d_fire[3] = {nullptr, nullptr, nullptr};
    int* d_fire_off[3] = {nullptr, nullptr, nullptr};
    int fire_grid[3] = {0, 0, 0};
    int fire_maxN[3] = {0, 0, 0};
    SpreadTask* d_spread = nullptr;
    int* d_spread_off = nullptr;
    int spread_grid = 0;
    RunState* d_rs = nullptr;

    // run() staging and Relaxed carry (planar [n_out][N0])
    float* d_in1 = nullptr;
    float* d_out1 = nullptr;
    float* d_carry = nullptr;

    // growable device buffers for pc_process
    float* d_big_in = nullptr;
    float* d_big_out = nullptr;
    size_t big_in_cap = 0, big_out_cap = 0;
    float* d_rtmp = nullptr;
    size_t rtmp_cap = 0;

    cudaGraphExec_t gexec = nullptr;
    int graph_launches_per_replay = 0;

    // algorithmic bytes per phase (profiling)
    std::vector<double> fire_bytes[3];
    std::vector<double> spread_bytes;

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

#define CK(call, where)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, where); \
    } while (0)

void free_device(pc_handle* h) {
    if (h->device >= 0) cudaSetDevice(h->device);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    if (h->arena) cudaFree(h->arena);
    h->arena = nullptr;
    if (h->d_big_in) cudaFree(h->d_big_in);
    if (h->d_big_out) cudaFree(h->d_big_out);
    if (h->d_rtmp) cudaFree(h->d_rtmp);
    h->d_big_in = h->d_big_out = h->d_rtmp = nullptr;
    h->big_in_cap = h->big_out_cap = h->rtmp_cap = 0;
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    h->ready = false;
}

// Launch one base step (every kernel class that has work in some phase).
int launch_step(pc_handle* h, const RunState& rs, const RunState* rs_dev, int s, cudaStream_t st) {
    for (int cls = 0; cls < 3; ++cls) {
        if (h->fire_grid[cls] <= 0) continue;
        CK(launch_fire(cls, h->fire_grid[cls], h->fire_maxN[cls], h->bank, h->d_fire[cls], h->d_fire_off[cls], rs,
                       rs_dev, s, st),
           "fire kernel launch");
    }
    CK(launch_spread(h->spread_grid, h->bank, h->d_spread, h->d_spread_off, rs, rs_dev, s, st), "spread launch");
    return PC_OK;
}

int kernels_per_step(const pc_handle* h) {
    int n = 0;
    for (int cls = 0; cls < 3; ++cls) n += h->fire_grid[cls] > 0;
    return n + (h->spread_grid > 0);
}

int build_graph(pc_handle* h) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    RunState dummy{};
    for (int s = 0; s < kGraphSteps; ++s) {
        int r = launch_step(h, dummy, h->d_rs, s, h->stream);
        if (r) {
            cudaStreamEndCapture(h->stream, &g);
            if (g) cudaGraphDestroy(g);
            return r;
        }
    }
    CK(cudaStreamEndCapture(h->stream, &g), "end capture");
    cudaError_t e = cudaGraphInstantiate(&h->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph instantiate");
    h->graph_launches_per_replay = kGraphSteps * kernels_per_step(h);
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
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream create");
    CK(prepare_kernels(), "kernel attributes");

    h->fs = fs;
    h->N0 = buffer_size;
    h->n_in = n_in;
    h->n_out = n_out;
    h->specs = std::move(specs);
    const int N0 = buffer_size;
    const int npc = (int)h->specs.size();

    // ---- sizes and offsets -------------------------------------------------
    int nlv = 0, maxN = 0, Hh = 1;
    for (auto& p : h->specs) {
        nlv += (int)p.N.size();
        maxN = std::max(maxN, p.N.back());
        Hh = std::max(Hh, p.N.back() / N0);
    }
    h->H = Hh;
    h->maxN = maxN;

    Carve cv;
    // static region
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
    // mixing lists
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

    // task tables
    std::vector<std::vector<FireTask>> fire(3);
    std::vector<std::vector<int>> fire_off(3, std::vector<int>(Hh + 1, 0));
    std::vector<SpreadTask> spread;
    std::vector<int> spread_off(Hh + 1, 0);
    {
        struct LvInfo { int gidx, N, P, T, sb, cs, M, L; };
        std::vector<LvInfo> all;
        int li = 0;
        for (auto& p : h->specs) {
            long s = 0;
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                all.push_back({li, p.N[L], p.P[L], p.N[L] / N0, (int)(s / N0), p.N[L] + 2, (int)p.N.size(), (int)L});
                s += (long)p.N[L] * p.P[L];
            }
        }
        for (int cls = 0; cls < 3; ++cls) h->fire_bytes[cls].assign(Hh, 0.0);
        h->spread_bytes.assign(Hh, 0.0);
        // bytes a fire task must move: spectra rows read/written, the
        // 2N-sample window read and N samples written (level 0 also reads the
        // other levels' due slices and appends N0 samples to the input ring)
        auto fire_bytes = [&](const LvInfo& l) {
            const double C = l.N + 1.0;
            double b = (l.T == 1 ? 8.0 * C * 2.0 * l.P : 24.0 * C) + 12.0 * l.N;
            if (l.L == 0) b += 4.0 * N0 * (l.M - 1) + 4.0 * N0;
            return b;
        };
        std::vector<LvInfo> order = all;
        std::stable_sort(order.begin(), order.end(), [](const LvInfo& a, const LvInfo& b) { return a.N > b.N; });
        for (int g = 0; g < Hh; ++g) {
            for (auto& l : order) {
                if ((g + 1 + l.sb) % l.T == 0) {
                    fire[fire_class_of(l.N)].push_back({l.gidx});
                    h->fire_bytes[fire_class_of(l.N)][g] += fire_bytes(l);
                }
            }
            for (int cls = 0; cls < 3; ++cls) fire_off[cls][g + 1] = (int)fire[cls].size();
            for (auto& l : all) {
                if (l.T < 2 || l.P < 2) continue;
                const int phi = (g + 1 + l.sb) % l.T;
                if (phi == 0) continue;
                const int j = phi - 1, nch = l.T - 1;
                const int lo = (int)(((long)j * l.cs / nch) & ~1L);
                const int hi = (j == nch - 1) ? l.cs : (int)(((long)(j + 1) * l.cs / nch) & ~1L);
                for (int k0 = lo; k0 < hi; k0 += 2 * kSpreadNT)
                    spread.push_back({l.gidx, k0, std::min(hi, k0 + 2 * kSpreadNT)});
                h->spread_bytes[g] += (16.0 * (l.P - 1) + 8.0) * (hi - lo);
            }
            spread_off[g + 1] = (int)spread.size();
        }
    }
    size_t off_fire[3], off_fire_off[3];
    for (int cls = 0; cls < 3; ++cls) {
        off_fire[cls] = cv.take(sizeof(FireTask) * std::max<size_t>(1, fire[cls].size()));
        off_fire_off[cls] = cv.take(sizeof(int) * (Hh + 1));
    }
    const size_t off_spread = cv.take(sizeof(SpreadTask) * std::max<size_t>(1, spread.size()));
    const size_t off_spread_off = cv.take(sizeof(int) * (Hh + 1));
    const size_t off_rs = cv.take(sizeof(RunState));
    const size_t off_in1 = cv.take(sizeof(float) * (size_t)N0 * n_in);
    const size_t off_out1 = cv.take(sizeof(float) * (size_t)N0 * n_out);

    // state region (zeroed by reset)
    const size_t state_begin = cv.take(0);
    std::vector<size_t> off_xring(npc), off_pcout(npc);
    std::vector<int> rin(npc);
    for (int i = 0; i < npc; ++i) {
        long r = 1;
        while (r < 2L * h->specs[i].N.back()) r <<= 1;
        rin[i] = (int)r;
        off_xring[i] = cv.take(sizeof(float) * r);
        off_pcout[i] = cv.take(sizeof(float) * N0);
    }
    std::vector<size_t> off_X(nlv), off_Yp(nlv), off_yr(nlv);
    std::vector<int> rl(nlv);
    {
        int li = 0;
        for (auto& p : h->specs) {
            long s = 0;
            for (size_t L = 0; L < p.N.size(); ++L, ++li) {
                const size_t cs = p.N[L] + 2;
                off_X[li] = cv.take(sizeof(float2) * p.P[L] * cs);
                off_Yp[li] = cv.take(sizeof(float2) * cs);
                long r = p.N[L];
                while (r < s + N0) r <<= 1;
                rl[li] = (int)r;
                off_yr[li] = cv.take(sizeof(float) * r);
                s += (long)p.N[L] * p.P[L];
            }
        }
    }
    const size_t off_mix = cv.take(sizeof(int) * n_out);
    const size_t off_carry = cv.take(sizeof(float) * (size_t)N0 * n_out);
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

    // descriptors
    h->h_pcs.assign(npc, DevPC{});
    h->h_lv.assign(nlv, DevLevel{});
    std::vector<int> zero_owner_count(npc, 0);
    if (!zero_list.empty()) zero_owner_count[0] = (int)zero_list.size();
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
            d.zero_outs = zero_owner_count[i];
            d.zero_off = 0;
            d.scale = p.scale;
            d.rin_mask = rin[i] - 1;
            d.xring = reinterpret_cast<float*>(A + off_xring[i]);
            d.pcout = reinterpret_cast<float*>(A + off_pcout[i]);
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
                l.H = reinterpret_cast<float2*>(A + off_H[li]);
                l.X = reinterpret_cast<float2*>(A + off_X[li]);
                l.Yp = reinterpret_cast<float2*>(A + off_Yp[li]);
                l.yring = reinterpret_cast<float*>(A + off_yr[li]);
                s += (long)p.N[L] * p.P[L];
            }
        }
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
    for (int cls = 0; cls < 3; ++cls) {
        h->d_fire[cls] = reinterpret_cast<FireTask*>(A + off_fire[cls]);
        h->d_fire_off[cls] = reinterpret_cast<int*>(A + off_fire_off[cls]);
        if (!fire[cls].empty())
            CK(cudaMemcpyAsync(h->d_fire[cls], fire[cls].data(), sizeof(FireTask) * fire[cls].size(),
                               cudaMemcpyHostToDevice, h->stream),
               "upload fire tasks");
        CK(cudaMemcpyAsync(h->d_fire_off[cls], fire_off[cls].data(), sizeof(int) * (Hh + 1), cudaMemcpyHostToDevice,
                           h->stream),
           "upload fire offsets");
        int g = 0;
        for (int ph = 0; ph < Hh; ++ph) g = std::max(g, fire_off[cls][ph + 1] - fire_off[cls][ph]);
        h->fire_grid[cls] = g;
        h->fire_maxN[cls] = 0;
    }
    for (auto& p : h->specs)
        for (int n : p.N) {
            int cls = fire_class_of(n);
            h->fire_maxN[cls] = std::max(h->fire_maxN[cls], n);
        }
    h->d_spread = reinterpret_cast<SpreadTask*>(A + off_spread);
    h->d_spread_off = reinterpret_cast<int*>(A + off_spread_off);
    if (!spread.empty())
        CK(cudaMemcpyAsync(h->d_spread, spread.data(), sizeof(SpreadTask) * spread.size(), cudaMemcpyHostToDevice,
                           h->stream),
           "upload spread tasks");
    CK(cudaMemcpyAsync(h->d_spread_off, spread_off.data(), sizeof(int) * (Hh + 1), cudaMemcpyHostToDevice,
                       h->stream),
       "upload spread offsets");
    {
        int g = 0;
        for (int ph = 0; ph < Hh; ++ph) g = std::max(g, spread_off[ph + 1] - spread_off[ph]);
        h->spread_grid = g;
    }
    h->d_rs = reinterpret_cast<RunState*>(A + off_rs);
    h->d_in1 = reinterpret_cast<float*>(A + off_in1);
    h->d_out1 = reinterpret_cast<float*>(A + off_out1);
    h->d_carry = reinterpret_cast<float*>(A + off_carry);

    h->bank.pcs = reinterpret_cast<const DevPC*>(A + off_pcs);
    h->bank.lv = reinterpret_cast<const DevLevel*>(A + off_lv);
    h->bank.W = reinterpret_cast<const float2*>(A + off_W);
    h->bank.wlog = kWlog;
    h->bank.N0 = N0;
    h->bank.H = Hh;
    h->bank.n_out = n_out;
    h->bank.out_off = reinterpret_cast<const int*>(A + off_out_off);
    h->bank.out_pcs = reinterpret_cast<const int*>(A + off_out_pcs);
    h->bank.mix_cnt = reinterpret_cast<int*>(A + off_mix);
    h->bank.zero_list = reinterpret_cast<const int*>(A + off_zero);

    // ---- filter spectra: one CTA per (PC, level, part) row -------------------
    {
        std::vector<float*> d_irs(npc, nullptr);
        std::vector<std::vector<SpectraJob>> jobs(3);
        for (int i = 0; i < npc; ++i) {
            PCSpec& p = h->specs[i];
            e = cudaMalloc(&d_irs[i], sizeof(float) * std::max<size_t>(1, p.ir.size()));
            if (e != cudaSuccess) {
                for (auto q : d_irs)
                    if (q) cudaFree(q);
                free_device(h);
                return fail(h, PC_ERR_NOMEM, "device allocation for the IR failed");
            }
            cudaMemcpyAsync(d_irs[i], p.ir.data(), sizeof(float) * p.ir.size(), cudaMemcpyHostToDevice, h->stream);
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
                    jobs[fire_class_of(l.N)].push_back(jb);
                }
                s += (long)l.N * l.P;
            }
        }
        std::vector<SpectraJob*> d_jobs(3, nullptr);
        int rc = PC_OK;
        for (int cls = 0; cls < 3 && rc == PC_OK; ++cls) {
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
        if (rc) {
            free_device(h);
            return rc;
        }
        if (se != cudaSuccess) {
            free_device(h);
            return cuda_fail(h, se, "filter spectra");
        }
    }

    int r = build_graph(h);
    if (r) {
        free_device(h);
        return r;
    }
    h->frame_num = 0;
    h->ready = true;
    if (h->verbosity > 0) {
        printf("partconv_gb300: %d PCs, N0 = %d, hyperperiod %d steps, %.1f MB device\n", npc, N0, Hh,
               h->arena_bytes / 1e6);
        for (int i = 0; i < npc; ++i) {
            printf("  PC %d: ", i);
            for (size_t L = 0; L < h->specs[i].N.size(); ++L)
                printf("%dx%d%s", h->specs[i].N[L], h->specs[i].P[L], L + 1 < h->specs[i].N.size() ? ", " : "\n");
        }
    }
    return PC_OK;
}

IOView make_view(const pc_handle* h, const float* in, float* out, long long frames, int layout, long long step0) {
    IOView v;
    v.in = in;
    v.out = out;
    v.step0 = step0;
    if (layout == PC_PLANAR) {
        v.in_step = h->N0;
        v.in_sample = 1;
        v.in_ch = frames;
        v.out_step = h->N0;
        v.out_sample = 1;
        v.out_ch = frames;
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

// Run nsteps base steps starting at h->frame_num through the view.
int run_steps(pc_handle* h, const IOView& view, long long nsteps, cudaStream_t st) {
    long long done = 0;
    RunState rs;
    rs.io = view;
    while (nsteps - done >= kGraphSteps && h->gexec) {
        rs.step_base = h->frame_num + done;
        CK(launch_set_state(h->d_rs, rs, st), "state launch");
        CK(cudaGraphLaunch(h->gexec, st), "graph launch");
        h->launches += 1 + h->graph_launches_per_replay;
        done += kGraphSteps;
    }
    for (; done < nsteps; ++done) {
        rs.step_base = h->frame_num + done;
        int r = launch_step(h, rs, nullptr, 0, st);
        if (r) return r;
        h->launches += kernels_per_step(h);
    }
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
    if (!d_out || !d_in || frames <= 0 || frames % h->N0)
        return fail(h, PC_ERR_ARG, "frames must be a positive multiple of buffer_size");
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
static std::string g_create_err;

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
        g_create_err = "out of host memory";
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
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t in_b = sizeof(float) * (size_t)h->N0 * h->n_in, out_b = sizeof(float) * (size_t)h->N0 * h->n_out;
    CK(cudaMemcpyAsync(h->d_in1, input, in_b, cudaMemcpyHostToDevice, h->stream), "input copy");
    int r = process_device_impl(h, h->d_out1, h->d_in1, h->N0, PC_INTERLEAVED, h->stream);
    if (r) return r;
    CK(cudaMemcpyAsync(output, h->d_out1, out_b, cudaMemcpyDeviceToHost, h->stream), "output copy");
    CK(cudaStreamSynchronize(h->stream), "run sync");
    return PC_OK;
}

int pc_process(pc_handle* h, float* output, const float* input, long long frames, int layout) {
    if (!h) return PC_ERR_ARG;
    if (!h->ready) return fail(h, PC_ERR_STATE, "process before setup");
    if (!output || !input || frames <= 0 || frames % h->N0)
        return fail(h, PC_ERR_ARG, "frames must be a positive multiple of buffer_size");
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
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    return process_device_impl(h, d_output, d_input, frames, layout, st);
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

const char* pc_last_error(const pc_handle* h) { return h ? h->err.c_str() : g_create_err.c_str(); }

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
    info->frame_num = h->frame_num;
    info->device_bytes = (long long)h->arena_bytes + (long long)sizeof(float) * (h->big_in_cap + h->big_out_cap + h->rtmp_cap);
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
    static const char* names[4] = {"fire_small", "fire_mid", "fire_large", "spread_mac"};
    struct Rec { int kind; int phase; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    // every step reads the staging input block and writes the staging output
    IOView v = make_view(h, h->d_in1, h->d_out1, h->N0, PC_INTERLEAVED, 0);
    v.in_step = 0;
    v.out_step = 0;
    RunState rs;
    rs.io = v;
    int rc = PC_OK;
    for (long long s = 0; s < nsteps && rc == PC_OK; ++s) {
        rs.step_base = h->frame_num + s;
        const int phase = (int)(rs.step_base & (h->H - 1));
        for (int kind = 0; kind < 4 && rc == PC_OK; ++kind) {
            const int grid = kind < 3 ? h->fire_grid[kind] : h->spread_grid;
            if (grid <= 0) continue;
            Rec r{kind, phase, nullptr, nullptr};
            cudaEventCreate(&r.a);
            cudaEventCreate(&r.b);
            cudaEventRecord(r.a, h->stream);
            cudaError_t e = kind < 3 ? launch_fire(kind, grid, h->fire_maxN[kind], h->bank, h->d_fire[kind],
                                                   h->d_fire_off[kind], rs, nullptr, 0, h->stream)
                                     : launch_spread(grid, h->bank, h->d_spread, h->d_spread_off, rs, nullptr, 0,
                                                     h->stream);
            cudaEventRecord(r.b, h->stream);
            recs.push_back(r);
            h->launches += 1;
            if (e != cudaSuccess) rc = cuda_fail(h, e, "profile launch");
        }
    }
    h->frame_num += nsteps;
    cudaError_t se = cudaStreamSynchronize(h->stream);
    double ms[4] = {0, 0, 0, 0}, bytes[4] = {0, 0, 0, 0};
    long long cnt[4] = {0, 0, 0, 0};
    for (auto& r : recs) {
        float t = 0.f;
        const double b = r.kind < 3 ? h->fire_bytes[r.kind][r.phase] : h->spread_bytes[r.phase];
        if (se == cudaSuccess && b > 0 && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
            ms[r.kind] += t;
            bytes[r.kind] += b;
            cnt[r.kind] += 1;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    if (rc) return rc;
    if (se != cudaSuccess) return cuda_fail(h, se, "profile sync");
    int n = 0;
    for (int kind = 0; kind < 4 && n < max_kinds; ++kind) {
        if (cnt[kind] == 0) continue;
        std::snprintf(out[n].name, sizeof out[n].name, "%s", names[kind]);
        out[n].launches = cnt[kind];
        out[n].total_ms = ms[kind];
        out[n].alg_bytes = bytes[kind];
        ++n;
    }
    if (n_kinds) *n_kinds = n;
    return PC_OK;
}

}  // extern "C"
