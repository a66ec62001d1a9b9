// serve.cu -- serving pool: partitioned convolvers (one per stream channel)
// that join and leave between base steps without rebuilding anything.
//
// No reference counterpart: the reference sets up a fixed PartConvMulti from
// a config file (src/partconvMulti.cpp:23-718).  A pool holds PCs of one base
// block size N0 in one device arena sized by an HBM budget.  Admission
// carves the PC's spectra and FDL state from the arena (refused with
// PC_ERR_NOMEM when the budget is spent), computes its filter spectra, and
// writes one descriptor per level whose schedule origin is the pool's next
// step; the CTA map that the pool kernel walks is rebuilt on the host.
// Release marks the descriptors inactive and returns the arena space.  All
// of this is ordered on the pool's stream, so it never races a step.
// Every step batches all active PCs: one launch per block-size class.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/partconv_gb300.h"
#include "engine_types.h"
#include "kernels.h"

using namespace pcg;

namespace {

constexpr int kWlog = 15;
constexpr int kPoolMaxLevels = kEmitLevels + 1;
constexpr size_t kAlign = 256;

// first-fit free list over [0, cap)
struct FreeList {
    std::map<size_t, size_t> free_;   // offset -> size
    size_t used = 0;
    void init(size_t cap) {
        free_.clear();
        free_[0] = cap;
        used = 0;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + kAlign - 1) & ~(kAlign - 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, o = it->first + bytes;
                free_.erase(it);
                if (rest) free_[o] = rest;
                used += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + kAlign - 1) & ~(kAlign - 1);
        used -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct PoolPC {
    bool live = false;
    // admitted, spectra still being built on the admission stream: becomes
    // live in pcs_poll once `ev` has completed
    bool pending = false;
    cudaEvent_t ev = nullptr;
    size_t toff = 0, tbytes = 0;  // IR and job scratch of the admission
    std::vector<Task> recs;       // descriptors to publish
    int M = 0;
    std::vector<int> N, P;
    size_t off = 0, bytes = 0;   // arena block
    std::vector<PoolCta> fires;  // map entries (class by level)
    int spread_tiles[kPoolMaxLevels] = {0};
};

}  // namespace

struct pcs_handle {
    std::string err;
    int device = -1;
    cudaStream_t stream = nullptr;
    int N0 = 0, max_pcs = 0;
    size_t budget = 0;
    char* arena = nullptr;
    FreeList fl;
    float2* d_W = nullptr;
    Task* d_slots = nullptr;                 // max_pcs * kPoolMaxLevels descriptors
    std::vector<Task> h_slots;
    PoolCta* d_map[3] = {nullptr, nullptr, nullptr};
    size_t map_cap = 0;
    int map_n[3] = {0, 0, 0};
    bool map_dirty = false;
    float* d_in = nullptr;                   // [max_pcs][N0] staging
    float* d_out = nullptr;
    Bank bank{};
    long long step = 0;
    int class_maxN[3] = {0, 0, 0};
    std::vector<PoolPC> pcs;
    int live = 0;
    std::vector<int> pending;   // ids of admitted PCs not yet live
    long long launches = 0;
    cudaEvent_t done = nullptr;
    std::vector<void*> allocs;
    // Admission builds a PC's spectra on its own stream, so it never waits
    // for the pool's steps; a released PC's space may still be read by
    // enqueued steps, so it returns to the budget only once an event
    // recorded after them has completed.
    cudaStream_t astream = nullptr;
    struct PendingTmp {
        cudaEvent_t ev;
        size_t off, bytes;
    };
    std::vector<PendingTmp> tmp;
};

namespace {

int sfail(pcs_handle* h, int code, const std::string& m) {
    h->err = m;
    return code;
}

#define SCK(call, where)                                                                                   \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return sfail(h, PC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// return released space whose last users have run (all of it when wait)
void reap_tmp(pcs_handle* h, bool wait) {
    for (size_t i = 0; i < h->tmp.size();) {
        auto& t = h->tmp[i];
        if (wait) cudaEventSynchronize(t.ev);
        if (cudaEventQuery(t.ev) == cudaSuccess) {
            h->fl.release(t.off, t.bytes);
            cudaEventDestroy(t.ev);
            h->tmp.erase(h->tmp.begin() + i);
        } else {
            ++i;
        }
    }
}

template <class T>
cudaError_t smalloc(pcs_handle* h, T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
    if (e == cudaSuccess) {
        h->allocs.push_back(*p);
        e = cudaMemsetAsync(*p, 0, sizeof(T) * std::max<size_t>(n, 1), h->stream);
    }
    return e;
}

// bytes a PC of this layout needs in the arena (spectra, rings, partial sums)
size_t pc_bytes(int N0, const std::vector<int>& N, const std::vector<int>& P, size_t* xr_bytes) {
    size_t b = 0;
    long r = 1;
    while (r < 2L * N.back()) r <<= 1;
    *xr_bytes = sizeof(float) * r;
    b += (*xr_bytes + kAlign - 1) & ~(kAlign - 1);
    long s = 0;
    for (size_t L = 0; L < N.size(); ++L) {
        const size_t cs = N[L] + 2;
        b += 2 * ((sizeof(float2) * P[L] * cs + kAlign - 1) & ~(kAlign - 1));   // H, X
        b += (sizeof(float2) * 2 * cs + kAlign - 1) & ~(kAlign - 1);            // Yp
        long R = N[L];
        while (R < s + N0) R <<= 1;
        b += (sizeof(float) * R + kAlign - 1) & ~(kAlign - 1);                  // yring
        s += (long)N[L] * P[L];
    }
    return b;
}

int rebuild_map(pcs_handle* h) {
    std::vector<PoolCta> m[3];
    for (int id = 0; id < (int)h->pcs.size(); ++id) {
        const PoolPC& p = h->pcs[id];
        if (!p.live) continue;
        for (int L = 0; L < p.M; ++L) {
            const int slot = id * kPoolMaxLevels + L;
            m[fire_class_of(p.N[L])].push_back({slot, 0});
            for (int t = 1; t <= p.spread_tiles[L]; ++t) m[fire_class_of(h->N0)].push_back({slot, t});
        }
    }
    size_t need = std::max({m[0].size(), m[1].size(), m[2].size(), (size_t)1});
    if (need > h->map_cap) {
        // steps already enqueued may still read the old maps
        SCK(cudaStreamSynchronize(h->stream), "map sync");
        for (auto& d : h->d_map) {
            if (d) cudaFree(d);
            d = nullptr;
        }
        size_t cap = std::max(need * 2, (size_t)1024);
        for (auto& d : h->d_map) SCK(cudaMalloc(&d, sizeof(PoolCta) * cap), "map alloc");
        h->map_cap = cap;
    }
    for (int c = 0; c < 3; ++c) {
        h->map_n[c] = (int)m[c].size();
        if (!m[c].empty())
            SCK(cudaMemcpyAsync(h->d_map[c], m[c].data(), sizeof(PoolCta) * m[c].size(), cudaMemcpyHostToDevice,
                                h->stream),
                "map upload");
    }
    // the host vectors die here: pageable copies are staged before returning
    h->map_dirty = false;
    return PC_OK;
}

}  // namespace

extern "C" {

pcs_handle* pcs_create(int buffer_size, long long hbm_budget_bytes, int max_pcs) {
    if (buffer_size < 16 || (buffer_size & (buffer_size - 1)) || buffer_size > 1024 || max_pcs < 1 ||
        hbm_budget_bytes < (1 << 20))
        return nullptr;
    pcs_handle* h = new (std::nothrow) pcs_handle();
    if (!h) return nullptr;
    h->N0 = buffer_size;
    h->max_pcs = max_pcs;
    h->budget = (size_t)hbm_budget_bytes;
    auto bad = [&]() {
        pcs_destroy(h);
        return (pcs_handle*)nullptr;
    };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bad();
    // steps run at the device's highest priority, admission work at its lowest
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return bad();
    if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, greatest) != cudaSuccess) return bad();
    if (cudaStreamCreateWithPriority(&h->astream, cudaStreamNonBlocking, least) != cudaSuccess) return bad();
    if (prepare_kernels() != cudaSuccess) return bad();
    if (cudaMalloc(&h->arena, h->budget) != cudaSuccess) {
        h->arena = nullptr;
        return bad();
    }
    h->fl.init(h->budget);
    std::vector<float2> W((size_t)1 << kWlog);
    for (size_t m = 0; m < W.size(); ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)W.size();
        W[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    if (smalloc(h, &h->d_W, W.size()) != cudaSuccess) return bad();
    if (cudaMemcpyAsync(h->d_W, W.data(), sizeof(float2) * W.size(), cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
        return bad();
    if (smalloc(h, &h->d_slots, (size_t)max_pcs * kPoolMaxLevels) != cudaSuccess) return bad();
    h->h_slots.assign((size_t)max_pcs * kPoolMaxLevels, Task{});
    if (smalloc(h, &h->d_in, (size_t)max_pcs * buffer_size) != cudaSuccess) return bad();
    if (smalloc(h, &h->d_out, (size_t)max_pcs * buffer_size) != cudaSuccess) return bad();
    h->pcs.assign(max_pcs, PoolPC{});
    if (cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming) != cudaSuccess) return bad();
    h->bank.W = h->d_W;
    h->bank.wlog = kWlog;
    h->bank.N0 = buffer_size;
    h->bank.n_out = max_pcs;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bad();
    return h;
}

// Admit one PC (one stream channel) without waiting: its state is cleared
// and its spectra built on the admission stream; pcs_poll makes it live once
// that work has completed.  Returns its id (also its I/O channel) in *pc_id.
// PC_ERR_NOMEM when the pool's HBM budget cannot hold it now.
int pcs_admit_async(pcs_handle* h, const float* ir, int ir_len, int M, const int* N, int* P, int* pc_id) {
    if (!h) return PC_ERR_ARG;
    if (!ir || ir_len < 1 || !N || !P || !pc_id) return sfail(h, PC_ERR_ARG, "bad admission arguments");
    if (M > kPoolMaxLevels) return sfail(h, PC_ERR_LIMIT, "at most 5 levels per pooled PC");
    if (N[0] != h->N0) return sfail(h, PC_ERR_LAYOUT, "first block size must equal the pool's block size");
    std::vector<int> Nv(N, N + M), Pv(P, P + M);
    char msg[256];
    int r = pc_check_layout(M, Nv.data(), Pv.data(), ir_len, 1, nullptr, msg, sizeof msg);
    if (r) return sfail(h, r, msg);
    if (Nv[M - 1] > kMaxBlockOneCta)
        return sfail(h, PC_ERR_LIMIT, "serving levels are limited to blocks of 16384 (larger blocks: pc_* engine)");
    for (int i = 0; i < M; ++i) P[i] = Pv[i];
    int id = -1;
    for (int i = 0; i < h->max_pcs; ++i)
        if (!h->pcs[i].live && !h->pcs[i].pending) {
            id = i;
            break;
        }
    if (id < 0) return sfail(h, PC_ERR_LIMIT, "pool is full (max_pcs)");
    size_t xr_bytes = 0;
    const size_t need = pc_bytes(h->N0, Nv, Pv, &xr_bytes);
    const size_t ir_bytes = ((sizeof(float) * ir_len + kAlign - 1) & ~(kAlign - 1));
    size_t jobs_n = 0;
    for (int L = 0; L < M; ++L) jobs_n += Pv[L];
    const size_t job_bytes = ((sizeof(SpectraJob) * jobs_n + kAlign - 1) & ~(kAlign - 1));
    size_t off = 0, toff = 0;
    reap_tmp(h, false);
    auto alloc = [&](size_t bytes, size_t* o) {
        if (h->fl.alloc(bytes, o)) return true;
        if (h->tmp.empty()) return false;
        reap_tmp(h, true);   // space of released PCs, once the steps that used it have run
        return h->fl.alloc(bytes, o);
    };
    if (!alloc(need, &off)) return sfail(h, PC_ERR_NOMEM, "HBM budget of the pool is exhausted");
    if (!alloc(ir_bytes + job_bytes, &toff)) {
        h->fl.release(off, need);
        return sfail(h, PC_ERR_NOMEM, "HBM budget of the pool is exhausted");
    }
    char* A = h->arena + off;
    SCK(cudaSetDevice(h->device), "cudaSetDevice");
    // the space is free of enqueued steps (released space waits in tmp), so
    // the admission stream may write it at once
    SCK(cudaMemsetAsync(A, 0, need, h->astream), "clear PC state");
    float* d_ir = reinterpret_cast<float*>(h->arena + toff);
    SpectraJob* d_jobs = reinterpret_cast<SpectraJob*>(h->arena + toff + ir_bytes);
    SCK(cudaMemcpyAsync(d_ir, ir, sizeof(float) * ir_len, cudaMemcpyHostToDevice, h->astream), "IR upload");

    PoolPC& pc = h->pcs[id];
    pc = PoolPC{};
    pc.M = M;
    pc.N = Nv;
    pc.P = Pv;
    pc.off = off;
    pc.bytes = need;
    size_t o = (xr_bytes + kAlign - 1) & ~(kAlign - 1);
    float* xring = reinterpret_cast<float*>(A);
    long s = 0;
    std::vector<SpectraJob> jobs[3];
    std::vector<float*> yrings(M);
    std::vector<int> rmasks(M);
    std::vector<Task> recs(M);
    for (int L = 0; L < M; ++L) {
        const int n = Nv[L], cs = n + 2;
        float2* H = reinterpret_cast<float2*>(A + o);
        o += (sizeof(float2) * Pv[L] * cs + kAlign - 1) & ~(kAlign - 1);
        float2* X = reinterpret_cast<float2*>(A + o);
        o += (sizeof(float2) * Pv[L] * cs + kAlign - 1) & ~(kAlign - 1);
        float2* Yp = reinterpret_cast<float2*>(A + o);
        o += (sizeof(float2) * 2 * cs + kAlign - 1) & ~(kAlign - 1);
        long R = n;
        while (R < s + h->N0) R <<= 1;
        float* yr = reinterpret_cast<float*>(A + o);
        o += (sizeof(float) * R + kAlign - 1) & ~(kAlign - 1);
        yrings[L] = yr;
        rmasks[L] = (int)R - 1;
        const int logN = (int)std::lround(std::log2((double)n));
        for (int q = 0; q < Pv[L]; ++q) {
            const long start = s + (long)q * n;
            SpectraJob jb;
            jb.src = d_ir + std::min<long>(start, ir_len);
            jb.len = (int)std::max<long>(0, std::min<long>(n, (long)ir_len - start));
            jb.N = n;
            jb.logN = logN;
            jb.dst = H + (size_t)q * cs;
            jobs[fire_class_of(n)].push_back(jb);
        }
        Task t{};
        t.kind = 0;
        t.N = n;
        t.logN = logN;
        t.P = Pv[L];
        t.T = n / h->N0;
        t.s_blocks = (int)(s / h->N0);
        t.cs = cs;
        t.rmask = (int)R - 1;
        t.M = M;
        t.in_ch = id;
        t.out_ch = id;
        t.mix_mode = 1;
        t.rin_mask = (int)(xr_bytes / sizeof(float)) - 1;
        t.lv_index = 0;
        t.active = 1;
        t.scale = 1.0f;
        t.origin = 0;   // set when the PC goes live
        t.H = H;
        t.X = X;
        t.Yp = Yp;
        t.yring = yr;
        t.xring = xring;
        recs[L] = t;
        // spread tiles per step: level 0 every bin, others their widest slice
        int bins;
        if (t.T == 1) bins = Pv[L] >= 3 ? cs : 0;
        else bins = Pv[L] >= 2 ? (cs + t.T - 2) / (t.T - 1) + 2 : 0;
        pc.spread_tiles[L] = (bins + 2 * 64 - 1) / (2 * 64);
        s += (long)n * Pv[L];
    }
    for (int L = 1; L <= kEmitLevels && L < M; ++L) {
        recs[0].eyring[L - 1] = yrings[L];
        recs[0].emask[L - 1] = rmasks[L];
    }
    size_t jo = 0;
    for (int c = 0; c < 3; ++c) {
        if (jobs[c].empty()) continue;
        int mN = 0;
        for (auto& j : jobs[c]) mN = std::max(mN, j.N);
        SCK(cudaMemcpyAsync(d_jobs + jo, jobs[c].data(), sizeof(SpectraJob) * jobs[c].size(), cudaMemcpyHostToDevice,
                            h->astream),
            "job upload");
        SCK(launch_spectra(c, (int)jobs[c].size(), mN, d_jobs + jo, h->d_W, kWlog, h->astream), "PC spectra");
        h->launches++;
        jo += jobs[c].size();
    }
    // the PC's state and spectra must be ready before its descriptors reach
    // the pool's stream: the admission work is marked by an event
    SCK(cudaEventCreateWithFlags(&pc.ev, cudaEventDisableTiming), "event");
    SCK(cudaEventRecord(pc.ev, h->astream), "event record");
    pc.toff = toff;
    pc.tbytes = ir_bytes + job_bytes;
    pc.recs = std::move(recs);
    pc.pending = true;
    h->pending.push_back(id);
    *pc_id = id;
    return PC_OK;
}

// Publish every pending PC whose admission work has completed (all of them
// when wait): descriptors to the pool's stream, time origin = the next step.
static int pcs_poll_impl(pcs_handle* h, bool wait, int* n_published) {
    int n = 0;
    for (size_t j = 0; j < h->pending.size();) {
        const int id = h->pending[j];
        PoolPC& pc = h->pcs[id];
        if (wait) SCK(cudaEventSynchronize(pc.ev), "admission sync");
        const cudaError_t q = cudaEventQuery(pc.ev);
        if (q == cudaErrorNotReady) {
            ++j;
            continue;
        }
        if (q != cudaSuccess) return sfail(h, PC_ERR_CUDA, std::string("admission: ") + cudaGetErrorString(q));
        cudaEventDestroy(pc.ev);
        pc.ev = nullptr;
        h->fl.release(pc.toff, pc.tbytes);
        for (auto& t : pc.recs) t.origin = h->step;
        for (int L = 0; L < pc.M; ++L) {
            h->h_slots[(size_t)id * kPoolMaxLevels + L] = pc.recs[L];
            const int cls = fire_class_of(pc.N[L]);
            h->class_maxN[cls] = std::max(h->class_maxN[cls], pc.N[L]);
        }
        h->class_maxN[fire_class_of(h->N0)] = std::max(h->class_maxN[fire_class_of(h->N0)], h->N0);
        SCK(cudaMemcpyAsync(h->d_slots + (size_t)id * kPoolMaxLevels, pc.recs.data(), sizeof(Task) * pc.M,
                            cudaMemcpyHostToDevice, h->stream),
            "descriptor upload");
        // pageable source: staged before the call returns, so pc.recs may change later
        pc.pending = false;
        pc.live = true;
        h->live++;
        ++n;
        h->pending.erase(h->pending.begin() + j);
    }
    if (n_published) *n_published = n;
    return n ? rebuild_map(h) : PC_OK;
}

// Admit one PC and make it live before returning (its schedule starts at
// the pool's next step).
int pcs_admit(pcs_handle* h, const float* ir, int ir_len, int M, const int* N, int* P, int* pc_id) {
    int r = pcs_admit_async(h, ir, ir_len, M, N, P, pc_id);
    if (r) return r;
    return pcs_poll_impl(h, true, nullptr);
}

int pcs_poll(pcs_handle* h, int* n_published) {
    if (!h) return PC_ERR_ARG;
    if (h->pending.empty()) {
        if (n_published) *n_published = 0;
        return PC_OK;
    }
    SCK(cudaSetDevice(h->device), "cudaSetDevice");
    return pcs_poll_impl(h, false, n_published);
}

int pcs_is_live(const pcs_handle* h, int pc_id) {
    if (!h || pc_id < 0 || pc_id >= h->max_pcs) return 0;
    return h->pcs[pc_id].live ? 1 : 0;
}

int pcs_release(pcs_handle* h, int pc_id) {
    if (!h || pc_id < 0 || pc_id >= h->max_pcs || !(h->pcs[pc_id].live || h->pcs[pc_id].pending))
        return h ? sfail(h, PC_ERR_ARG, "no such PC") : PC_ERR_ARG;
    PoolPC& pc = h->pcs[pc_id];
    if (pc.pending) {   // never stepped: its space is free once the admission work has run
        SCK(cudaEventSynchronize(pc.ev), "admission sync");
        cudaEventDestroy(pc.ev);
        pc.ev = nullptr;
        h->fl.release(pc.toff, pc.tbytes);
        h->fl.release(pc.off, pc.bytes);
        pc.pending = false;
        h->pending.erase(std::find(h->pending.begin(), h->pending.end(), pc_id));
        return PC_OK;
    }
    std::vector<Task> recs(pc.M, Task{});   // inactive descriptors
    SCK(cudaMemcpyAsync(h->d_slots + (size_t)pc_id * kPoolMaxLevels, recs.data(), sizeof(Task) * pc.M,
                        cudaMemcpyHostToDevice, h->stream),
        "descriptor clear");
    // steps already enqueued may still use the space: it returns to the
    // budget once they have run
    {
        cudaEvent_t ev;
        SCK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        SCK(cudaEventRecord(ev, h->stream), "event record");
        h->tmp.push_back({ev, pc.off, pc.bytes});
    }
    pc.live = false;
    h->live--;
    return rebuild_map(h);
}

// One base step for every active PC: input [max_pcs][N0] host (pinned for
// asynchrony), output likewise; returns after enqueueing.  Channels of
// inactive PCs are copied but produce zeros.
int pcs_step(pcs_handle* h, const float* in, float* out, int n_channels) {
    if (!h || !in || !out) return PC_ERR_ARG;
    if (!h->tmp.empty()) reap_tmp(h, false);
    if (n_channels < 0 || n_channels > h->max_pcs) return sfail(h, PC_ERR_ARG, "bad channel count");
    SCK(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t nb = sizeof(float) * (size_t)n_channels * h->N0;
    if (nb) SCK(cudaMemcpyAsync(h->d_in, in, nb, cudaMemcpyHostToDevice, h->stream), "input copy");
    RunState rs{};
    rs.step_base = h->step;
    rs.io.in = h->d_in;
    rs.io.out = h->d_out;
    rs.io.step0 = h->step;
    rs.io.in_step = 0;
    rs.io.in_sample = 1;
    rs.io.in_ch = h->N0;
    rs.io.out_step = 0;
    rs.io.out_sample = 1;
    rs.io.out_ch = h->N0;
    const int c0 = fire_class_of(h->N0);
    for (int k = 0; k < 3; ++k) {
        const int cls = (c0 + k) % 3;
        if (h->map_n[cls] <= 0) continue;
        SCK(launch_pool_class(cls, h->map_n[cls], std::max(h->class_maxN[cls], 16), h->bank, h->d_slots, h->d_map[cls],
                              rs, h->stream),
            "pool step");
        h->launches++;
    }
    if (nb) SCK(cudaMemcpyAsync(out, h->d_out, nb, cudaMemcpyDeviceToHost, h->stream), "output copy");
    SCK(cudaEventRecord(h->done, h->stream), "event");
    h->step++;
    return PC_OK;
}

// 1 when the last pcs_step has completed, 0 while it runs
int pcs_query(pcs_handle* h) {
    if (!h) return PC_ERR_ARG;
    return cudaEventQuery(h->done) == cudaSuccess ? 1 : 0;
}

int pcs_sync(pcs_handle* h) {
    if (!h) return PC_ERR_ARG;
    SCK(cudaStreamSynchronize(h->stream), "pool sync");
    return PC_OK;
}

long long pcs_bytes_in_use(const pcs_handle* h) { return h ? (long long)h->fl.used : 0; }
int pcs_live(const pcs_handle* h) { return h ? h->live : 0; }
long long pcs_kernel_launches(const pcs_handle* h) { return h ? h->launches : 0; }
const char* pcs_last_error(const pcs_handle* h) { return h ? h->err.c_str() : ""; }

void pcs_destroy(pcs_handle* h) {
    if (!h) return;
    if (h->device >= 0) cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->astream) cudaStreamSynchronize(h->astream);
    for (auto& pc : h->pcs)
        if (pc.ev) cudaEventDestroy(pc.ev);
    for (auto& t : h->tmp) cudaEventDestroy(t.ev);
    h->tmp.clear();
    for (void* p : h->allocs) cudaFree(p);
    for (auto d : h->d_map)
        if (d) cudaFree(d);
    if (h->arena) cudaFree(h->arena);
    if (h->done) cudaEventDestroy(h->done);
    if (h->astream) cudaStreamDestroy(h->astream);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

}  // extern "C"
