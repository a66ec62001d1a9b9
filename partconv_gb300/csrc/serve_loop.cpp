// serve_loop.cpp -- the real-time serving loop over pools of pcs_* handles,
// in native code.
//
// The reference runs one fixed PartConvMulti from an audio callback loop
// (src/pcRTMulti.cpp:138-185, :303-365) and counts the callbacks that missed
// their deadline.  Here many streams of different base block sizes arrive
// and leave while the pools run: one pool per block size, each stepping all
// of its live channels once per block period on a monotonic clock.  A host
// thread (the caller's; no Python lock held) admits arriving requests in
// arrival order as HBM budget allows (pcs_admit_async: the spectra build on
// the pool's admission stream while the pools keep stepping), makes them live
// when their spectra are ready (pcs_poll), gathers each pool's per-tick input
// from every live channel, launches the pool's step (pcs_step, pinned
// buffers) and, when it completes (pcs_query), records the step's latency
// from its release and whether it ended after the next release (a missed
// deadline), and releases requests whose audio is done.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <random>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/partconv_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Chan {
    int pid;          // channel id in its pool
    long long off;    // input offset in the noise buffer
    long long pos;    // next block
    long long left;   // blocks still to feed
    int req;
};

struct Sample {
    double lat_us;
    double weight;   // channels stepped
};

// latency at quantile q, each step weighted by the channels it carried
double weighted_pct(std::vector<Sample> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end(), [](const Sample& a, const Sample& b) { return a.lat_us < b.lat_us; });
    double tot = 0.0;
    for (auto& s : v) tot += s.weight;
    double acc = 0.0;
    for (auto& s : v) {
        acc += s.weight;
        if (acc / tot >= q) return s.lat_us;
    }
    return v.back().lat_us;
}

}  // namespace

extern "C" int pcs_run_load(pcs_handle* const* pools, const int* pool_block, int n_pools, int n_req,
                            const double* arrival, const int* pool_of, const int* channels, const long long* frames,
                            const float* const* irs, const int* ir_len, const int* num_levels, const int* N_flat,
                            const int* P_flat, const float* noise, long long noise_len, unsigned long long seed,
                            int max_concurrent, double max_seconds, double fs, pcs_load_stats* stats) {
    if (!pools || !pool_block || n_pools < 1 || n_pools > PCS_LOAD_MAX_POOLS || n_req < 0 || !stats || !noise ||
        fs <= 0)
        return PC_ERR_ARG;
    for (int i = 0; i < n_req; ++i)
        if (pool_of[i] < 0 || pool_of[i] >= n_pools || channels[i] < 1 || frames[i] <= 0 ||
            frames[i] % pool_block[pool_of[i]] || frames[i] > noise_len)
            return PC_ERR_ARG;
    std::memset(stats, 0, sizeof *stats);

    // pinned per-pool input/output blocks, one row of block samples per channel id
    int max_ch = 0;
    for (int i = 0; i < n_req; ++i) max_ch = std::max(max_ch, channels[i]);
    std::vector<float*> hin(n_pools, nullptr), hout(n_pools, nullptr);
    std::vector<int> cap(n_pools, 0);
    auto free_all = [&]() {
        for (int b = 0; b < n_pools; ++b) {
            if (hin[b]) cudaFreeHost(hin[b]);
            if (hout[b]) cudaFreeHost(hout[b]);
        }
    };
    auto ensure = [&](int b, int nch) -> bool {   // room for channel ids < nch
        if (nch <= cap[b]) return true;
        int c = std::max(nch, std::max(64, 2 * cap[b]));
        float *a = nullptr, *o = nullptr;
        const size_t bytes = sizeof(float) * (size_t)c * pool_block[b];
        if (cudaHostAlloc(reinterpret_cast<void**>(&a), bytes, cudaHostAllocDefault) != cudaSuccess) return false;
        if (cudaHostAlloc(reinterpret_cast<void**>(&o), bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaFreeHost(a);
            return false;
        }
        if (hin[b]) {   // no step of this pool is in flight when it grows (checked by the caller)
            std::memcpy(a, hin[b], sizeof(float) * (size_t)cap[b] * pool_block[b]);
            cudaFreeHost(hin[b]);
            cudaFreeHost(hout[b]);
        }
        hin[b] = a;
        hout[b] = o;
        cap[b] = c;
        return true;
    };

    std::vector<int> order(n_req);
    for (int i = 0; i < n_req; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return arrival[a] < arrival[b]; });
    std::vector<long long> ch0(n_req + 1, 0), lv0(n_req + 1, 0);
    for (int i = 0; i < n_req; ++i) {
        ch0[i + 1] = ch0[i] + channels[i];
        lv0[i + 1] = lv0[i] + num_levels[i];
    }
    std::mt19937_64 rng(seed);

    std::deque<int> pend(order.begin(), order.end()), queue;
    struct Waiting {
        int req;
        std::vector<int> pids;
    };
    std::vector<Waiting> waiting;
    std::vector<std::vector<int>> pcs_of(n_req);
    std::vector<std::vector<Chan>> live(n_pools);
    std::vector<double> next_tick(n_pools, 0.0), period(n_pools);
    for (int b = 0; b < n_pools; ++b) period[b] = pool_block[b] / fs;
    struct Inflight {
        bool on = false;
        double tick_t = 0.0;
        long long nmem = 0;
    };
    std::vector<Inflight> infl(n_pools);
    std::vector<Sample> lat;
    std::vector<std::vector<Sample>> pool_lat(n_pools);
    std::vector<long long> pool_blocks(n_pools, 0), pool_miss(n_pools, 0);
    long long miss = 0, blocks = 0, finished = 0, concurrent = 0, peak = 0;
    double audio = 0.0;
    int rc = PC_OK;

    // The tick loop must not wait on the host allocator: the pinned per-pool
    // blocks are sized up front (a pool's channel ids stay below the channels
    // of its requests).  Page-locking the impulse responses for the run, so
    // that admissions upload them by DMA, was measured and rejected: deadline
    // misses alike, but single stalls of 65-124 ms.
    {
        std::vector<long long> need(n_pools, 0);
        for (int i = 0; i < n_req; ++i) need[pool_of[i]] += channels[i];
        for (int b = 0; b < n_pools; ++b)
            if (need[b] > 0 && !ensure(b, (int)std::min<long long>(need[b], 1 << 16))) {
                free_all();
                return PC_ERR_NOMEM;
            }
    }

    const auto t0 = Clock::now();
    auto now = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
    while (finished < n_req && rc == PC_OK) {
        const double t = now();
        if (t > max_seconds) break;
        while (!pend.empty() && arrival[pend.front()] <= t) {
            queue.push_back(pend.front());
            pend.pop_front();
        }
        // admissions in arrival order: a request that does not fit waits, and
        // so do the ones behind it
        while (!queue.empty() && concurrent < max_concurrent) {
            const int ri = queue.front();
            pcs_handle* pool = pools[pool_of[ri]];
            std::vector<int> got;
            bool ok = true;
            for (int c = 0; c < channels[ri]; ++c) {
                std::vector<int> P(P_flat + lv0[ri], P_flat + lv0[ri + 1]);
                int pid = -1;
                const int r = pcs_admit_async(pool, irs[ch0[ri] + c], ir_len[ri], num_levels[ri], N_flat + lv0[ri],
                                              P.data(), &pid);
                if (r == PC_ERR_NOMEM || r == PC_ERR_LIMIT) {
                    ok = false;
                    break;
                }
                if (r != PC_OK) {
                    rc = r;
                    ok = false;
                    break;
                }
                got.push_back(pid);
            }
            if (!ok) {
                for (int pid : got) pcs_release(pool, pid);
                break;
            }
            queue.pop_front();
            pcs_of[ri] = got;
            waiting.push_back({ri, got});
            ++concurrent;
            peak = std::max(peak, concurrent);
        }
        if (rc != PC_OK) break;
        // admitted channels whose spectra are ready join at their pool's next tick
        if (!waiting.empty()) {
            for (int b = 0; b < n_pools; ++b) pcs_poll(pools[b], nullptr);
            std::vector<Waiting> still;
            for (auto& w : waiting) {
                const int b = pool_of[w.req];
                bool all_live = true;
                for (int pid : w.pids) all_live = all_live && pcs_is_live(pools[b], pid) == 1;
                if (!all_live) {
                    still.push_back(std::move(w));
                    continue;
                }
                for (int pid : w.pids) {
                    std::uniform_int_distribution<long long> d(0, noise_len - frames[w.req]);
                    live[b].push_back({pid, d(rng), 0, frames[w.req] / pool_block[b], w.req});
                }
            }
            waiting.swap(still);
        }
        bool progressed = false;
        for (int b = 0; b < n_pools && rc == PC_OK; ++b) {
            pcs_handle* pool = pools[b];
            const int blk = pool_block[b];
            if (infl[b].on && pcs_query(pool) == 1) {
                const double l = (now() - infl[b].tick_t) * 1e6;
                const long long nm = infl[b].nmem;
                lat.push_back({l, (double)nm});
                pool_lat[b].push_back({l, (double)nm});
                pool_blocks[b] += nm;
                blocks += nm;
                if (l > period[b] * 1e6) {
                    miss += nm;
                    pool_miss[b] += nm;
                }
                infl[b].on = false;
                progressed = true;
                // channels whose last block just completed leave the pool;
                // a request is done when all of its channels are
                std::vector<Chan> keep;
                keep.reserve(live[b].size());
                std::vector<int> done_reqs;
                for (auto& c : live[b]) {
                    if (c.left == 0) done_reqs.push_back(c.req);
                    else keep.push_back(c);
                }
                live[b].swap(keep);
                std::sort(done_reqs.begin(), done_reqs.end());
                done_reqs.erase(std::unique(done_reqs.begin(), done_reqs.end()), done_reqs.end());
                for (int ri : done_reqs) {
                    for (int pid : pcs_of[ri]) pcs_release(pool, pid);
                    pcs_of[ri].clear();
                    ++finished;
                    --concurrent;
                    audio += (double)channels[ri] * (double)frames[ri] / fs;
                }
            }
            if (!infl[b].on && !live[b].empty() && next_tick[b] <= t) {
                int nch = 0;
                for (auto& c : live[b]) nch = std::max(nch, c.pid + 1);
                if (!ensure(b, nch)) {
                    rc = PC_ERR_NOMEM;
                    break;
                }
                for (auto& c : live[b]) {
                    std::memcpy(hin[b] + (size_t)c.pid * blk, noise + c.off + c.pos * blk, sizeof(float) * blk);
                    ++c.pos;
                    --c.left;
                }
                const double tick_t = now();
                if (next_tick[b] < tick_t - period[b]) next_tick[b] = tick_t;   // fell behind: restart the cadence
                next_tick[b] += period[b];
                const int r = pcs_step(pool, hin[b], hout[b], nch);
                if (r != PC_OK) {
                    rc = r;
                    break;
                }
                infl[b] = {true, tick_t, (long long)live[b].size()};
                progressed = true;
            }
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
    for (int b = 0; b < n_pools; ++b)
        if (infl[b].on) pcs_sync(pools[b]);
    for (int ri = 0; ri < n_req; ++ri) {   // requests cut off by max_seconds
        for (int pid : pcs_of[ri]) pcs_release(pools[pool_of[ri]], pid);
        pcs_of[ri].clear();
    }
    for (auto& w : waiting)
        for (int pid : w.pids) pcs_release(pools[pool_of[w.req]], pid);
    free_all();

    const double wall = now();
    stats->requests = n_req;
    stats->finished = finished;
    stats->peak_concurrent = peak;
    stats->steps = (long long)lat.size();
    stats->blocks = blocks;
    stats->wall_s = wall;
    stats->audio_s = audio;
    stats->latency_p50_us = weighted_pct(lat, 0.50);
    stats->latency_p99_us = weighted_pct(lat, 0.99);
    double mx = 0.0;
    for (auto& s : lat) mx = std::max(mx, s.lat_us);
    stats->latency_max_us = mx;
    stats->miss_rate = blocks ? (double)miss / (double)blocks : 0.0;
    stats->n_pools = n_pools;
    for (int b = 0; b < n_pools; ++b) {
        stats->pool_block[b] = pool_block[b];
        stats->pool_steps[b] = (long long)pool_lat[b].size();
        stats->pool_blocks[b] = pool_blocks[b];
        stats->pool_p50_us[b] = weighted_pct(pool_lat[b], 0.50);
        stats->pool_p99_us[b] = weighted_pct(pool_lat[b], 0.99);
        stats->pool_miss_rate[b] = pool_blocks[b] ? (double)pool_miss[b] / (double)pool_blocks[b] : 0.0;
    }
    return rc;
}
