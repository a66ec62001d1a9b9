// Headless real-time driver: the audio device's callback loop without an
// audio device.  The reference drives PartConvMulti::run from a PortAudio or
// ALSA callback (src/pcRTMulti.cpp:138-185, :303-506) and counts output
// underflows; here a host thread releases one callback per block period on
// an absolute monotonic clock, calls pc_run on the block, and records how
// long each callback took from its release and whether it finished after its
// deadline (the next release, when the device would play the block).  A late
// callback does not move the clock: the following ones are released on
// schedule and start as soon as the late one returns, as with a sound card.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <thread>
#include <vector>

#include "../../include/partconv_gb300.h"

namespace {
using Clock = std::chrono::steady_clock;

double pct(std::vector<double>& v, double q) {
    if (v.empty()) return 0.0;
    const size_t k = std::min(v.size() - 1, (size_t)std::floor(q * (double)(v.size() - 1) + 0.5));
    std::nth_element(v.begin(), v.begin() + (long)k, v.end());
    return v[k];
}
}  // namespace

extern "C" int pc_rt_drive(pc_handle* h, const float* in, float* out, long long frames, double period_s,
                           int realtime, pc_rt_stats* stats) {
    if (!h || !in || !out || !stats) return PC_ERR_ARG;
    pc_info info;
    int r = pc_get_info(h, &info);
    if (r) return r;
    const int N0 = info.buffer_size;
    if (N0 <= 0 || info.fs <= 0) return PC_ERR_STATE;   // not set up
    if (frames <= 0 || frames % N0) return PC_ERR_ARG;
    if (period_s <= 0.0) period_s = (double)N0 / (double)info.fs;
    const long long n = frames / N0;
    std::vector<double> lat(n), comp(n);
    long long misses = 0;
    const auto per = std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(period_s));
    const auto t0 = Clock::now() + per;   // first release one period from now
    for (long long k = 0; k < n; ++k) {
        const auto rel = t0 + per * k;
        if (realtime) {
            // sleep to shortly before the release, then spin to it
            const auto early = rel - std::chrono::microseconds(200);
            if (Clock::now() < early) std::this_thread::sleep_until(early);
            while (Clock::now() < rel) {
            }
        }
        const auto a = Clock::now();
        r = pc_run(h, out + k * (long long)N0 * info.num_output_channels, in + k * (long long)N0 * info.num_input_channels,
                   N0);
        const auto b = Clock::now();
        if (r) return r;
        comp[k] = std::chrono::duration<double, std::micro>(b - a).count();
        lat[k] = realtime ? std::chrono::duration<double, std::micro>(b - rel).count() : comp[k];
        if (realtime && b > rel + per) ++misses;
    }
    double mean = 0.0;
    for (double c : comp) mean += c;
    stats->callbacks = n;
    stats->misses = misses;
    stats->period_us = period_s * 1e6;
    stats->compute_mean_us = n ? mean / (double)n : 0.0;
    stats->latency_p50_us = pct(lat, 0.50);
    stats->latency_p99_us = pct(lat, 0.99);
    stats->latency_max_us = n ? *std::max_element(lat.begin(), lat.end()) : 0.0;
    stats->wall_s = std::chrono::duration<double>(Clock::now() - (t0 - per)).count();
    return PC_OK;
}
