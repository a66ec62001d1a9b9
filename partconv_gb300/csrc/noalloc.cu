// noalloc.cu -- uniformly partitioned convolution whose working memory is a
// fixed static device array, for callers that must not allocate device
// memory.
//
// Some hosts own every device allocation themselves: an audio plug-in loaded
// into a host application that pre-allocates and accounts for all GPU
// memory, code running under an allocator or memory pool that forbids
// cudaMalloc, or a real-time thread that must never block in the driver's
// allocator.  pc_convolve_noalloc serves them: the caller passes device
// pointers for the input, the impulse response and the output, and every
// other byte the computation needs (filter spectra, spectrum ring, partial
// sums, input ring, task table, twiddles) lives in kScratchBytes of
// file-scope __device__ memory that every GPU loading this library holds
// until the process exits.  No call here allocates or frees device memory.
//
// The work is the step kernel of the multi-level engine run on a one-level
// layout (block size N0, P = ceil(len(h) / N0) parts), so the result equals
// pc_run over the same samples with a fresh handle.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/partconv_gb300.h"
#include "engine_types.h"
#include "kernels.h"

using namespace pcg;

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;   // PC_NOALLOC_SCRATCH_BYTES
static_assert(kScratchBytes == (size_t)PC_NOALLOC_SCRATCH_BYTES, "header and implementation disagree");
constexpr int kWlog = 15;
constexpr int kMaxDevices = 64;

// The scratch array.  In host code its name is only a host-side stand-in;
// the device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

int fail(int code, const std::string& m) {
    pcg_set_global_error(m);
    return code;
}

size_t take(size_t& off, size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
}

}  // namespace

extern "C" int pc_convolve_noalloc(const float* d_x, long long n_frames, const float* d_h, int h_len, float* d_y,
                                   int block_size, void* stream) {
    if (!d_x || !d_h || !d_y) return fail(PC_ERR_ARG, "null device pointer");
    if (block_size < 16 || block_size > 1024 || (block_size & (block_size - 1)))
        return fail(PC_ERR_ARG, "block_size must be a power of two in [16, 1024]");
    if (n_frames <= 0 || n_frames % block_size) return fail(PC_ERR_ARG, "n_frames must be a positive multiple of block_size");
    if (h_len < 1) return fail(PC_ERR_ARG, "empty impulse response");
    cudaStream_t st = (cudaStream_t)stream;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(PC_ERR_LIMIT, "device index beyond the supported range");
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            // first call on this device (it is the current device): resolve the
            // device address of the scratch array
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess)
                return fail(PC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            e = prepare_kernels();
            if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        }
        base = g_scratch_addr[dev];
    }

    // ---- one-level layout and the scratch carve-up ---------------------------------
    const int N = block_size, logN = (int)std::lround(std::log2((double)N));
    const int P = (int)((h_len + N - 1) / N);
    const int cs = N + 2;
    const int cls = fire_class_of(N);
    int Rin = 1;
    while (Rin < 2 * N) Rin <<= 1;
    const int nspread = P >= 3 ? (cs + spread_task_bins() - 1) / spread_task_bins() : 0;
    const int ntasks = 1 + nspread;

    size_t off = 0;
    const size_t o_W = take(off, sizeof(float2) << kWlog);
    const size_t o_pc = take(off, sizeof(DevPC));
    const size_t o_lv = take(off, sizeof(DevLevel));
    const size_t o_mix = take(off, 4 * sizeof(int));
    const size_t o_tasks = take(off, sizeof(Task) * ntasks);
    const size_t o_jobs = take(off, sizeof(SpectraJob) * (size_t)P);
    const size_t o_H = take(off, sizeof(float2) * (size_t)P * cs);
    const size_t state0 = off;
    const size_t o_X = take(off, sizeof(float2) * (size_t)P * cs);
    const size_t o_Yp = take(off, sizeof(float2) * 2 * (size_t)cs);
    const size_t o_xr = take(off, sizeof(float) * (size_t)Rin);
    const size_t state1 = off;
    if (off > kScratchBytes) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "impulse response of %d taps at block size %d needs %zu bytes of scratch; the static array holds %zu",
                 h_len, N, off, kScratchBytes);
        return fail(PC_ERR_LIMIT, buf);
    }

    // ---- host images of the tables ----------------------------------------------------
    std::vector<float2> W((size_t)1 << kWlog);
    for (size_t m = 0; m < W.size(); ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)W.size();
        W[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    DevLevel lv{};
    lv.N = N;
    lv.logN = logN;
    lv.P = P;
    lv.T = 1;
    lv.s_blocks = 0;
    lv.cs = cs;
    lv.rmask = 0;
    lv.pc = 0;
    lv.H = reinterpret_cast<float2*>(base + o_H);
    lv.X = reinterpret_cast<float2*>(base + o_X);
    lv.Yp = reinterpret_cast<float2*>(base + o_Yp);
    lv.yring = nullptr;
    DevPC pc{};
    pc.M = 1;
    pc.lv0 = 0;
    pc.mix_mode = 1;
    pc.scale = 1.0f;
    pc.rin_mask = Rin - 1;
    pc.xring = reinterpret_cast<float*>(base + o_xr);
    pc.pcout = nullptr;
    int mix[4] = {0, 1, 0, 0};   // out_off = {0, 1}, out_pcs = {0}
    std::vector<Task> tasks(ntasks);
    {
        Task& t = tasks[0];
        t = Task{};
        t.kind = 0;
        t.N = N;
        t.logN = logN;
        t.P = P;
        t.T = 1;
        t.cs = cs;
        t.M = 1;
        t.mix_mode = 1;
        t.rin_mask = Rin - 1;
        t.scale = 1.0f;
        t.H = lv.H;
        t.X = lv.X;
        t.Yp = lv.Yp;
        t.xring = pc.xring;
        for (int s = 0; s < nspread; ++s) {
            Task& u = tasks[1 + s];
            u = Task{};
            u.kind = 1;
            u.N = N;
            u.P = P;
            u.T = 1;
            u.cs = cs;
            u.k0 = s * spread_task_bins();
            u.k1 = std::min(cs, u.k0 + spread_task_bins());
            u.p_lo = 2;
            u.H = lv.H;
            u.X = lv.X;
            u.Yp = lv.Yp;
        }
    }
    std::vector<SpectraJob> jobs(P);
    for (int p = 0; p < P; ++p) {
        const long start = (long)p * N;
        jobs[p].src = d_h + start;
        jobs[p].len = (int)std::min<long>(N, (long)h_len - start);
        jobs[p].N = N;
        jobs[p].logN = logN;
        jobs[p].dst = lv.H + (size_t)p * cs;
    }

    // ---- uploads (pageable host sources are staged by the driver before the
    //      call returns), clear the state, filter spectra, steps ------------------
    auto cp = [&](size_t o, const void* src, size_t bytes) {
        return cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, st);
    };
    if ((e = cp(o_W, W.data(), sizeof(float2) * W.size())) != cudaSuccess ||
        (e = cp(o_pc, &pc, sizeof pc)) != cudaSuccess || (e = cp(o_lv, &lv, sizeof lv)) != cudaSuccess ||
        (e = cp(o_mix, mix, sizeof mix)) != cudaSuccess ||
        (e = cp(o_tasks, tasks.data(), sizeof(Task) * tasks.size())) != cudaSuccess ||
        (e = cp(o_jobs, jobs.data(), sizeof(SpectraJob) * jobs.size())) != cudaSuccess ||
        (e = cudaMemsetAsync(base + state0, 0, state1 - state0, st)) != cudaSuccess)
        return fail(PC_ERR_CUDA, std::string("scratch upload: ") + cudaGetErrorString(e));
    e = launch_spectra(cls, P, N, reinterpret_cast<const SpectraJob*>(base + o_jobs),
                       reinterpret_cast<const float2*>(base + o_W), kWlog, st);
    if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("filter spectra: ") + cudaGetErrorString(e));

    Bank bank{};
    bank.pcs = reinterpret_cast<const DevPC*>(base + o_pc);
    bank.lv = reinterpret_cast<const DevLevel*>(base + o_lv);
    bank.W = reinterpret_cast<const float2*>(base + o_W);
    bank.wlog = kWlog;
    bank.N0 = N;
    bank.n_out = 1;
    bank.out_off = reinterpret_cast<const int*>(base + o_mix);
    bank.out_pcs = reinterpret_cast<const int*>(base + o_mix) + 2;
    bank.mix_cnt = nullptr;
    bank.zero_list = nullptr;
    RunState rs{};
    rs.io.in = d_x;
    rs.io.out = d_y;
    rs.io.step0 = 0;
    rs.io.in_step = N;
    rs.io.in_sample = 1;
    rs.io.in_ch = 0;
    rs.io.out_step = N;
    rs.io.out_sample = 1;
    rs.io.out_ch = 0;
    const long long nsteps = n_frames / N;
    const Task* d_tasks = reinterpret_cast<const Task*>(base + o_tasks);
    for (long long c = 0; c < nsteps; ++c) {
        rs.step_base = c;
        // the first step follows the spectra kernel, so it must not overlap it
        e = launch_step_class(cls, ntasks, N, bank, d_tasks, rs, nullptr, 0, st, c > 0);
        if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    }
    pcg_set_global_error("");
    return PC_OK;
}
