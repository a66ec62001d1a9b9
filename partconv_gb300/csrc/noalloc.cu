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
// The twiddle table is written once per device, by the first call on it,
// at the front of the array.  Every later call writes its descriptor tables
// with a one-CTA kernel from scalar launch arguments, so a call reads no
// host memory and makes no host-to-device copy.
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

// Where each table sits in the scratch array, and what the table kernel
// needs to write them (passed by value as the kernel's argument).
struct TableArgs {
    unsigned char* base;
    const float* h;
    int h_len, N, logN, P, cs, rin, nspread, spread_bins;
    size_t o_W, o_pc, o_lv, o_mix, o_tasks, o_jobs, o_H, o_X, o_Yp, o_xr;
};

// Writes the one-level layout's descriptors: the PC, its level, the mixing
// list of its single output, the fire task, the spread tasks (parts >= 2 in
// slices of spread_bins bins) and one filter-spectrum job per part.
__global__ void noalloc_tables_kernel(TableArgs a) {
    float2* H = reinterpret_cast<float2*>(a.base + a.o_H);
    float2* X = reinterpret_cast<float2*>(a.base + a.o_X);
    float2* Yp = reinterpret_cast<float2*>(a.base + a.o_Yp);
    float* xr = reinterpret_cast<float*>(a.base + a.o_xr);
    Task* tasks = reinterpret_cast<Task*>(a.base + a.o_tasks);
    SpectraJob* jobs = reinterpret_cast<SpectraJob*>(a.base + a.o_jobs);
    if (threadIdx.x == 0) {
        DevLevel lv{};
        lv.N = a.N;
        lv.logN = a.logN;
        lv.P = a.P;
        lv.T = 1;
        lv.cs = a.cs;
        lv.H = H;
        lv.X = X;
        lv.Yp = Yp;
        *reinterpret_cast<DevLevel*>(a.base + a.o_lv) = lv;
        DevPC pc{};
        pc.M = 1;
        pc.mix_mode = 1;
        pc.scale = 1.0f;
        pc.rin_mask = a.rin - 1;
        pc.xring = xr;
        *reinterpret_cast<DevPC*>(a.base + a.o_pc) = pc;
        int* mix = reinterpret_cast<int*>(a.base + a.o_mix);   // out_off = {0, 1}, out_pcs = {0}
        mix[0] = 0;
        mix[1] = 1;
        mix[2] = 0;
        mix[3] = 0;
        Task t{};
        t.kind = 0;
        t.N = a.N;
        t.logN = a.logN;
        t.P = a.P;
        t.T = 1;
        t.cs = a.cs;
        t.M = 1;
        t.mix_mode = 1;
        t.rin_mask = a.rin - 1;
        t.scale = 1.0f;
        t.H = H;
        t.X = X;
        t.Yp = Yp;
        t.xring = xr;
        tasks[0] = t;
    }
    for (int s = threadIdx.x; s < a.nspread; s += blockDim.x) {
        Task u{};
        u.kind = 1;
        u.N = a.N;
        u.P = a.P;
        u.T = 1;
        u.cs = a.cs;
        u.k0 = s * a.spread_bins;
        u.k1 = min(a.cs, u.k0 + a.spread_bins);
        u.p_lo = 2;
        u.H = H;
        u.X = X;
        u.Yp = Yp;
        tasks[1 + s] = u;
    }
    for (int p = threadIdx.x; p < a.P; p += blockDim.x) {
        const long start = (long)p * a.N;
        SpectraJob j;
        j.src = a.h + start;
        j.len = (int)min((long)a.N, (long)a.h_len - start);
        j.N = a.N;
        j.logN = a.logN;
        j.dst = H + (size_t)p * a.cs;
        jobs[p] = j;
    }
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

    // ---- one-level layout and the scratch carve-up (twiddles first) -------------------
    const int N = block_size, logN = (int)std::lround(std::log2((double)N));
    const int P = (int)((h_len + N - 1) / N);
    const int cs = N + 2;
    const int cls = fire_class_of(N);
    int Rin = 1;
    while (Rin < 2 * N) Rin <<= 1;
    const int nspread = P >= 3 ? (cs + spread_task_bins() - 1) / spread_task_bins() : 0;
    const int ntasks = 1 + nspread;

    size_t off = 0;
    TableArgs ta{};
    ta.o_W = take(off, sizeof(float2) << kWlog);
    ta.o_pc = take(off, sizeof(DevPC));
    ta.o_lv = take(off, sizeof(DevLevel));
    ta.o_mix = take(off, 4 * sizeof(int));
    ta.o_tasks = take(off, sizeof(Task) * ntasks);
    ta.o_jobs = take(off, sizeof(SpectraJob) * (size_t)P);
    ta.o_H = take(off, sizeof(float2) * (size_t)P * cs);
    const size_t state0 = off;
    ta.o_X = take(off, sizeof(float2) * (size_t)P * cs);
    ta.o_Yp = take(off, sizeof(float2) * 2 * (size_t)cs);
    ta.o_xr = take(off, sizeof(float) * (size_t)Rin);
    const size_t state1 = off;
    if (off > kScratchBytes) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "impulse response of %d taps at block size %d needs %zu bytes of scratch; the static array holds %zu",
                 h_len, N, off, kScratchBytes);
        return fail(PC_ERR_LIMIT, buf);
    }

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(PC_ERR_LIMIT, "device index beyond the supported range");
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            // first call on this device (it is the current device): resolve the
            // device address of the scratch array and write the twiddle table
            // exp(-2 pi i m / 2^15), computed in double like the engine's, at
            // its front once (a synchronous copy)
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess)
                return fail(PC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            e = prepare_kernels();
            if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(e));
            std::vector<float2> W((size_t)1 << kWlog);
            for (size_t m = 0; m < W.size(); ++m) {
                const double a = -2.0 * M_PI * (double)m / (double)W.size();
                W[m] = make_float2((float)std::cos(a), (float)std::sin(a));
            }
            e = cudaMemcpy(p, W.data(), sizeof(float2) * W.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("twiddle upload: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        }
        base = g_scratch_addr[dev];
    }

    // ---- descriptor tables (a kernel: no host memory is read), cleared state,
    //      filter spectra, steps ------------------------------------------------------------
    ta.base = base;
    ta.h = d_h;
    ta.h_len = h_len;
    ta.N = N;
    ta.logN = logN;
    ta.P = P;
    ta.cs = cs;
    ta.rin = Rin;
    ta.nspread = nspread;
    ta.spread_bins = spread_task_bins();
    noalloc_tables_kernel<<<1, 256, 0, st>>>(ta);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemsetAsync(base + state0, 0, state1 - state0, st)) != cudaSuccess)
        return fail(PC_ERR_CUDA, std::string("scratch tables: ") + cudaGetErrorString(e));
    e = launch_spectra(cls, P, N, reinterpret_cast<const SpectraJob*>(base + ta.o_jobs),
                       reinterpret_cast<const float2*>(base + ta.o_W), kWlog, st);
    if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("filter spectra: ") + cudaGetErrorString(e));

    Bank bank{};
    bank.pcs = reinterpret_cast<const DevPC*>(base + ta.o_pc);
    bank.lv = reinterpret_cast<const DevLevel*>(base + ta.o_lv);
    bank.W = reinterpret_cast<const float2*>(base + ta.o_W);
    bank.wlog = kWlog;
    bank.N0 = N;
    bank.n_out = 1;
    bank.out_off = reinterpret_cast<const int*>(base + ta.o_mix);
    bank.out_pcs = reinterpret_cast<const int*>(base + ta.o_mix) + 2;
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
    const Task* d_tasks = reinterpret_cast<const Task*>(base + ta.o_tasks);
    for (long long c = 0; c < nsteps; ++c) {
        rs.step_base = c;
        // the first step follows the spectra kernel, so it must not overlap it
        e = launch_step_class(cls, ntasks, N, bank, d_tasks, rs, nullptr, 0, st, c > 0);
        if (e != cudaSuccess) return fail(PC_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    }
    pcg_set_global_error("");
    return PC_OK;
}
