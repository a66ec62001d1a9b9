// kernels.h -- launchers for the kernels in step_kernels.cu and cluster_fire.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <string>

#include "engine_types.h"

namespace pcg {

// one filter-spectrum row: dst[0..N] = rfft([0_N, src[0..len)]) / 2N
struct SpectraJob {
    const float* src;
    int len;       // valid samples at src (<= N); the rest of the row is zero
    int N;
    int logN;
    float2* dst;
};

// kernel class by block size: 0 (N <= 1024), 1 (N <= 4096), 2 (N <= 16384),
// 3 (N <= 65536: a cluster of kClusterCtas CTAs per fire, cluster_fire.cu)
int fire_class_of(int N);
constexpr int kNumClasses = 4;
constexpr int kMaxBlockOneCta = 16384;   // largest block one CTA transforms (classes 0-2)
constexpr int kClusterCtas = 8;          // CTAs per class-3 fire
constexpr int kClusterMaxN = 65536;      // largest block of class 3
constexpr int kClusterInStepMinN = 8192;    // smallest in-step level that may run on a cluster
constexpr int kClusterInStepMaxCtas = 64;   // ... when its handle's in-step cluster fires need at most this many CTAs
// threads per CTA of a class
int class_threads(int cls);
// default bins and parts per spread task (the tile shape pc_set_tiles overrides)
int spread_task_bins();
int spread_task_parts();
// bins per spread task the spread kernels accept (64, 128, 256 or 512)
bool spread_bins_ok(int bins);
size_t class_smem_bytes(int cls, int maxN);
// dynamic shared memory of a step launch (class, largest block, the bank's
// base blocks per step)
size_t step_smem_bytes(int cls, int maxN, const Bank& bank);
// largest base-blocks-per-step K (a power of two <= 4) the level-0 kernel
// supports for base block N0 (K N0 <= 1024); 1 if none
int max_step_blocks(int N0);
// parts a K-block level-0 fire sums itself (the rest come from spread rows):
// the most that keep two of its CTAs per SM, at least 2K
int multi_fire_parts(int N0, int K);

cudaError_t prepare_kernels();
// pdl: let the launch overlap the previous kernel in the stream, which must
// be a step kernel of the same handle (or nothing)
// prio: 0 = the stream's priority, 1 = the device's highest, -1 = its lowest.
// whole_sm: request enough shared memory that no other CTA fits beside one
// of these (classes 1 and 2).
cudaError_t launch_step_class(int cls, int grid, int maxN, const Bank& bank, const Task* tasks, const RunState& rs,
                              const RunState* rs_dev, int step_in_batch, cudaStream_t st, bool pdl, int prio = 0,
                              bool whole_sm = false);
// spread tasks of levels >= 1 (several base blocks per step) as their own launch
cudaError_t launch_side_spreads(int grid, const Task* tasks, const RunState& rs, const RunState* rs_dev,
                                int step_in_batch, cudaStream_t st);
cudaError_t launch_pool_class(int cls, int grid, int maxN, const Bank& bank, const Task* slots, const PoolCta* map,
                              const RunState& rs, cudaStream_t st);
cudaError_t launch_spectra(int cls, int njobs, int maxN, const SpectraJob* jobs, const float2* W, int wlog,
                           cudaStream_t st);
cudaError_t launch_set_state(RunState* dst, const RunState& v, cudaStream_t st);

// class 3 (cluster_fire.cu): fires and filter spectra of levels with
// 16384 < N <= 65536, one cluster of kClusterCtas CTAs per task or job
size_t cluster_smem_bytes();
cudaError_t prepare_cluster_kernels();
cudaError_t launch_cluster_fire(int ntasks, const Bank& bank, const Task* tasks, const RunState& rs,
                                const RunState* rs_dev, int step_in_batch, cudaStream_t st, bool pdl, int prio);
cudaError_t launch_cluster_spectra(int njobs, const SpectraJob* jobs, const float2* W, int wlog, cudaStream_t st);
// PartConvFilter's runLevel for such a level (filter.cu), one cluster
cudaError_t launch_cluster_filter_level(int N, int P, int cs, unsigned bcurr, const float2* H, float2* X,
                                        float* win_old, const float* blk, float* out, const float2* W, int wlog,
                                        cudaStream_t st);

}  // namespace pcg

// last error of calls that have no handle (thread-local)
const char* pcg_global_error();
void pcg_set_global_error(const std::string& m);
