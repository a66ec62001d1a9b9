/*
 * partconv_gb300.h -- C ABI of the GB300 (sm_103a) partitioned-convolution
 * engine.
 *
 * The engine is a drop-in for PartConvMulti / PartConvMultiRelaxed
 * (src/partconvMulti.h:52-148 in ebattenberg/partconv).  One handle holds one
 * multi-instance convolver: a set of partitioned convolvers ("PCs"), each
 * mapping one input channel through one impulse response (IR) to one output
 * channel, like a pc.config line.
 *
 * Conventions:
 *   - Every call returns PC_OK (0) or a positive PC_ERR_* code.  Unlike the
 *     reference, which calls exit(-1) on bad configs and frame counts
 *     (src/partconvMulti.cpp:31-40, :74-106, :817-821), no call exits the
 *     process.  pc_last_error() gives the message of the last failure.
 *   - Host buffers are interleaved float32 [frame][channel] like the
 *     reference's run() buffers unless a call takes a layout flag.
 *   - Calls on one handle are not re-entrant (run() in the reference is
 *     called from one audio thread).  Different handles are independent.
 *   - Signatures use plain pointers and sizes only; cudaStream_t is passed
 *     as void*.
 */
#ifndef PARTCONV_GB300_H
#define PARTCONV_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PC_OK 0
#define PC_ERR_ARG 1      /* bad argument (null pointer, frame count, channel index) */
#define PC_ERR_LAYOUT 2   /* partition layout rejected (see pc_check_layout) */
#define PC_ERR_CONFIG 3   /* config file missing or malformed */
#define PC_ERR_IO 4       /* impulse-response file missing or unreadable */
#define PC_ERR_CUDA 5     /* CUDA runtime failure or no device */
#define PC_ERR_NOMEM 6    /* device allocation failed */
#define PC_ERR_STATE 7    /* call out of order (run before setup, setup twice) */
#define PC_ERR_LIMIT 8    /* size beyond a documented limit */

/* Interleaved [frame][channel] and planar [channel][frame] host/device layouts. */
#define PC_INTERLEAVED 0
#define PC_PLANAR 1

/* Largest block size a level may use (the FFT length is twice this).  The
 * pc_* engine and PartConvFilter (pcf_*) transform blocks above 16384 with a
 * cluster of CTAs; the MIMO (pcm_*), differentiable (pcd_*) and serving
 * (pcs_*) paths take blocks up to 16384 and return PC_ERR_LIMIT above. */
#define PC_MAX_BLOCK 65536
/* Most levels one convolver may have. */
#define PC_MAX_LEVELS 16

typedef struct pc_handle pc_handle;

/* Counters and sizes of a set-up handle (read-only snapshot). */
typedef struct pc_info {
    int fs;                  /* sample rate (reported only) */
    int buffer_size;         /* base block N0 = frames per run() call */
    int num_input_channels;
    int num_output_channels;
    int num_pcs;
    int max_block_size;
    int relaxed;             /* 1: PartConvMultiRelaxed semantics */
    int hyperperiod;         /* steps after which the level schedule repeats */
    long long frame_num;     /* run() calls so far (PartConvMulti::frameNum) */
    long long device_bytes;  /* device memory held by the handle */
    int step_blocks;         /* base blocks computed per step (pc_set_step_blocks) */
    int spread_bins;         /* bins per spread task in use (pc_set_tiles) */
    int spread_parts;        /* parts per spread task in use (pc_set_tiles) */
} pc_info;

/*
 * Layout check, host only.  Replaces the validation in
 * PartConvFilter::setup (src/partconv.cpp:87-181): block sizes are powers of
 * two and strictly increasing, every level but the last has >= 1 part, the
 * slack test passes, and the last level is needed.  relaxed = 0 is the
 * reference's check 2*N0 + s_{L} >= 2*N_{L} (partconv.cpp:148-166);
 * relaxed = 1 is matlab/MFDL_part_conv.m:25-31, s_L >= N_L.  On success
 * P[M-1] is recomputed from ir_len (partconv.cpp:169-181) and delays[L]
 * (may be NULL) gets (2*N0 + s_L)/N0 as in partconv.cpp:148-153.
 * Also rejects N[M-1] > PC_MAX_BLOCK and M > PC_MAX_LEVELS (PC_ERR_LIMIT).
 */
int pc_check_layout(int M, const int* N, int* P, int ir_len, int relaxed, int* delays,
                    char* msg, int msglen);

/* PartConvMulti(int verbosity) -- src/partconvMulti.h:56. */
pc_handle* pc_create(int verbosity);

/*
 * PartConvMulti::setup(config_file, max_threads_per_level, max_level0_threads,
 * min_work) -- src/partconvMulti.h:58, src/partconvMulti.cpp:23-718.
 * Parses the pc.config format (header "FS buffer_size nIn nOut numPCs
 * numRepeats", then per PC "file mute inCh outCh scale M N0 P0 N1 P1 ...",
 * src/pc.config:43-44) and reads each IR from a WAV file (16/24/32-bit PCM or
 * 32-bit float, channel 0, like readImpulseResponse in src/sndtools.cpp:3-47).
 * Relative IR paths are resolved against the config file's directory.
 * The thread arguments are accepted for signature compatibility; the GPU
 * schedule has no host worker threads.
 */
int pc_setup_config(pc_handle* h, const char* config_file, int max_threads_per_level,
                    int max_level0_threads, double min_work);

/*
 * Programmatic setup (no file).  Same semantics as a pc.config with num_pcs
 * lines: PC i has num_levels[i] levels with block sizes and part counts at
 * offset sum(num_levels[0..i)) in block_sizes / num_parts (the last level's
 * part count is ignored and recomputed), IR irs[i] of ir_lens[i] samples,
 * input channel in_ch[i], output channel out_ch[i], input scale scale[i] and
 * mute flag mute[i] (muted PCs are computed but not mixed,
 * partconvMulti.cpp:911-921).  Layouts must pass the relaxed check; every
 * PC's first block size must equal buffer_size (partconvMulti.cpp:95-101).
 */
int pc_setup_layout(pc_handle* h, int fs, int buffer_size, int n_in, int n_out, int num_pcs,
                    const int* num_levels, const int* block_sizes, const int* num_parts,
                    const float* const* irs, const int* ir_lens, const int* in_ch,
                    const int* out_ch, const float* scale, const int* mute);

/*
 * Selects PartConvMultiRelaxed semantics (src/partconvMulti.h:142-148): the
 * output of each run() is the previous call's result, one base block later
 * (src/partconvMulti.cpp:1077-1111).  Call after setup; resets state.
 */
int pc_set_relaxed(pc_handle* h, int relaxed);

/*
 * Offline throughput option, no reference counterpart: compute k base blocks
 * per step (k a power of two, 1..8; call before setup; up to 4 are used).  Each step's
 * level-0 work for all PCs is one launch that transforms and convolves k
 * consecutive blocks at once, and every larger level runs beside the steps.
 * The output equals that of k times as many one-block steps to float32
 * rounding (the same partitions and products, summed in another order).
 * Setup lowers k to the largest value the layouts allow (k buffer_size <=
 * 1024, every level's N_L a multiple of k buffer_size); pc_get_info reports
 * it.  With k > 1, pc_run returns PC_ERR_STATE and pc_process needs a
 * multiple of k buffer_size frames.
 */
int pc_set_step_blocks(pc_handle* h, int k);

/*
 * Kernel tile shape, no reference counterpart (the measured-GPU autotuner,
 * partconv_gb300/autotune.py, picks it the way the reference's tune.py picks
 * layouts, src/tune.py:21-154): the streaming FDL multiply-accumulate of the
 * parts a fire does not sum itself is cut into spread tasks of spread_bins
 * bins (64, 128, 256 or 512) and spread_parts parts (1..64; a level
 * keeps one partial-sum row per group of spread_parts parts).  0 keeps the
 * default (128 bins, 16 parts).  Call before setup; results differ between
 * tile shapes only by float32 rounding (sums grouped differently).
 */
int pc_set_tiles(pc_handle* h, int spread_bins, int spread_parts);

/*
 * PartConvMulti::run(output, input, frameCount) -- src/partconvMulti.h:60,
 * src/partconvMulti.cpp:815-928.  Host interleaved buffers of frame_count ==
 * buffer_size frames.  Copies the block to the device, runs one base step and
 * copies the mixed output back before returning.
 */
int pc_run(pc_handle* h, float* output, const float* input, int frame_count);

/*
 * Batched form of run(): frames (a multiple of buffer_size) are processed as
 * frames/buffer_size consecutive callbacks with results identical to that
 * many pc_run calls.  Host buffers in the given layout (PC_INTERLEAVED or
 * PC_PLANAR with row length frames).  Steps run as CUDA-graph replays.
 * No reference counterpart (the reference has only run()).
 */
int pc_process(pc_handle* h, float* output, const float* input, long long frames, int layout);

/*
 * Same as pc_process with device-resident buffers, enqueued on the caller's
 * stream (void* = cudaStream_t; NULL is the CUDA default stream, as in every
 * CUDA API).  Returns after enqueueing; the caller synchronises the stream.
 */
int pc_process_device(pc_handle* h, float* d_output, const float* d_input, long long frames,
                      int layout, void* stream);

/* PartConvMulti::reset() -- src/partconvMulti.cpp:806-813: clears all state. */
int pc_reset(pc_handle* h);

/* PartConvMulti::cleanup() -- src/partconvMulti.cpp:720-804: frees device
 * resources; the handle can be set up again. */
int pc_cleanup(pc_handle* h);

/* Frees the handle (after cleanup if needed). */
void pc_destroy(pc_handle* h);

/* Message of the last failing call on h (or of pc_create when h is NULL). */
const char* pc_last_error(const pc_handle* h);

/* Snapshot of sizes and counters. */
int pc_get_info(const pc_handle* h, pc_info* info);

/* Partition layout of PC `pc` after setup (last-level part count recomputed). */
int pc_get_layout(const pc_handle* h, int pc, int* num_levels, int* block_sizes, int* num_parts);

/*
 * Kernel launches the handle made since creation (every kernel of this
 * library counts one).  Lets callers check that work ran on the GPU.
 */
long long pc_kernel_launches(const pc_handle* h);

/* Per-kernel timing record filled by pc_profile_kernels. */
typedef struct pc_kernel_stats {
    char name[32];         /* "step_small", "step_mid", "step_large", "step_huge": the step
                              kernel of block-size class N <= 1024, <= 4096, <= 16384,
                              <= 65536 (a cluster of 8 CTAs per fire); "spread_side" */
    long long launches;    /* launches that had work in their phase */
    double total_ms;       /* CUDA-event time summed over those launches */
    double alg_bytes;      /* algorithmic bytes those launches had to move */
} pc_kernel_stats;

/*
 * Profiling aid (no reference counterpart; the reference's
 * PartConvFilter::bench, src/partconv.cpp:508-566, times one level on the
 * CPU).  Runs nsteps further base steps from the handle's staging input (the
 * FDL state continues), launching each kernel separately on the handle's
 * stream with CUDA events around it, and writes up to max_kinds records.
 * Algorithmic bytes per level block: filter spectra and input-spectrum rows
 * read, the new spectrum row written, the 2N-sample window read and N
 * samples written.
 */
int pc_profile_kernels(pc_handle* h, long long nsteps, pc_kernel_stats* out, int max_kinds, int* n_kinds);

/* Statistics of one pc_rt_drive run (times in microseconds). */
typedef struct pc_rt_stats {
    long long callbacks;      /* blocks processed */
    long long misses;         /* callbacks that returned after their deadline */
    double period_us;         /* block period */
    double compute_mean_us;   /* mean time inside pc_run */
    double latency_p50_us;    /* release-to-return time (compute time when not real-time) */
    double latency_p99_us;
    double latency_max_us;
    double wall_s;            /* wall time of the run */
} pc_rt_stats;

/*
 * Headless real-time driver, in place of the audio callback loop of the
 * reference's programs (src/pcRTMulti.cpp:138-185 PortAudio, :303-506 ALSA,
 * which count output underflows).  Calls pc_run once per block of
 * buffer_size frames, releasing callback k at k periods after the start on a
 * monotonic clock (realtime != 0; 0 runs back to back), and counts a miss
 * when a callback returns after the next release, the time the device would
 * play its block.  period_s <= 0 means buffer_size / fs.  `in` / `out` are
 * interleaved host buffers of `frames` frames (a multiple of buffer_size).
 * The handle's frame counter advances as with pc_run.
 */
int pc_rt_drive(pc_handle* h, const float* in, float* out, long long frames, double period_s, int realtime,
                pc_rt_stats* stats);

/* ---------------------------------------------------------------------------
 * PartConvFilter: one partitioned convolver driven level by level, the class
 * the reference's Python module exposes (src/partconv.h:40-114, wrapped by
 * src/partconv.i:3-12) and tune.py drives.  Same index state and DelayBuffer /
 * DoubleBuffer schedule as the reference (src/partconv.cpp:354-648,
 * :1401-1511); buffers and runLevel's FFT/MAC/IFFT run on the GPU.
 * ------------------------------------------------------------------------- */
typedef struct pcf_handle pcf_handle;

/* PartConvFilter(verbosity, sampleRate) -- src/partconv.h:47. */
pcf_handle* pcf_create(int verbosity, int sample_rate);

/* PartConvFilter::setup(M, N, num_parts, impulse, fftwOptLevel, wisdom) --
 * src/partconv.cpp:70-306.  ir == NULL benches with an all-ones IR of
 * sum(N*P) taps (partconv.cpp:132-142).  Layout rules as pc_check_layout;
 * relaxed_check = 0 is the reference's check.  P[M-1] is recomputed.
 * Returns PC_ERR_LAYOUT where the reference returns 1. */
int pcf_setup(pcf_handle* h, int M, const int* N, int* P, const float* ir, int ir_len, int relaxed_check);

/* sync_levels() (relaxed = 0) / sync_levels_relaxed() (relaxed = 1) --
 * src/partconv.cpp:568-603. */
int pcf_sync_levels(pcf_handle* h, int relaxed);

/* input(const float*) -- src/partconv.cpp:605-613: N[0] host samples. */
int pcf_input(pcf_handle* h, const float* x);

/* runLevel(L) -- src/partconv.cpp:354-490.  Where the reference exits on a
 * DelayBuffer overlap (partconv.cpp:1449-1455) this returns PC_ERR_STATE. */
int pcf_run_level(pcf_handle* h, int L);

/* output(float*) (relaxed = 0) / output_relaxed(float*) (relaxed = 1) --
 * src/partconv.cpp:616-648: N[0] host samples. */
int pcf_output(pcf_handle* h, float* y, int relaxed);

/* reset() -- src/partconv.cpp:492-506. */
int pcf_reset(pcf_handle* h);

/* bench(L, trials, pollute_every, max_time, benchData) --
 * src/partconv.cpp:508-566: mean seconds of runLevel(L) (CUDA events);
 * pollution writes a buffer larger than the GPU's L2.  Negative on error. */
double pcf_bench(pcf_handle* h, int L, int trials, int pollute_every, double max_time, double* bench_data);

/* cleanup() -- src/partconv.cpp:308-352; pcf_destroy frees the handle. */
int pcf_cleanup(pcf_handle* h);
void pcf_destroy(pcf_handle* h);
const char* pcf_last_error(const pcf_handle* h);
int pcf_get_parts(const pcf_handle* h, int* P);
/* 1 if a runLevel found the DelayBuffer read and write blocks equal. */
int pcf_overlap_error(const pcf_handle* h);

/* ---------------------------------------------------------------------------
 * MIMO convolution: n_in inputs, n_out outputs, y_o = sum_i x_i * h_{i,o},
 * all paths with one layout.  No reference counterpart as one object: the
 * reference runs one PartConvFilter per path and sums outputs in time
 * (src/partconvMulti.cpp:911-921); here each input's spectrum is computed
 * once and every output's FDL sums over inputs per frequency bin.
 * ------------------------------------------------------------------------- */
typedef struct pcm_handle pcm_handle;

pcm_handle* pcm_create(int verbosity);

/* irs: n_in * n_out * ir_len floats, path (i, o) at (i * n_out + o) * ir_len.
 * N/P as in pc_setup_layout (relaxed check; P[M-1] recomputed in place). */
int pcm_setup(pcm_handle* h, int fs, int buffer_size, int n_in, int n_out, int M, const int* N, int* P,
              const float* irs, int ir_len);

/* frames (a multiple of buffer_size) of device input -> device output,
 * PC_INTERLEAVED or PC_PLANAR, enqueued on stream (NULL = default). */
int pcm_process_device(pcm_handle* h, float* d_out, const float* d_in, long long frames, int layout,
                       void* stream);
int pcm_reset(pcm_handle* h);
/* Per-kernel CUDA-event timing (names "mimo_xfft", "mimo_mac", "mimo_yifft"). */
int pcm_profile_kernels(pcm_handle* h, long long nsteps, pc_kernel_stats* out, int max_kinds, int* n_kinds);
long long pcm_device_bytes(const pcm_handle* h);
long long pcm_kernel_launches(const pcm_handle* h);
const char* pcm_last_error(const pcm_handle* h);
void pcm_destroy(pcm_handle* h);

/* ---------------------------------------------------------------------------
 * Differentiable partitioned convolution (no reference counterpart: the
 * reference has no gradients).  y_s = (x_s * h)[0:T] for a batch of signals,
 * all blocks of a level computed in parallel, and hand-written adjoints:
 * dL/dx with conjugated filter spectra (anti-causal), dL/dh as a partitioned
 * cross-correlation of the input with dL/dy in the same layout.
 * ------------------------------------------------------------------------- */
typedef struct pcd_plan pcd_plan;

/* Layout as pc_check_layout (relaxed; P[M-1] recomputed); batch signals of
 * `length` samples; h of ir_len taps.  Builds the plan's FFT job tables on
 * the current device (one allocation, freed by pcd_destroy); calls must run
 * on that device.  NULL on error (message in msg). */
pcd_plan* pcd_create(int M, const int* N, int* P, int ir_len, int batch, long long length, char* msg,
                     int msglen);
/* Device workspace the caller provides to forward/backward (they allocate
 * nothing); forward leaves filter and input spectra in it for backward. */
long long pcd_workspace_bytes(const pcd_plan* p);
/* y[batch][length] from x[batch][length] and h[ir_len] (device pointers). */
int pcd_forward(pcd_plan* p, const float* d_x, const float* d_h, float* d_y, void* d_ws, void* stream);
/* dL/dx (d_gx, may be NULL) and dL/dh (d_gh, may be NULL) from dL/dy.
 * recompute = 1 rebuilds the spectra from x and h instead of reading the
 * ones the forward pass left (needed when the workspace was reused, and for
 * a second backward: the adjoint pass overwrites the input spectra). */
int pcd_backward(pcd_plan* p, const float* d_x, const float* d_h, const float* d_gy, float* d_gx, float* d_gh,
                 void* d_ws, int recompute, void* stream);
void pcd_destroy(pcd_plan* p);
const char* pcd_last_error(const pcd_plan* p);
long long pcd_kernel_launches(const pcd_plan* p);

/* ---------------------------------------------------------------------------
 * Serving pool (no reference counterpart: the reference's PartConvMulti is
 * fixed at setup).  Partitioned convolvers of one base block size join and
 * leave between steps; their spectra and FDL state live in one device arena
 * of hbm_budget_bytes, and admission beyond it is refused (PC_ERR_NOMEM) so
 * the caller can queue the request.  Each pcs_step advances every active PC
 * by one base block in one batched launch per block-size class.
 * ------------------------------------------------------------------------- */
typedef struct pcs_handle pcs_handle;

/* buffer_size: a power of two in [16, 1024]; max_pcs: channel capacity. */
pcs_handle* pcs_create(int buffer_size, long long hbm_budget_bytes, int max_pcs);
/* Admit one PC (IR, layout as pc_check_layout, at most 5 levels); its id is
 * also its I/O channel.  Its schedule starts at the pool's next step. */
int pcs_admit(pcs_handle* h, const float* ir, int ir_len, int M, const int* N, int* P, int* pc_id);
/* Same without waiting for the PC's spectra: the PC is pending until a
 * pcs_poll finds its admission work completed and makes it live (its
 * schedule then starts at the pool's next step; pcs_is_live tells). */
int pcs_admit_async(pcs_handle* h, const float* ir, int ir_len, int M, const int* N, int* P, int* pc_id);
/* Make live every pending PC whose admission work has completed; the count
 * goes to *n_published (may be NULL). */
int pcs_poll(pcs_handle* h, int* n_published);
int pcs_is_live(const pcs_handle* h, int pc_id);
int pcs_release(pcs_handle* h, int pc_id);
/* One step: host in/out [n_channels][buffer_size] (pinned for asynchrony);
 * returns after enqueueing; pcs_query / pcs_sync observe completion. */
int pcs_step(pcs_handle* h, const float* in, float* out, int n_channels);
int pcs_query(pcs_handle* h);
int pcs_sync(pcs_handle* h);
long long pcs_bytes_in_use(const pcs_handle* h);
int pcs_live(const pcs_handle* h);
long long pcs_kernel_launches(const pcs_handle* h);
const char* pcs_last_error(const pcs_handle* h);
void pcs_destroy(pcs_handle* h);

/* Most pools pcs_run_load drives. */
#define PCS_LOAD_MAX_POOLS 8

/* Statistics of one pcs_run_load run (latencies in microseconds, weighted by
 * the channels each step carried). */
typedef struct pcs_load_stats {
    long long requests, finished, peak_concurrent, steps, blocks;
    double wall_s, audio_s;
    double latency_p50_us, latency_p99_us, latency_max_us;
    double miss_rate;                 /* channel blocks whose step ended after the next release */
    int n_pools;
    int pool_block[PCS_LOAD_MAX_POOLS];
    long long pool_steps[PCS_LOAD_MAX_POOLS], pool_blocks[PCS_LOAD_MAX_POOLS];
    double pool_p50_us[PCS_LOAD_MAX_POOLS], pool_p99_us[PCS_LOAD_MAX_POOLS], pool_miss_rate[PCS_LOAD_MAX_POOLS];
} pcs_load_stats;

/*
 * Real-time serving loop in native code (the counterpart of the reference's
 * audio callback loop, src/pcRTMulti.cpp:138-185 and :303-365, which runs one
 * fixed convolver and counts late callbacks).  Pools pools[0..n_pools) of
 * base block sizes pool_block[] step every pool_block / fs seconds on a
 * monotonic clock.  Request r arrives at arrival[r] seconds after the start,
 * joins pool pool_of[r] with channels[r] channels (IR irs[c] for its channels
 * c at the prefix sum of channels, ir_len[r] taps each; layout num_levels[r]
 * levels at the prefix sum of num_levels in N_flat / P_flat) when the pool's
 * HBM budget admits it (in arrival order), reads frames[r] samples per
 * channel from the float32 buffer noise (a seeded offset per channel), and
 * leaves when they are done.  Outputs are discarded.  Per step the latency
 * from its release to its completion is recorded, and a deadline miss when
 * it ends after the next release.  Stops after max_seconds.  Runs on the
 * calling thread; pcs handles must not be used elsewhere meanwhile.
 */
int pcs_run_load(pcs_handle* const* pools, const int* pool_block, int n_pools, int n_req, const double* arrival,
                 const int* pool_of, const int* channels, const long long* frames, const float* const* irs,
                 const int* ir_len, const int* num_levels, const int* N_flat, const int* P_flat, const float* noise,
                 long long noise_len, unsigned long long seed, int max_concurrent, double max_seconds, double fs,
                 pcs_load_stats* stats);

/* Size of the static device scratch array used by pc_convolve_noalloc. */
#define PC_NOALLOC_SCRATCH_BYTES (32 << 20)

/*
 * Convolution for callers that cannot allocate device memory.  No
 * counterpart in the reference: it exists for hosts that own every device
 * allocation themselves -- a plug-in inside an application that accounts
 * for all GPU memory, code under a memory pool or allocator that forbids
 * cudaMalloc, or a real-time thread that must never block in the driver's
 * allocator.
 *
 * Computes y[n] = sum_k h[k] x[n-k] for 0 <= n < n_frames from zero initial
 * state, with the uniformly partitioned frequency-domain delay line of block
 * size block_size (one level, ceil(h_len / block_size) parts); the result
 * equals n_frames / block_size pc_run calls of a fresh handle set up with
 * that layout.  d_x (n_frames samples), d_h (h_len taps) and d_y (n_frames
 * samples) are device pointers owned by the caller; enqueued on `stream`
 * (NULL = default stream), returns after enqueueing.
 *
 * All other working memory (twiddles, filter spectra, spectrum ring, partial
 * sums, input ring, task table) is one file-scope device array of
 * PC_NOALLOC_SCRATCH_BYTES (32 MiB) that every GPU loading this library
 * holds until the process exits; the call allocates and frees nothing.  With
 * P = ceil(h_len / block_size) parts and N = block_size, a call needs
 *     262144 + 16 (N + 2)(P + 1) + 32 P + 192 (1 + ceil((N + 2) / 128)) + 8 N
 * bytes, plus at most 2.5 KiB of 256-byte alignment: about 20 bytes per tap
 * at N = 16 (IRs up to ~1.66 M taps) and 16 bytes per tap at N = 1024 (up to
 * ~2.07 M taps).  A layout needing more fails with PC_ERR_LIMIT and a message
 * from pc_last_error(NULL).  block_size: a power of two in [16, 1024].
 *
 * The first call on a device (that device current) resolves the array's
 * device address with cudaGetSymbolAddress and writes the twiddle table into
 * it with a synchronous copy; make that first call before any stream
 * capture.  Every call after it writes its tables with a kernel and reads no
 * host memory, so it does not wait for earlier work on the stream.  Every
 * call reuses the same array and clears the state it needs, so calls that
 * overlap on the GPU (different streams, or different host threads on one
 * device) race; serialise them.
 */
int pc_convolve_noalloc(const float* d_x, long long n_frames, const float* d_h, int h_len, float* d_y,
                        int block_size, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PARTCONV_GB300_H */
