/*
 * partconvMulti.h -- C++ drop-in for the reference's PartConvMulti /
 * PartConvMultiRelaxed / Waiter (src/partconvMulti.h:52-165 of
 * ebattenberg/partconv), implemented over the C ABI in partconv_gb300.h.
 *
 * Same constructor, methods and public fields.  Differences, all on error
 * paths: where the reference calls exit(-1) (unreadable config, frameCount
 * != buffer_size) the methods return a non-zero PC_ERR_* code and
 * lastError() explains it.  Link with libpartconv_gb300.so.
 */
#ifndef PARTCONV_GB300_PARTCONVMULTI_H
#define PARTCONV_GB300_PARTCONVMULTI_H

#include <condition_variable>
#include <mutex>
#include <vector>

#include "partconv_gb300.h"

/* src/partconvMulti.h:152-165 */
class Waiter {
   public:
    explicit Waiter(int inVal = 0) : val(inVal), initVal(inVal) {}
    void waitFor(int target) {
        std::unique_lock<std::mutex> lk(mutex);
        cond.wait(lk, [&] { return val == target; });
    }
    void changeAndSignal(int newVal) {
        {
            std::lock_guard<std::mutex> lk(mutex);
            val = newVal;
        }
        cond.notify_all();
    }

   private:
    std::condition_variable cond;
    std::mutex mutex;
    int val;
    int initVal;
};

/* src/partconvMulti.h:52-140 */
class PartConvMulti {
   public:
    explicit PartConvMulti(int inVerbosity = 0) : verbosity(inVerbosity) { h = pc_create(inVerbosity); }
    virtual ~PartConvMulti() { pc_destroy(h); }
    PartConvMulti(const PartConvMulti&) = delete;
    PartConvMulti& operator=(const PartConvMulti&) = delete;

    int setup(const char* config_file_name, int max_threads_per_level = 1, int max_level0_threads = 0,
              double min_work = 0) {
        int r = pc_setup_config(h, config_file_name, max_threads_per_level, max_level0_threads, min_work);
        if (r == PC_OK) r = after_setup();
        return r;
    }
    /* programmatic setup (no config file); see pc_setup_layout */
    int setup_layout(int fs, int buffer_size, int n_in, int n_out, int num_pcs, const int* num_levels,
                     const int* block_sizes, const int* num_parts, const float* const* irs, const int* ir_lens,
                     const int* in_ch, const int* out_ch, const float* scale, const int* mute) {
        int r = pc_setup_layout(h, fs, buffer_size, n_in, n_out, num_pcs, num_levels, block_sizes, num_parts, irs,
                                ir_lens, in_ch, out_ch, scale, mute);
        if (r == PC_OK) r = after_setup();
        return r;
    }
    int cleanup() { return pc_cleanup(h); }
    virtual int run(float* const output, const float* const input, const int frameCount) {
        int r = pc_run(h, output, input, frameCount);
        if (r == PC_OK) {
            frameNum++;
            if (frameNum == lastFrame && doneWaiter != nullptr) doneWaiter->changeAndSignal(1);
        }
        return r;
    }
    void reset() {
        pc_reset(h);
        frameNum = 0;
    }
    const char* lastError() const { return pc_last_error(h); }
    pc_handle* handle() const { return h; }

    float* output_mix = nullptr;
    float* input_mix = nullptr;
    int FS = 0;
    int buffer_size = 0;
    int max_block_size = 0;
    int verbosity = 0;
    int numInputChannels = 0;
    int numOutputChannels = 0;
    unsigned long frameNum = 0;
    Waiter* doneWaiter = nullptr;
    unsigned long lastFrame = 0;

   protected:
    virtual int relaxedMode() const { return 0; }
    int after_setup() {
        int r = pc_set_relaxed(h, relaxedMode());
        if (r != PC_OK) return r;
        pc_info inf;
        r = pc_get_info(h, &inf);
        if (r != PC_OK) return r;
        FS = inf.fs;
        buffer_size = inf.buffer_size;
        max_block_size = inf.max_block_size;
        numInputChannels = inf.num_input_channels;
        numOutputChannels = inf.num_output_channels;
        mix_out.assign((size_t)buffer_size * numOutputChannels, 0.0f);
        mix_in.assign((size_t)buffer_size * numInputChannels, 0.0f);
        output_mix = mix_out.data();
        input_mix = mix_in.data();
        frameNum = 0;
        return PC_OK;
    }
    pc_handle* h = nullptr;
    std::vector<float> mix_out, mix_in;
};

/* src/partconvMulti.h:142-148: output one buffer_size block later */
class PartConvMultiRelaxed : public PartConvMulti {
   public:
    explicit PartConvMultiRelaxed(int inVerbosity = 0) : PartConvMulti(inVerbosity) {}

   protected:
    int relaxedMode() const override { return 1; }
};

#endif /* PARTCONV_GB300_PARTCONVMULTI_H */
