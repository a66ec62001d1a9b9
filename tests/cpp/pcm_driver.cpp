// Drives the C++ PartConvMulti drop-in (include/partconvMulti.h) the way an
// audio callback would: setup from a pc.config, then run() once per
// buffer_size frames.  Usage: pcm_driver CONFIG IN.f32 OUT.f32 [relaxed]
// IN.f32 / OUT.f32 are raw interleaved float32 [frames][channels].
// Exit status: 0 ok, 10 + PC_ERR_* code of a failing setup, 30 + code of a failing run.
#include <cstdio>
#include <vector>

#include "partconvMulti.h"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s CONFIG IN.f32 OUT.f32 [relaxed]\n", argv[0]);
        return 2;
    }
    const bool relaxed = argc > 4 && argv[4][0] == '1';
    PartConvMulti plain(0);
    PartConvMultiRelaxed relax(0);
    PartConvMulti& pc = relaxed ? static_cast<PartConvMulti&>(relax) : plain;
    int r = pc.setup(argv[1], 1, 0, 0.0);
    if (r != PC_OK) {
        std::fprintf(stderr, "setup failed (%d): %s\n", r, pc.lastError());
        return 10 + r;
    }
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    std::vector<float> in;
    float buf[4096];
    size_t n;
    while ((n = std::fread(buf, sizeof(float), 4096, f)) > 0) in.insert(in.end(), buf, buf + n);
    std::fclose(f);
    const size_t step_in = (size_t)pc.buffer_size * pc.numInputChannels;
    const size_t step_out = (size_t)pc.buffer_size * pc.numOutputChannels;
    const size_t steps = in.size() / step_in;
    std::vector<float> out(steps * step_out, 0.0f);
    Waiter done(0);
    pc.doneWaiter = &done;
    pc.lastFrame = steps;
    for (size_t s = 0; s < steps; ++s) {
        r = pc.run(out.data() + s * step_out, in.data() + s * step_in, pc.buffer_size);
        if (r != PC_OK) {
            std::fprintf(stderr, "run failed (%d): %s\n", r, pc.lastError());
            return 30 + r;
        }
    }
    done.waitFor(1);   // signalled by run() at lastFrame
    r = pc.run(out.data(), in.data(), pc.buffer_size + 1);   // wrong frame count: an error, not an exit
    if (r != PC_ERR_ARG) return 4;
    f = std::fopen(argv[3], "wb");
    if (!f) return 5;
    std::fwrite(out.data(), sizeof(float), out.size(), f);
    std::fclose(f);
    std::printf("ok %zu steps, frameNum %lu\n", steps, pc.frameNum);
    return pc.cleanup();
}
