// ref_driver.cpp -- runs the reference's own PartConvFilter (compiled from
// the reference's src/partconv.cpp and src/buffers.cpp against the FFTW
// stand-in in fftw_shim/) through the callback sequence of
// PartConvMulti::run, so the oracle can be checked against the reference's
// code.  TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by
// oracle/Makefile.ref where the reference sources are present (an x86_64
// host: partconv.cpp's MAC is SSE3), used by CPU tests and by the script that
// writes tests/golden/ref_golden.npz.
//
// Per callback and PC, as src/partconvMulti.cpp:815-928 orders it:
//   input_mix = input[chan] * scale                       (:839-847)
//   sync_levels(); input(input_mix)                       (:850-859)
//   runLevel(L) for L = 0 .. start_sync_depth             (:862-888; the level
//       workers' blocks run at once here, which gives the same result: a
//       level's block reads only the DelayBuffer block prepNextRead fixed and
//       is read back only after the swap at end_sync_depth)
//   output(output_mix)                                    (:908-909)
//   output[out_chan] += output_mix unless muted, PCs in order (:911-921)
// and for PartConvMultiRelaxed (src/partconvMulti.cpp:1017-1134):
//   sync_levels_relaxed(); output_relaxed(output_mix); input(input_mix);
//   runLevel(L) for L = 0 .. sync_depth; mix.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "partconv.h"

namespace {

struct RefPC {
    PartConvFilter f;
    std::vector<int> cnt, per;   // callback counters per level, as sync_levels keeps them
    int M = 0;
};

struct RefMulti {
    int buffer_size = 0, n_in = 0, n_out = 0, relaxed = 0;
    std::vector<std::unique_ptr<RefPC>> pc;
    std::vector<int> in_ch, out_ch, mute;
    std::vector<float> scale;

    ~RefMulti() {
        for (auto& p : pc) {
            delete[] p->f.output_mix;
            delete[] p->f.input_mix;
            p->f.cleanup();
        }
    }

    // deepest level whose block starts at this callback (PartConvFilter keeps
    // the same counters privately: ind_N0_in_level, src/partconv.cpp:568-586)
    static int start_depth(RefPC& p) {
        int d = 0;
        for (int L = 0; L < p.M; ++L) {
            if (++p.cnt[L] == p.per[L]) {
                p.cnt[L] = 0;
                d = L;
            }
        }
        return d;
    }

    void run(float* out, const float* in) {
        const int F = buffer_size, npc = (int)pc.size();
        std::memset(out, 0, sizeof(float) * (size_t)n_out * F);
        for (int i = 0; i < npc; ++i) {
            RefPC& p = *pc[i];
            for (int j = 0; j < F; ++j) p.f.input_mix[j] = in[in_ch[i] + j * n_in] * scale[i];
            const int depth = start_depth(p);
            if (!relaxed) {
                p.f.sync_levels();
                p.f.input(p.f.input_mix);
                for (int L = 0; L <= depth; ++L) p.f.runLevel(L);
                p.f.output(p.f.output_mix);
            } else {
                p.f.sync_levels_relaxed();
                p.f.output_relaxed(p.f.output_mix);
                p.f.input(p.f.input_mix);
                for (int L = 0; L <= depth; ++L) p.f.runLevel(L);
            }
            if (!mute[i])
                for (int j = 0; j < F; ++j) out[out_ch[i] + j * n_out] += p.f.output_mix[j];
        }
    }
};

void put_msg(char* dst, int len, const std::string& s) {
    if (dst && len > 0) std::snprintf(dst, (size_t)len, "%s", s.c_str());
}

}  // namespace

extern "C" {

// PartConvFilter::setup's verdict on a layout (src/partconv.cpp:70-181):
// 0 and P[M-1] filled in, or 1 where the reference rejects it.
int ref_layout_check(int M, const int* N, int* P, int ir_len) {
    PartConvFilter f;
    Vector h(ir_len);
    for (int i = 0; i < ir_len; ++i) h[i] = 0.0f;
    std::vector<int> Nv(N, N + M), Pv(P, P + M);
    int r = f.setup(M, Nv.data(), Pv.data(), &h, 0, nullptr);
    if (r == 0) {
        P[M - 1] = f.num_parts[M - 1];
        delete[] f.output_mix;
        delete[] f.input_mix;
        f.cleanup();
    }
    return r;
}

// Same arguments as the oracle's orc_multi_create (without its schedule
// choice): every PC runs the reference's own PartConvFilter.  NULL when the
// reference's setup rejects a PC's layout.
void* ref_multi_create(int buffer_size, int n_in, int n_out, int num_pcs, const int* M, const int* N_flat,
                       const int* P_flat, const float* const* irs, const int* ir_lens, const int* in_ch,
                       const int* out_ch, const float* scale, const int* mute, int relaxed_variant, char* msg,
                       int msglen) {
    auto m = std::make_unique<RefMulti>();
    m->buffer_size = buffer_size;
    m->n_in = n_in;
    m->n_out = n_out;
    m->relaxed = relaxed_variant;
    int off = 0;
    for (int i = 0; i < num_pcs; ++i) {
        auto p = std::make_unique<RefPC>();
        p->M = M[i];
        std::vector<int> Nv(N_flat + off, N_flat + off + M[i]), Pv(P_flat + off, P_flat + off + M[i]);
        if (Nv[0] != buffer_size) {
            put_msg(msg, msglen, "PC " + std::to_string(i) + ": first block size must equal buffer_size");
            return nullptr;
        }
        Vector h(ir_lens[i]);
        h.copyFrom(const_cast<float*>(irs[i]));
        if (p->f.setup(M[i], Nv.data(), Pv.data(), &h, 0, nullptr) != 0) {
            put_msg(msg, msglen, "PC " + std::to_string(i) + ": PartConvFilter::setup rejected the layout");
            return nullptr;
        }
        for (int L = 0; L < M[i]; ++L) {
            p->per.push_back(Nv[L] / Nv[0]);
            p->cnt.push_back(Nv[L] / Nv[0] - 1);   // as PartConvFilter::setup initialises them
        }
        m->pc.push_back(std::move(p));
        off += M[i];
    }
    m->in_ch.assign(in_ch, in_ch + num_pcs);
    m->out_ch.assign(out_ch, out_ch + num_pcs);
    m->scale.assign(scale, scale + num_pcs);
    m->mute.assign(mute, mute + num_pcs);
    put_msg(msg, msglen, "");
    return m.release();
}

// frames/buffer_size callbacks of interleaved input and output
int ref_multi_run(void* h, float* out, const float* in, long frames) {
    auto* m = static_cast<RefMulti*>(h);
    if (frames % m->buffer_size) return 1;
    const long nb = frames / m->buffer_size;
    for (long b = 0; b < nb; ++b)
        m->run(out + b * m->buffer_size * (long)m->n_out, in + b * m->buffer_size * (long)m->n_in);
    return 0;
}

// PartConvMulti::reset (src/partconvMulti.cpp:806-813): PartConvFilter::reset
// on every PC, and the callback counters back to their set-up values
void ref_multi_reset(void* h) {
    auto* m = static_cast<RefMulti*>(h);
    for (auto& p : m->pc) {
        p->f.reset();
        for (int L = 0; L < p->M; ++L) p->cnt[L] = p->per[L] - 1;
    }
}

void ref_multi_destroy(void* h) { delete static_cast<RefMulti*>(h); }

}  // extern "C"
