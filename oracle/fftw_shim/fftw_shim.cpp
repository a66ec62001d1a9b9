// fftw_shim.cpp -- the FFTW3 stand-in declared in fftw3.h (test
// infrastructure only), on the oracle's float32 transform.
#include "fftw3.h"

#include <cstdlib>
#include <vector>

#include "../orc_fft.h"

struct orc_fftwf_plan_s {
    int n = 0;
    bool r2c = true;
    float* rin = nullptr;           // r2c input / c2r output (n floats)
    float* cbuf = nullptr;          // r2c output / c2r input (n/2 + 1 complex)
    orc::RealFFT fft;
    std::vector<float> tmp;         // c2r: a copy of the bins, FFTW's c2r may overwrite them
};

static fftwf_plan make(int n, bool r2c, float* r, float* c) {
    if (n < 2 || !orc::is_pow2(n)) return nullptr;   // the reference only plans powers of two
    auto* p = new orc_fftwf_plan_s();
    p->n = n;
    p->r2c = r2c;
    p->rin = r;
    p->cbuf = c;
    p->fft.init(n);
    p->tmp.resize((size_t)(n + 2));
    return p;
}

extern "C" {

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned) {
    return make(n, true, in, reinterpret_cast<float*>(out));
}

fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex* in, float* out, unsigned) {
    return make(n, false, out, reinterpret_cast<float*>(in));
}

void fftwf_execute(const fftwf_plan p) {
    if (!p) return;
    if (p->r2c) {
        p->fft.forward(p->rin, p->cbuf);
    } else {
        for (int j = 0; j < p->n + 2; ++j) p->tmp[j] = p->cbuf[j];
        p->fft.inverse(p->tmp.data(), p->rin);
    }
}

void fftwf_destroy_plan(fftwf_plan p) { delete p; }

void* fftwf_malloc(size_t n) {
    void* q = nullptr;
    if (posix_memalign(&q, 64, n ? n : 64) != 0) return nullptr;
    return q;
}

void fftwf_free(void* p) { std::free(p); }

int fftwf_import_wisdom_from_file(FILE*) { return 1; }
void fftwf_export_wisdom_to_file(FILE*) {}

}  // extern "C"
