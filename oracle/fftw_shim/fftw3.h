/*
 * fftw3.h -- a stand-in for the single-precision FFTW3 interface, just wide
 * enough for the reference's partconv.cpp and buffers.cpp to compile and run
 * here (test infrastructure only: it exists so the oracle can be checked
 * against the reference's own code).
 *
 * FFTW 3 (fftw-3.2.2, the version named in the reference's src/wisdom.wis:1)
 * is not in this image.  The reference calls (src/partconv.cpp:219-222,
 * :259-285, :313-314, :363, :482; src/buffers.cpp:25-31, :69-109) are served
 * by the oracle's own float32 transform (orc_fft.h):
 *   fftwf_plan_dft_r2c_1d  n real samples -> n/2 + 1 bins, unnormalised
 *   fftwf_plan_dft_c2r_1d  n/2 + 1 bins -> n real samples, unnormalised,
 *                          imaginary parts of DC and Nyquist ignored
 *   fftwf_execute / fftwf_destroy_plan
 *   fftwf_malloc / fftwf_free   (64-byte aligned, as SSE loads need 16)
 *   fftwf_import/export_wisdom_from/to_file   accepted, no effect
 * Planner flags are accepted and ignored: there is one algorithm.
 */
#ifndef ORC_FFTW3_SHIM_H
#define ORC_FFTW3_SHIM_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct orc_fftwf_plan_s* fftwf_plan;

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex* in, float* out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);
int fftwf_import_wisdom_from_file(FILE* f);
void fftwf_export_wisdom_to_file(FILE* f);

#ifdef __cplusplus
}
#endif

#endif /* ORC_FFTW3_SHIM_H */
