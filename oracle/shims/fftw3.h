/* Shim of the FFTW 3.3.x single-precision API used by the Meraxes
 * reionization sources, for building them as a test oracle only.
 * Transforms are executed by the oracle's own FFT (mx_numerics.c). */
#ifndef MXS_FFTW3_H
#define MXS_FFTW3_H
#include <complex.h>
#include <stddef.h>
typedef float _Complex fftwf_complex;
typedef struct mxs_fftwf_plan_s* fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)
#define FFTW_MEASURE (0U)
float* fftwf_alloc_real(size_t n);
fftwf_complex* fftwf_alloc_complex(size_t n);
void fftwf_free(void* p);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
int fftwf_import_wisdom_from_filename(const char* f);
int fftwf_export_wisdom_to_filename(const char* f);
#endif
