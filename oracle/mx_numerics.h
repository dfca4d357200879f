/*
 * Oracle numerics — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatements of the third-party numerical routines that the Meraxes
 * reionization step calls but that are not part of the Meraxes tree:
 *
 *   - FFTW 3.3.x single-precision r2c/c2r 3-D transforms (unnormalised,
 *     FFTW sign convention, FFTW in-place padded real layout).  Restated from
 *     the DFT definition as a mixed-radix Cooley-Tukey FFT computed in double
 *     precision and rounded to float on output.
 *   - GSL natural cubic spline (gsl_interp_cspline), restated from the
 *     standard tridiagonal second-derivative construction.
 *   - GSL gsl_integration_qag with the 61-point Gauss-Kronrod rule: the
 *     QUADPACK QAG adaptive bisection algorithm (Piessens, de Doncker-Kapenga,
 *     Ueberhuber & Kahaner 1983).
 *   - GSL Brent root bracketing solver and gsl_root_test_interval (Brent 1973).
 *
 * Only tests, the smoke check and the CPU baseline of the benchmark use this
 * code; the product library never links it.
 */
#ifndef MX_NUMERICS_H
#define MX_NUMERICS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- FFT ---- */
/* Forward real-to-complex 3-D transform of a D^3 real grid.
 * in:  real values, padded layout ([D][D][2(D/2+1)]) if in_padded != 0, else
 *      the unpadded [D][D][D] layout.
 * out: interleaved float complex [D][D][D/2+1] (FFTW r2c output layout).
 * Unnormalised, exp(-2 pi i jk/n) kernel.  in and out may alias (in-place). */
void mxo_r2c_3d(int D, const float* in, int in_padded, float* out);

/* Backward complex-to-real 3-D transform (FFTW c2r semantics: the imaginary
 * parts of the kz = 0 and kz = D/2 terms are ignored along the last axis).
 * in:  interleaved float complex [D][D][D/2+1].
 * out: padded real layout [D][D][2(D/2+1)]; may alias in (in-place).
 * Unnormalised, exp(+2 pi i jk/n) kernel. */
void mxo_c2r_3d(int D, const float* in, float* out);

/* 1-D complex FFT of length n (any n with factors 2,3,5,7 or general),
 * computed in double.  data is interleaved re/im, contiguous. sign = -1
 * forward, +1 backward.  Unnormalised. */
void mxo_fft_1d(double* data, int n, int sign);

/* ------------------------------------------------------------- spline ---- */
typedef struct mxo_spline
{
  int n;
  double* x;
  double* y;
  double* c; /* second-derivative / 2 coefficients, natural end conditions */
} mxo_spline;

int mxo_spline_init(mxo_spline* s, const double* x, const double* y, int n);
void mxo_spline_free(mxo_spline* s);
/* Returns NaN outside [x[0], x[n-1]] (GSL reports a domain error there). */
double mxo_spline_eval(const mxo_spline* s, double x);

/* ---------------------------------------------------------------- QAG ---- */
typedef double (*mxo_fn)(double x, void* params);

/* QUADPACK QAG with the 61-point Gauss-Kronrod rule.  Returns 0 on
 * convergence, a positive code otherwise (result still set, as GSL does). */
int mxo_qag61(mxo_fn f,
              void* params,
              double a,
              double b,
              double epsabs,
              double epsrel,
              size_t limit,
              double* result,
              double* abserr);

/* -------------------------------------------------------------- Brent ---- */
typedef struct mxo_brent
{
  mxo_fn f;
  void* params;
  double root, x_lower, x_upper;
  double a, b, c, d, e, fa, fb, fc;
} mxo_brent;

int mxo_brent_set(mxo_brent* s, mxo_fn f, void* params, double x_lower, double x_upper);
int mxo_brent_iterate(mxo_brent* s);
/* 0 = converged, 1 = continue (gsl_root_test_interval semantics). */
int mxo_root_test_interval(double x_lower, double x_upper, double epsabs, double epsrel);

#ifdef __cplusplus
}
#endif

#endif
