/*
 * Oracle numerics — TEST INFRASTRUCTURE ONLY (see mx_numerics.h).
 *
 * Third-party algorithms restated here because the libraries are absent:
 *   FFTW 3.3.x (the reference calls it at src/core/reionization.c:685-901 and
 *     executes it at src/core/find_HII_bubbles.c:124-269, ComputeTs.c:379-409,
 *     BrightnessTemperature.c:201,215);
 *   GSL cspline / qag(GAUSS61) / brent (called at
 *     src/core/XRayHeatingFunctions.c:142-144, 255-292, 371, 783-792 and
 *     src/core/recombinations.c:79-81, 154, 184).
 */
#include "mx_numerics.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ====================================================================== FFT */

typedef struct fft_plan_t
{
  int n;
  int nf;
  int f[40];
  double* tw; /* tw[2j], tw[2j+1] = cos, sin of 2 pi j / n */
} fft_plan_t;

#define MXO_MAX_PLANS 16
static fft_plan_t g_plans[MXO_MAX_PLANS];
static int g_nplans = 0;

static const fft_plan_t* get_plan(int n)
{
  for (int i = 0; i < g_nplans; i++)
    if (g_plans[i].n == n)
      return &g_plans[i];
  fft_plan_t* p;
  if (g_nplans < MXO_MAX_PLANS) {
    p = &g_plans[g_nplans++];
  } else {
    p = &g_plans[0];
    free(p->tw);
  }
  p->n = n;
  p->nf = 0;
  int m = n;
  static const int pref[] = { 4, 2, 3, 5, 7 };
  for (int k = 0; k < 5 && m > 1; k++) {
    while (m % pref[k] == 0) {
      p->f[p->nf++] = pref[k];
      m /= pref[k];
    }
  }
  for (int q = 11; m > 1; q += 2) {
    while (m % q == 0) {
      p->f[p->nf++] = q;
      m /= q;
    }
  }
  p->tw = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
  for (int j = 0; j < n; j++) {
    double ang = 2.0 * M_PI * (double)j / (double)n;
    p->tw[2 * j] = cos(ang);
    p->tw[2 * j + 1] = sin(ang);
  }
  return p;
}

/* Recursive decimation-in-time, out-of-place into `out` (contiguous). */
static void fft_rec(const double* in,
                    double* out,
                    int n,
                    int is,
                    int sign,
                    const fft_plan_t* P,
                    int level,
                    int twstride)
{
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  const int p = P->f[level];
  const int m = n / p;
  for (int r = 0; r < p; r++)
    fft_rec(in + 2 * (size_t)r * is, out + 2 * (size_t)r * m, m, is * p, sign, P, level + 1, twstride * p);

  const int N = P->n;
  double tre[64], tim[64];
  double* bre = tre;
  double* bim = tim;
  double* heap = NULL;
  if (p > 64) {
    heap = (double*)malloc(sizeof(double) * 2 * (size_t)p);
    bre = heap;
    bim = heap + p;
  }
  for (int k = 0; k < m; k++) {
    for (int r = 0; r < p; r++) {
      double yr = out[2 * ((size_t)r * m + k)];
      double yi = out[2 * ((size_t)r * m + k) + 1];
      long idx = ((long)r * k % n) * (long)twstride % N;
      double c = P->tw[2 * idx];
      double s = sign * P->tw[2 * idx + 1];
      bre[r] = yr * c - yi * s;
      bim[r] = yr * s + yi * c;
    }
    for (int q = 0; q < p; q++) {
      double sr = 0.0, si = 0.0;
      for (int r = 0; r < p; r++) {
        long idx = ((long)r * q % p) * (long)m * twstride % N;
        double c = P->tw[2 * idx];
        double s = sign * P->tw[2 * idx + 1];
        sr += bre[r] * c - bim[r] * s;
        si += bre[r] * s + bim[r] * c;
      }
      out[2 * ((size_t)k + (size_t)q * m)] = sr;
      out[2 * ((size_t)k + (size_t)q * m) + 1] = si;
    }
  }
  free(heap);
}

void mxo_fft_1d(double* data, int n, int sign)
{
  if (n <= 1)
    return;
  const fft_plan_t* P = get_plan(n);
  double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  fft_rec(data, tmp, n, 1, sign, P, 0, 1);
  memcpy(data, tmp, sizeof(double) * 2 * (size_t)n);
  free(tmp);
}

/* ------------------------------------------- 3-D transforms (FFTW layout)
 *
 * The work array of a 3-D transform holds the half spectrum [D][D][H]
 * (H = D/2 + 1) as interleaved complex values of type fft_real: double by
 * default, float when the library is compiled with MXO_FFT_SINGLE (the
 * precision of the reference's fftwf calls; that build only serves CPU
 * timing).
 *
 * Power-of-two lengths run a batched Stockham autosort FFT (radix-4 stages,
 * one radix-2 stage when log2 n is odd): up to FFT_BATCH lines at a time are
 * gathered into a buffer [n][B] whose batch index is fastest, so every
 * butterfly is a short unit-stride loop over the batch.  Stockham's
 * decimation in frequency, for a stage of length L and stride s (L s = n),
 * maps x[q + s (p + r L/4)], r = 0..3, to y[q + s (4p + t)] with the
 * twiddle w_L^{p t}; the next stage has length L/4 and stride 4s.  Other
 * lengths use mxo_fft_1d line by line.  Lines are independent and spread
 * over OpenMP threads; no line's arithmetic depends on the thread count. */
#ifdef MXO_FFT_SINGLE
typedef float fft_real;
#else
typedef double fft_real;
#endif

#define FFT_BATCH 16

typedef struct p2_plan
{
  int n;
  fft_real* tw; /* tw[2j], tw[2j+1] = cos, sin of 2 pi j / n */
} p2_plan;

static p2_plan g_p2[MXO_MAX_PLANS];
static int g_np2 = 0;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* Not thread-safe: called before the parallel regions. */
static const p2_plan* get_p2(int n)
{
  for (int i = 0; i < g_np2; i++)
    if (g_p2[i].n == n)
      return &g_p2[i];
  p2_plan* p;
  if (g_np2 < MXO_MAX_PLANS) {
    p = &g_p2[g_np2++];
  } else {
    p = &g_p2[0];
    free(p->tw);
  }
  p->n = n;
  p->tw = (fft_real*)malloc(sizeof(fft_real) * 2 * (size_t)n);
  for (int j = 0; j < n; j++) {
    const double ang = 2.0 * M_PI * (double)j / (double)n;
    p->tw[2 * j] = (fft_real)cos(ang);
    p->tw[2 * j + 1] = (fft_real)sin(ang);
  }
  return p;
}

/* B transforms of length n = P->n held in x as [n][B] (element (i, b) at
 * x[2 (i B + b)]); y is scratch of the same size.  The result is left in x.
 * sign = -1 forward, +1 backward; unnormalised. */
static void p2_fft_batch(fft_real* x, fft_real* y, int B, int sign, const p2_plan* P)
{
  const int n = P->n;
  const fft_real sg = (fft_real)sign;
  fft_real* src = x;
  fft_real* dst = y;
  int s = 1;
  for (int len = n; len > 1; len /= (len % 4 == 0 ? 4 : 2)) {
    const int step = n / len; /* w_len^p = tw[p * step] */
    if (len % 4 == 0) {
      const int m = len / 4;
      for (int p = 0; p < m; p++) {
        const fft_real* t1 = P->tw + 2 * (size_t)p * step;
        const fft_real* t2 = P->tw + 4 * (size_t)p * step;
        const fft_real* t3 = P->tw + 6 * (size_t)p * step;
        const fft_real w1r = t1[0], w1i = sg * t1[1];
        const fft_real w2r = t2[0], w2i = sg * t2[1];
        const fft_real w3r = t3[0], w3i = sg * t3[1];
        for (int q = 0; q < s; q++) {
          const fft_real* a = src + 2 * (size_t)(q + s * p) * B;
          const fft_real* b = src + 2 * (size_t)(q + s * (p + m)) * B;
          const fft_real* c = src + 2 * (size_t)(q + s * (p + 2 * m)) * B;
          const fft_real* d = src + 2 * (size_t)(q + s * (p + 3 * m)) * B;
          fft_real* o0 = dst + 2 * (size_t)(q + s * (4 * p)) * B;
          fft_real* o1 = o0 + 2 * (size_t)s * B;
          fft_real* o2 = o1 + 2 * (size_t)s * B;
          fft_real* o3 = o2 + 2 * (size_t)s * B;
          for (int j = 0; j < B; j++) {
            const fft_real apcr = a[2 * j] + c[2 * j], apci = a[2 * j + 1] + c[2 * j + 1];
            const fft_real amcr = a[2 * j] - c[2 * j], amci = a[2 * j + 1] - c[2 * j + 1];
            const fft_real bpdr = b[2 * j] + d[2 * j], bpdi = b[2 * j + 1] + d[2 * j + 1];
            /* sign * i * (b - d) */
            const fft_real jr = -sg * (b[2 * j + 1] - d[2 * j + 1]), ji = sg * (b[2 * j] - d[2 * j]);
            o0[2 * j] = apcr + bpdr;
            o0[2 * j + 1] = apci + bpdi;
            const fft_real y1r = amcr + jr, y1i = amci + ji;
            const fft_real y2r = apcr - bpdr, y2i = apci - bpdi;
            const fft_real y3r = amcr - jr, y3i = amci - ji;
            o1[2 * j] = y1r * w1r - y1i * w1i;
            o1[2 * j + 1] = y1r * w1i + y1i * w1r;
            o2[2 * j] = y2r * w2r - y2i * w2i;
            o2[2 * j + 1] = y2r * w2i + y2i * w2r;
            o3[2 * j] = y3r * w3r - y3i * w3i;
            o3[2 * j + 1] = y3r * w3i + y3i * w3r;
          }
        }
      }
      s *= 4;
    } else { /* len == 2 */
      for (int q = 0; q < s; q++) {
        const fft_real* a = src + 2 * (size_t)q * B;
        const fft_real* b = src + 2 * (size_t)(q + s) * B;
        fft_real* o0 = dst + 2 * (size_t)q * B;
        fft_real* o1 = dst + 2 * (size_t)(q + s) * B;
        for (int j = 0; j < 2 * B; j++) {
          const fft_real u = a[j], v = b[j];
          o0[j] = u + v;
          o1[j] = u - v;
        }
      }
      s *= 2;
    }
    fft_real* t = src;
    src = dst;
    dst = t;
  }
  if (src != x)
    memcpy(x, src, sizeof(fft_real) * 2 * (size_t)n * B);
}

/* Complex transforms of the half spectrum w along x (axis 0) or y (axis 1). */
static void transform_axis(fft_real* w, int D, int H, int axis, int sign)
{
  if (is_pow2(D)) {
    const p2_plan* P = get_p2(D);
    const int nkb = (H + FFT_BATCH - 1) / FFT_BATCH;
#pragma omp parallel
    {
      fft_real* buf = (fft_real*)malloc(sizeof(fft_real) * 4 * (size_t)D * FFT_BATCH);
      fft_real* tmp = buf + 2 * (size_t)D * FFT_BATCH;
#pragma omp for schedule(static)
      for (long q = 0; q < (long)D * nkb; q++) {
        const int a = (int)(q / nkb), kz0 = (int)(q % nkb) * FFT_BATCH;
        const int B = H - kz0 < FFT_BATCH ? H - kz0 : FFT_BATCH;
        for (int t = 0; t < D; t++) {
          const size_t i = (axis == 0 ? ((size_t)t * D + a) : ((size_t)a * D + t)) * H + kz0;
          memcpy(buf + 2 * (size_t)t * B, w + 2 * i, sizeof(fft_real) * 2 * (size_t)B);
        }
        p2_fft_batch(buf, tmp, B, sign, P);
        for (int t = 0; t < D; t++) {
          const size_t i = (axis == 0 ? ((size_t)t * D + a) : ((size_t)a * D + t)) * H + kz0;
          memcpy(w + 2 * i, buf + 2 * (size_t)t * B, sizeof(fft_real) * 2 * (size_t)B);
        }
      }
      free(buf);
    }
    return;
  }
  (void)get_plan(D); /* create the shared plan before the parallel region */
#pragma omp parallel
  {
    double* line = (double*)malloc(sizeof(double) * 2 * (size_t)D);
#pragma omp for schedule(static)
    for (long q = 0; q < (long)D * H; q++) {
      const int a = (int)(q / H), kz = (int)(q % H);
      for (int t = 0; t < D; t++) {
        const size_t i = (axis == 0 ? ((size_t)t * D + a) : ((size_t)a * D + t)) * H + kz;
        line[2 * t] = w[2 * i];
        line[2 * t + 1] = w[2 * i + 1];
      }
      mxo_fft_1d(line, D, sign);
      for (int t = 0; t < D; t++) {
        const size_t i = (axis == 0 ? ((size_t)t * D + a) : ((size_t)a * D + t)) * H + kz;
        w[2 * i] = (fft_real)line[2 * t];
        w[2 * i + 1] = (fft_real)line[2 * t + 1];
      }
    }
    free(line);
  }
}

/* z: rows of D real values (row q at in + q * rstride) -> the first H
 * values of each row's forward DFT, into w */
static void r2c_rows(int D, const float* in, int rstride, fft_real* w)
{
  const int H = D / 2 + 1;
  const long rows = (long)D * D;
  if (is_pow2(D)) {
    const p2_plan* P = get_p2(D);
#pragma omp parallel
    {
      fft_real* buf = (fft_real*)malloc(sizeof(fft_real) * 4 * (size_t)D * FFT_BATCH);
      fft_real* tmp = buf + 2 * (size_t)D * FFT_BATCH;
#pragma omp for schedule(static)
      for (long q0 = 0; q0 < rows; q0 += FFT_BATCH) {
        const int B = rows - q0 < FFT_BATCH ? (int)(rows - q0) : FFT_BATCH;
        for (int b = 0; b < B; b++) {
          const float* src = in + (size_t)(q0 + b) * rstride;
          for (int z = 0; z < D; z++) {
            buf[2 * ((size_t)z * B + b)] = (fft_real)src[z];
            buf[2 * ((size_t)z * B + b) + 1] = 0;
          }
        }
        p2_fft_batch(buf, tmp, B, -1, P);
        for (int b = 0; b < B; b++) {
          fft_real* dst = w + 2 * (size_t)(q0 + b) * H;
          for (int k = 0; k < H; k++) {
            dst[2 * k] = buf[2 * ((size_t)k * B + b)];
            dst[2 * k + 1] = buf[2 * ((size_t)k * B + b) + 1];
          }
        }
      }
      free(buf);
    }
    return;
  }
  (void)get_plan(D);
#pragma omp parallel
  {
    double* line = (double*)malloc(sizeof(double) * 2 * (size_t)D);
#pragma omp for schedule(static)
    for (long q = 0; q < rows; q++) {
      const float* src = in + (size_t)q * rstride;
      for (int z = 0; z < D; z++) {
        line[2 * z] = (double)src[z];
        line[2 * z + 1] = 0.0;
      }
      mxo_fft_1d(line, D, -1);
      for (int k = 0; k < 2 * H; k++)
        w[2 * (size_t)q * H + k] = (fft_real)line[k];
    }
    free(line);
  }
}

/* z: half-complex rows of w -> real rows of out (padded, pitch 2H), with
 * the Hermitian extension and the imaginary parts of kz = 0 and kz = D/2
 * ignored (FFTW c2r semantics) */
static void c2r_rows(int D, const fft_real* w, float* out)
{
  const int H = D / 2 + 1;
  const long rows = (long)D * D;
  if (is_pow2(D)) {
    const p2_plan* P = get_p2(D);
#pragma omp parallel
    {
      fft_real* buf = (fft_real*)malloc(sizeof(fft_real) * 4 * (size_t)D * FFT_BATCH);
      fft_real* tmp = buf + 2 * (size_t)D * FFT_BATCH;
#pragma omp for schedule(static)
      for (long q0 = 0; q0 < rows; q0 += FFT_BATCH) {
        const int B = rows - q0 < FFT_BATCH ? (int)(rows - q0) : FFT_BATCH;
        for (int b = 0; b < B; b++) {
          const fft_real* src = w + 2 * (size_t)(q0 + b) * H;
          for (int k = 0; k < H; k++) {
            buf[2 * ((size_t)k * B + b)] = src[2 * k];
            buf[2 * ((size_t)k * B + b) + 1] = src[2 * k + 1];
          }
          buf[2 * (size_t)b + 1] = 0;
          buf[2 * ((size_t)(D / 2) * B + b) + 1] = 0;
          for (int k = H; k < D; k++) {
            buf[2 * ((size_t)k * B + b)] = src[2 * (D - k)];
            buf[2 * ((size_t)k * B + b) + 1] = -src[2 * (D - k) + 1];
          }
        }
        p2_fft_batch(buf, tmp, B, +1, P);
        for (int b = 0; b < B; b++) {
          float* dst = out + (size_t)(q0 + b) * 2 * H;
          for (int z = 0; z < D; z++)
            dst[z] = (float)buf[2 * ((size_t)z * B + b)];
          for (int z = D; z < 2 * H; z++)
            dst[z] = 0.0f;
        }
      }
      free(buf);
    }
    return;
  }
  (void)get_plan(D);
#pragma omp parallel
  {
    double* line = (double*)malloc(sizeof(double) * 2 * (size_t)D);
#pragma omp for schedule(static)
    for (long q = 0; q < rows; q++) {
      const fft_real* src = w + 2 * (size_t)q * H;
      for (int k = 0; k < H; k++) {
        line[2 * k] = src[2 * k];
        line[2 * k + 1] = src[2 * k + 1];
      }
      line[1] = 0.0;
      if (D % 2 == 0)
        line[2 * (D / 2) + 1] = 0.0;
      for (int k = H; k < D; k++) {
        line[2 * k] = src[2 * (D - k)];
        line[2 * k + 1] = -src[2 * (D - k) + 1];
      }
      mxo_fft_1d(line, D, +1);
      float* dst = out + (size_t)q * 2 * H;
      for (int z = 0; z < D; z++)
        dst[z] = (float)line[2 * z];
      for (int z = D; z < 2 * H; z++)
        dst[z] = 0.0f;
    }
    free(line);
  }
}

void mxo_r2c_3d(int D, const float* in, int in_padded, float* out)
{
  const int H = D / 2 + 1;
  const size_t nc = (size_t)D * D * H;
  fft_real* w = (fft_real*)malloc(sizeof(fft_real) * 2 * nc);
  r2c_rows(D, in, in_padded ? 2 * H : D, w); /* z */
  transform_axis(w, D, H, 1, -1);            /* y */
  transform_axis(w, D, H, 0, -1);            /* x */
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)(2 * nc); i++)
    out[i] = (float)w[i];
  free(w);
}

void mxo_c2r_3d(int D, const float* in, float* out)
{
  const int H = D / 2 + 1;
  const size_t nc = (size_t)D * D * H;
  fft_real* w = (fft_real*)malloc(sizeof(fft_real) * 2 * nc);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)(2 * nc); i++)
    w[i] = (fft_real)in[i];
  transform_axis(w, D, H, 0, +1); /* x */
  transform_axis(w, D, H, 1, +1); /* y */
  c2r_rows(D, w, out);            /* z */
  free(w);
}

/* =================================================================== spline */

int mxo_spline_init(mxo_spline* s, const double* x, const double* y, int n)
{
  s->n = n;
  s->x = (double*)malloc(sizeof(double) * (size_t)n);
  s->y = (double*)malloc(sizeof(double) * (size_t)n);
  s->c = (double*)calloc((size_t)n, sizeof(double));
  memcpy(s->x, x, sizeof(double) * (size_t)n);
  memcpy(s->y, y, sizeof(double) * (size_t)n);
  if (n < 3)
    return 0;
  /* Natural spline: solve the symmetric tridiagonal system for c[1..n-2]
   * (c = second derivative / 2), c[0] = c[n-1] = 0. */
  const int m = n - 2;
  double* diag = (double*)malloc(sizeof(double) * (size_t)m);
  double* off = (double*)malloc(sizeof(double) * (size_t)m);
  double* rhs = (double*)malloc(sizeof(double) * (size_t)m);
  for (int i = 0; i < m; i++) {
    const double h_i = x[i + 1] - x[i];
    const double h_ip1 = x[i + 2] - x[i + 1];
    const double dy_i = y[i + 1] - y[i];
    const double dy_ip1 = y[i + 2] - y[i + 1];
    const double g_i = (h_i != 0.0) ? 1.0 / h_i : 0.0;
    const double g_ip1 = (h_ip1 != 0.0) ? 1.0 / h_ip1 : 0.0;
    off[i] = h_ip1;
    diag[i] = 2.0 * (h_ip1 + h_i);
    rhs[i] = 3.0 * (dy_ip1 * g_ip1 - dy_i * g_i);
  }
  if (m == 1) {
    s->c[1] = rhs[0] / diag[0];
  } else {
    /* Thomas algorithm on the symmetric tridiagonal matrix. */
    double* cp = (double*)malloc(sizeof(double) * (size_t)m);
    double* dp = (double*)malloc(sizeof(double) * (size_t)m);
    cp[0] = off[0] / diag[0];
    dp[0] = rhs[0] / diag[0];
    for (int i = 1; i < m; i++) {
      const double den = diag[i] - off[i - 1] * cp[i - 1];
      cp[i] = (i < m - 1) ? off[i] / den : 0.0;
      dp[i] = (rhs[i] - off[i - 1] * dp[i - 1]) / den;
    }
    s->c[m] = dp[m - 1];
    for (int i = m - 2; i >= 0; i--)
      s->c[i + 1] = dp[i] - cp[i] * s->c[i + 2];
    free(cp);
    free(dp);
  }
  free(diag);
  free(off);
  free(rhs);
  return 0;
}

void mxo_spline_free(mxo_spline* s)
{
  free(s->x);
  free(s->y);
  free(s->c);
  s->x = s->y = s->c = NULL;
}

double mxo_spline_eval(const mxo_spline* s, double xv)
{
  const int n = s->n;
  const double* x = s->x;
  if (xv < x[0] || xv > x[n - 1])
    return NAN;
  /* index i with x[i] <= xv < x[i+1]; xv == x[n-1] maps to the last interval */
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) / 2;
    if (x[mid] > xv)
      hi = mid;
    else
      lo = mid;
  }
  const int i = lo;
  const double x_lo = x[i], x_hi = x[i + 1];
  const double dx = x_hi - x_lo;
  const double y_lo = s->y[i], y_hi = s->y[i + 1];
  if (dx <= 0.0)
    return NAN;
  const double dy = y_hi - y_lo;
  const double delx = xv - x_lo;
  const double c_i = s->c[i], c_ip1 = s->c[i + 1];
  const double b_i = dy / dx - dx * (c_ip1 + 2.0 * c_i) / 3.0;
  const double d_i = (c_ip1 - c_i) / (3.0 * dx);
  return y_lo + delx * (b_i + delx * (c_i + delx * d_i));
}

/* ====================================================================== QAG */

/* 61-point Gauss-Kronrod abscissae and weights (QUADPACK dqk61). */
static const double xgk61[31] = {
  0.999484410050490637571325895705811, 0.996893484074649540271630050918695, 0.991630996870404594858628366109486,
  0.983668123279747209970032581605663, 0.973116322501126268374693868423707, 0.960021864968307512216871025581798,
  0.944374444748559979415831324037439, 0.926200047429274325879324277080474, 0.905573307699907798546522558925958,
  0.882560535792052681543116462530226, 0.857205233546061098958658510658944, 0.829565762382768397442898119732502,
  0.799727835821839083013668942322683, 0.767777432104826194917977340974503, 0.733790062453226804726171131369528,
  0.697850494793315796932292388026640, 0.660061064126626961370053668149271, 0.620526182989242861140477556431189,
  0.579345235826361691756024932172540, 0.536624148142019899264169793311073, 0.492480467861778574993693061207709,
  0.447033769538089176780609900322854, 0.400401254830394392535476211542661, 0.352704725530878113471037207089374,
  0.304073202273625077372677107199257, 0.254636926167889846439805129817805, 0.204525116682309891438957671002025,
  0.153869913608583546963794672743256, 0.102806937966737030147096751318001, 0.051471842555317695833025213166723,
  0.000000000000000000000000000000000
};
static const double wg61[15] = {
  0.007968192496166605615465883474674, 0.018466468311090959142302131912047, 0.028784707883323369349719179611292,
  0.038799192569627049596801936446348, 0.048402672830594052902938140422808, 0.057493156217619066481721689402056,
  0.065974229882180495128128515115962, 0.073755974737705206268243850022191, 0.080755895229420215354694938460530,
  0.086899787201082979802387530715126, 0.092122522237786128717632707087619, 0.096368737174644259639468626351810,
  0.099593420586795267062780282103569, 0.101762389748405504596428952168554, 0.102852652893558840341285636705415
};
static const double wgk61[31] = {
  0.001389013698677007624551591226760, 0.003890461127099884051267201844516, 0.006630703915931292173319826369750,
  0.009273279659517763428441146892024, 0.011823015253496341742232898853251, 0.014369729507045804812451432443580,
  0.016920889189053272627572289420322, 0.019414141193942381173408951050128, 0.021828035821609192297167485738339,
  0.024191162078080601365686370725232, 0.026509954882333101610601709335075, 0.028754048765041292843978785354334,
  0.030907257562387762472884252943092, 0.032981447057483726031814191016854, 0.034979338028060024137499670731468,
  0.036882364651821229223911065617136, 0.038678945624727592950348651532281, 0.040374538951535959111995279752468,
  0.041969810215164246147147541285970, 0.043452539701356069316831728117073, 0.044814800133162663192355551616723,
  0.046059238271006988116271735559374, 0.047185546569299153945261478181099, 0.048185861757087129140779492298305,
  0.049055434555029778887528165367238, 0.049795683427074206357811569379942, 0.050405921402782346840893085653585,
  0.050881795898749606492297473049805, 0.051221547849258772170656282604944, 0.051426128537459025933862879215781,
  0.051494729429451567558340433647099
};

static double rescale_error(double err, double result_abs, double result_asc)
{
  err = fabs(err);
  if (result_asc != 0 && err != 0) {
    double scale = pow((200 * err / result_asc), 1.5);
    if (scale < 1)
      err = result_asc * scale;
    else
      err = result_asc;
  }
  if (result_abs > DBL_MIN / (50 * DBL_EPSILON)) {
    double min_err = 50 * DBL_EPSILON * result_abs;
    if (min_err > err)
      err = min_err;
  }
  return err;
}

static void qk61(mxo_fn f,
                 void* params,
                 double a,
                 double b,
                 double* result,
                 double* abserr,
                 double* resabs,
                 double* resasc)
{
  const int n = 31;
  double fv1[31], fv2[31];
  const double center = 0.5 * (a + b);
  const double half_length = 0.5 * (b - a);
  const double abs_half_length = fabs(half_length);
  const double f_center = f(center, params);
  double result_gauss = 0;
  double result_kronrod = f_center * wgk61[n - 1];
  double result_abs = fabs(result_kronrod);
  double result_asc = 0;
  for (int j = 0; j < (n - 1) / 2; j++) {
    const int jtw = j * 2 + 1;
    const double absc = half_length * xgk61[jtw];
    const double fval1 = f(center - absc, params);
    const double fval2 = f(center + absc, params);
    const double fsum = fval1 + fval2;
    fv1[jtw] = fval1;
    fv2[jtw] = fval2;
    result_gauss += wg61[j] * fsum;
    result_kronrod += wgk61[jtw] * fsum;
    result_abs += wgk61[jtw] * (fabs(fval1) + fabs(fval2));
  }
  for (int j = 0; j < n / 2; j++) {
    const int jtwm1 = j * 2;
    const double absc = half_length * xgk61[jtwm1];
    const double fval1 = f(center - absc, params);
    const double fval2 = f(center + absc, params);
    fv1[jtwm1] = fval1;
    fv2[jtwm1] = fval2;
    result_kronrod += wgk61[jtwm1] * (fval1 + fval2);
    result_abs += wgk61[jtwm1] * (fabs(fval1) + fabs(fval2));
  }
  const double mean = result_kronrod * 0.5;
  result_asc = wgk61[n - 1] * fabs(f_center - mean);
  for (int j = 0; j < n - 1; j++)
    result_asc += wgk61[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  const double err = (result_kronrod - result_gauss) * half_length;
  result_kronrod *= half_length;
  result_abs *= abs_half_length;
  result_asc *= abs_half_length;
  *result = result_kronrod;
  *resabs = result_abs;
  *resasc = result_asc;
  *abserr = rescale_error(err, result_abs, result_asc);
}

typedef struct qag_ws
{
  size_t limit, size, nrmax, i, maximum_level;
  double *alist, *blist, *rlist, *elist;
  size_t *order, *level;
} qag_ws;

static void ws_sort(qag_ws* w)
{
  const size_t last = w->size - 1;
  const size_t limit = w->limit;
  double* elist = w->elist;
  size_t* order = w->order;
  size_t i_nrmax = w->nrmax;
  size_t i_maxerr = order[i_nrmax];
  if (last < 2) {
    order[0] = 0;
    order[1] = 1;
    w->i = i_maxerr;
    return;
  }
  const double errmax = elist[i_maxerr];
  while (i_nrmax > 0 && errmax > elist[order[i_nrmax - 1]]) {
    order[i_nrmax] = order[i_nrmax - 1];
    i_nrmax--;
  }
  long top;
  if (last < (limit / 2 + 2))
    top = (long)last;
  else
    top = (long)(limit - last + 1);
  long i = (long)i_nrmax + 1;
  while (i < top && errmax < elist[order[i]]) {
    order[i - 1] = order[i];
    i++;
  }
  order[i - 1] = i_maxerr;
  const double errmin = elist[last];
  long k = top - 1;
  while (k > i - 2 && errmin >= elist[order[k]]) {
    order[k + 1] = order[k];
    k--;
  }
  order[k + 1] = last;
  i_maxerr = order[i_nrmax];
  w->i = i_maxerr;
  w->nrmax = i_nrmax;
}

static void ws_update(qag_ws* w,
                      double a1,
                      double b1,
                      double area1,
                      double error1,
                      double a2,
                      double b2,
                      double area2,
                      double error2)
{
  const size_t i_max = w->i;
  const size_t i_new = w->size;
  const size_t new_level = w->level[i_max] + 1;
  if (error2 > error1) {
    w->alist[i_max] = a2;
    w->rlist[i_max] = area2;
    w->elist[i_max] = error2;
    w->level[i_max] = new_level;
    w->alist[i_new] = a1;
    w->blist[i_new] = b1;
    w->rlist[i_new] = area1;
    w->elist[i_new] = error1;
    w->level[i_new] = new_level;
  } else {
    w->blist[i_max] = b1;
    w->rlist[i_max] = area1;
    w->elist[i_max] = error1;
    w->level[i_max] = new_level;
    w->alist[i_new] = a2;
    w->blist[i_new] = b2;
    w->rlist[i_new] = area2;
    w->elist[i_new] = error2;
    w->level[i_new] = new_level;
  }
  w->size++;
  if (new_level > w->maximum_level)
    w->maximum_level = new_level;
  ws_sort(w);
}

int mxo_qag61(mxo_fn f,
              void* params,
              double a,
              double b,
              double epsabs,
              double epsrel,
              size_t limit,
              double* result,
              double* abserr)
{
  qag_ws w;
  w.limit = limit;
  w.alist = (double*)malloc(sizeof(double) * limit);
  w.blist = (double*)malloc(sizeof(double) * limit);
  w.rlist = (double*)malloc(sizeof(double) * limit);
  w.elist = (double*)malloc(sizeof(double) * limit);
  w.order = (size_t*)malloc(sizeof(size_t) * limit);
  w.level = (size_t*)malloc(sizeof(size_t) * limit);
  w.size = 0;
  w.nrmax = 0;
  w.i = 0;
  w.alist[0] = a;
  w.blist[0] = b;
  w.rlist[0] = 0.0;
  w.elist[0] = 0.0;
  w.order[0] = 0;
  w.level[0] = 0;
  w.maximum_level = 0;

  int status = 0;
  double result0, abserr0, resabs0, resasc0;
  qk61(f, params, a, b, &result0, &abserr0, &resabs0, &resasc0);
  w.size = 1;
  w.rlist[0] = result0;
  w.elist[0] = abserr0;

  double tolerance = fmax(epsabs, epsrel * fabs(result0));
  const double round_off = 50 * DBL_EPSILON * resabs0;

  if (abserr0 <= round_off && abserr0 > tolerance) {
    *result = result0;
    *abserr = abserr0;
    status = 18; /* roundoff */
    goto done;
  } else if ((abserr0 <= tolerance && abserr0 != resasc0) || abserr0 == 0.0) {
    *result = result0;
    *abserr = abserr0;
    status = 0;
    goto done;
  } else if (limit == 1) {
    *result = result0;
    *abserr = abserr0;
    status = 11;
    goto done;
  }

  {
    double area = result0;
    double errsum = abserr0;
    size_t iteration = 1;
    int roundoff_type1 = 0, roundoff_type2 = 0, error_type = 0;
    do {
      const double a_i = w.alist[w.i], b_i = w.blist[w.i], r_i = w.rlist[w.i], e_i = w.elist[w.i];
      const double a1 = a_i, b1 = 0.5 * (a_i + b_i);
      const double a2 = b1, b2 = b_i;
      double area1, area2, error1, error2, resabs1, resabs2, resasc1, resasc2;
      qk61(f, params, a1, b1, &area1, &error1, &resabs1, &resasc1);
      qk61(f, params, a2, b2, &area2, &error2, &resabs2, &resasc2);
      const double area12 = area1 + area2;
      const double error12 = error1 + error2;
      errsum += (error12 - e_i);
      area += area12 - r_i;
      if (resasc1 != error1 && resasc2 != error2) {
        const double delta = r_i - area12;
        if (fabs(delta) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i)
          roundoff_type1++;
        if (iteration >= 10 && error12 > e_i)
          roundoff_type2++;
      }
      tolerance = fmax(epsabs, epsrel * fabs(area));
      if (errsum > tolerance) {
        if (roundoff_type1 >= 6 || roundoff_type2 >= 20)
          error_type = 2;
        const double tmp = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
        if (fabs(a1) <= tmp && fabs(b2) <= tmp)
          error_type = 3;
      }
      ws_update(&w, a1, b1, area1, error1, a2, b2, area2, error2);
      iteration++;
    } while (iteration < limit && !error_type && errsum > tolerance);

    double sum = 0.0;
    for (size_t k = 0; k < w.size; k++)
      sum += w.rlist[k];
    *result = sum;
    *abserr = errsum;
    if (errsum <= tolerance)
      status = 0;
    else if (error_type == 2)
      status = 18;
    else if (error_type == 3)
      status = 21;
    else if (iteration == limit)
      status = 11;
    else
      status = 5;
  }

done:
  free(w.alist);
  free(w.blist);
  free(w.rlist);
  free(w.elist);
  free(w.order);
  free(w.level);
  return status;
}

/* ==================================================================== Brent */

int mxo_brent_set(mxo_brent* s, mxo_fn f, void* params, double x_lower, double x_upper)
{
  s->f = f;
  s->params = params;
  s->root = 0.5 * (x_lower + x_upper);
  s->x_lower = x_lower;
  s->x_upper = x_upper;
  const double f_lower = f(x_lower, params);
  const double f_upper = f(x_upper, params);
  s->a = x_lower;
  s->fa = f_lower;
  s->b = x_upper;
  s->fb = f_upper;
  s->c = x_upper;
  s->fc = f_upper;
  s->d = x_upper - x_lower;
  s->e = x_upper - x_lower;
  if ((f_lower < 0.0 && f_upper < 0.0) || (f_lower > 0.0 && f_upper > 0.0))
    return 4; /* endpoints do not straddle y=0 */
  return 0;
}

int mxo_brent_iterate(mxo_brent* s)
{
  double tol, m;
  int ac_equal = 0;
  double a = s->a, b = s->b, c = s->c;
  double fa = s->fa, fb = s->fb, fc = s->fc;
  double d = s->d, e = s->e;

  if ((fb < 0 && fc < 0) || (fb > 0 && fc > 0)) {
    ac_equal = 1;
    c = a;
    fc = fa;
    d = b - a;
    e = b - a;
  }
  if (fabs(fc) < fabs(fb)) {
    ac_equal = 1;
    a = b;
    b = c;
    c = a;
    fa = fb;
    fb = fc;
    fc = fa;
  }
  tol = 0.5 * DBL_EPSILON * fabs(b);
  m = 0.5 * (c - b);
  if (fb == 0) {
    s->root = b;
    s->x_lower = b;
    s->x_upper = b;
    return 0;
  }
  if (fabs(m) <= tol) {
    s->root = b;
    if (b < c) {
      s->x_lower = b;
      s->x_upper = c;
    } else {
      s->x_lower = c;
      s->x_upper = b;
    }
    return 0;
  }
  if (fabs(e) < tol || fabs(fa) <= fabs(fb)) {
    d = m; /* bisection */
    e = m;
  } else {
    double p, q, r;
    const double sv = fb / fa;
    if (ac_equal) {
      p = 2 * m * sv;
      q = 1 - sv;
    } else {
      q = fa / fc;
      r = fb / fc;
      p = sv * (2 * m * q * (q - r) - (b - a) * (r - 1));
      q = (q - 1) * (r - 1) * (sv - 1);
    }
    if (p > 0)
      q = -q;
    else
      p = -p;
    if (2 * p < fmin(3 * m * q - fabs(tol * q), fabs(e * q))) {
      e = d;
      d = p / q;
    } else {
      d = m; /* interpolation failed, fall back to bisection */
      e = m;
    }
  }
  a = b;
  fa = fb;
  if (fabs(d) > tol)
    b += d;
  else
    b += (m > 0 ? +tol : -tol);
  fb = s->f(b, s->params);
  s->root = b;
  if ((fb < 0 && fc < 0) || (fb > 0 && fc > 0))
    c = a;
  if (b < c) {
    s->x_lower = b;
    s->x_upper = c;
  } else {
    s->x_lower = c;
    s->x_upper = b;
  }
  s->a = a;
  s->b = b;
  s->c = c;
  s->fa = fa;
  s->fb = fb;
  s->fc = fc;
  s->d = d;
  s->e = e;
  return 0;
}

int mxo_root_test_interval(double x_lower, double x_upper, double epsabs, double epsrel)
{
  const double abs_lower = fabs(x_lower), abs_upper = fabs(x_upper);
  double min_abs;
  if ((x_lower > 0.0 && x_upper > 0.0) || (x_lower < 0.0 && x_upper < 0.0))
    min_abs = fmin(abs_lower, abs_upper);
  else
    min_abs = 0;
  const double tolerance = epsabs + epsrel * min_abs;
  if (fabs(x_upper - x_lower) < tolerance)
    return 0;
  return 1;
}
