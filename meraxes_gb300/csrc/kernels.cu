// Device kernels of the reionization grid step (see kernels.cuh).
//
// Layouts: PADDED real grids index k + 2H (j + D i); REAL grids k + D (j + D i);
// half spectra k + H (j + D i), H = D/2 + 1 (src/core/misc_tools.c:200-214).
#include <math_constants.h>

#include <cfloat>
#include <cmath>

#include "kernels.cuh"

namespace mx {

namespace {
int g_launches = 0;

constexpr float REL_TOL = 1e-5f;
constexpr float ABS_TOL = 1e-8f;
constexpr double PI_D = 3.14159265358979323846;
constexpr double TCMB = 2.728;
constexpr double T21 = 0.0628;
constexpr double A10 = 2.85e-15;
constexpr double BOLTZMANN = 1.3806e-16;
constexpr double FRACT_FLOAT_ERR = 1e-7;
constexpr float MAX_TK = 5e4f;
constexpr int NXHII = 14;
constexpr int RR_Z_NPTS = 300;
constexpr int RR_LNG_NPTS = 150;
constexpr float RR_DEL_Z = 0.2f;
constexpr float RR_DEL_LNG = 0.1f;
constexpr double RR_LNG_MIN = -10.0;
constexpr int TS_MAX_ITER = 10000;

int blocks_for(long long n, int threads)
{
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 32)
    b = 152LL * 32;
  if (b < 1)
    b = 1;
  return (int)b;
}

// Block-wide sum of NV doubles into partials[blockIdx.x * NV + v].
template <int NV>
__device__ void block_reduce_store(double (&v)[NV], double* partials)
{
  __shared__ double sh[NV][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1)
      x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0)
      sh[q][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < RED_THREADS / 32; w++)
      s += sh[threadIdx.x][w];
    partials[(long long)blockIdx.x * NV + threadIdx.x] = s;
  }
}

__device__ __forceinline__ long long pad_of(long long ir, int D, int H)
{
  const long long row = ir / D;
  return ir - row * D + row * 2LL * H;
}

// natural cubic spline evaluation (bracketing by bisection), NaN outside
__device__ double spline_eval(const double* x, const double* y, const double* c, int n, double xv)
{
  if (!(xv >= x[0] && xv <= x[n - 1]))
    return CUDART_NAN;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] > xv)
      hi = mid;
    else
      lo = mid;
  }
  const double h = x[lo + 1] - x[lo];
  const double dx = xv - x[lo];
  const double b = (y[lo + 1] - y[lo]) / h - h * (c[lo + 1] + 2.0 * c[lo]) / 3.0;
  const double d = (c[lo + 1] - c[lo]) / (3.0 * h);
  return y[lo] + dx * (b + dx * (c[lo] + dx * d));
}
}  // namespace

int kernel_launch_count() { return g_launches; }
void reset_kernel_launch_count() { g_launches = 0; }

// ================================================================= filter
// filter(), src/core/reionization.c:2110-2170, fused with the 1/N scale of
// find_HII_bubbles.c:168-182 (scale_mode 0) or ComputeTs.c:383-384 (mode 1),
// for every radius of the batch.  Each thread reads every field once and
// writes one filtered copy per radius.
__global__ void k_filter(const float2* const* __restrict__ in,
                         int G,
                         float2* __restrict__ out,
                         long long out_field_stride,
                         FilterBatch fb,
                         int D,
                         int H,
                         long long C,
                         float delta_k,
                         double inv_scale_d,
                         float scale_f,
                         int pow2)
{
  const int middle = D / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < C; e += (long long)gridDim.x * blockDim.x) {
    const int nz = (int)(e % H);
    const long long rest = e / H;
    const int ny = (int)(rest % D);
    const int nx = (int)(rest / D);
    const float kx = (nx > middle) ? __fmul_rn((float)(nx - D), delta_k) : __fmul_rn((float)nx, delta_k);
    const float ky = (ny > middle) ? __fmul_rn((float)(ny - D), delta_k) : __fmul_rn((float)ny, delta_k);
    const float kz = __fmul_rn((float)nz, delta_k);
    const float kmag = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz)));
    float2 v[MAX_FIELDS];
    for (int g = 0; g < G; g++) {
      float2 t = in[g][e];
      if (fb.scale_mode == 0) {
        if (pow2) {
          t.x = __fmul_rn(t.x, scale_f);
          t.y = __fmul_rn(t.y, scale_f);
        } else {
          t.x = (float)((double)t.x * inv_scale_d);
          t.y = (float)((double)t.y * inv_scale_d);
        }
      } else {
        t.x = __fdiv_rn(t.x, scale_f);
        t.y = __fdiv_rn(t.y, scale_f);
      }
      v[g] = t;
    }
    for (int r = 0; r < fb.n; r++) {
      float w = 1.0f;
      bool zero = false;
      if (fb.apply[r]) {
        float kR = __fmul_rn(kmag, fb.R[r]);
        if (fb.filter_type == 0) {
          if ((double)kR > 1e-4)
            w = (float)(3.0 * (double)(__fsub_rn(__fdiv_rn(sinf(kR), powf(kR, 3.0f)), __fdiv_rn(cosf(kR), powf(kR, 2.0f)))));
        } else if (fb.filter_type == 1) {
          kR = (float)((double)kR * 0.413566994);
          zero = kR > 1.0f;
        } else {
          kR = (float)((double)kR * 0.643);
          w = powf((float)2.71828182845904523536, (float)((double)__fmul_rn(-kR, kR) / 2.0));
        }
      }
      float2* o = out + (long long)r * G * out_field_stride;
      for (int g = 0; g < G; g++) {
        float2 t = v[g];
        if (zero) {
          t.x = 0.0f;
          t.y = 0.0f;
        } else if (fb.apply[r] && fb.filter_type != 1) {
          t.x = __fmul_rn(t.x, w);
          t.y = __fmul_rn(t.y, w);
        }
        o[(long long)g * out_field_stride + e] = t;
      }
    }
  }
}

void launch_filter(const float2* const* in,
                   int G,
                   float2* out,
                   long long out_field_stride,
                   const FilterBatch& fb,
                   const GridDims& gd,
                   float box_size,
                   cudaStream_t s)
{
  const float delta_k = (float)(2.0 * PI_D / box_size);
  const double N = (double)gd.N;
  const bool pow2 = (gd.N & (gd.N - 1)) == 0;
  const float scale_f = fb.scale_mode == 0 ? (float)(1.0 / N) : (float)N;
  k_filter<<<blocks_for(gd.C, 256), 256, 0, s>>>(in, G, out, out_field_stride, fb, gd.D, gd.H, gd.C, delta_k,
                                                  1.0 / N, scale_f, pow2 ? 1 : 0);
  g_launches++;
}

// ======================================================== threshold loop
// The per-cell test of find_HII_bubbles.c:271-311 (aliasing clamps) and
// :342-443 (ionisation criterion and bookkeeping) for every radius of the
// batch, largest first, with the cell state held in registers.
__global__ void k_threshold(ThresholdArgs a, int D, int H, long long N)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    float xH = a.xH[ir];
    float zion = a.z_at_ion[ir];
    float rb = a.r_bubble[ir];
    float J21 = a.uvb ? a.J21[ir] : 0.0f;
    float J21i = a.uvb ? a.J21_at_ion[ir] : 0.0f;
    float G12 = a.recomb ? a.Gamma12[ir] : 0.0f;
    for (int r = 0; r < a.n_r; r++) {
      const RadiusParams rp = a.rp[r];
      const float* f = a.fields + (long long)r * a.G * a.P;
      const bool direct = rp.last != 0;
      auto field = [&](int g) -> float { return direct ? a.direct[g][ip] : f[(long long)g * a.P + ip]; };
      const float dx = fmaxf(field(0), -1 + REL_TOL);
      float st = fmaxf(field(1), 0.0f);
      if (st < ABS_TOL)
        st = 0;
      float ws = fmaxf(field(2), 0.0f);
      if (ws < ABS_TOL)
        ws = 0;
      double rec = 0.0;
      if (a.recomb) {
        float nr = fmaxf(field(a.idx_nr), 0.0f);
        if (nr < ABS_TOL)
          nr = 0;
        rec = (double)nr / (1.0 + (double)dx);
      }
      double nf = 1.0;
      if (a.spin) {
        float xe = fmaxf(field(a.idx_xe), 0.0f);
        if (xe < ABS_TOL)
          xe = 0;
        xe = fminf(xe, 0.999f);
        nf = 1.0 - (double)xe;
      }
      const double dom = 1.0 + (double)dx;
      const double f_coll = (double)st / (rp.M_mean * dom) * (4.0 / 3.0) * PI_D * rp.R_cubed / a.pixel_volume;
      const double wsd = (double)ws / a.pixel_volume;
      const float J21_aux = a.uvb ? (float)(wsd * rp.J21_const) : 0.0f;
      if (f_coll * a.eff > nf * (1. + rec)) {
        if (xH > REL_TOL) {
          if (a.uvb)
            J21 = J21_aux;
          if (a.recomb)
            G12 = (float)(rp.Gamma_pref * wsd);
        }
        xH = 0.0f;
        rb = (float)rp.R;
      } else if (rp.last && (xH > REL_TOL)) {
        xH = (float)__dsub_rn(nf, __dmul_rn(f_coll, a.eff));
        if (xH < 0.f)
          xH = 0.f;
        else if (xH > 1.0f)
          xH = 1.f;
      }
      if ((xH < REL_TOL) && (zion < 0)) {
        zion = (float)a.redshift;
        if (a.uvb)
          J21i = J21_aux * a.gamma_halo_bias;
      }
    }
    a.xH[ir] = xH;
    a.z_at_ion[ir] = zion;
    a.r_bubble[ir] = rb;
    if (a.uvb) {
      a.J21[ir] = J21;
      a.J21_at_ion[ir] = J21i;
    }
    if (a.recomb)
      a.Gamma12[ir] = G12;
  }
}

void launch_threshold(const ThresholdArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_threshold<<<blocks_for(gd.N, 256), 256, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

// ============================================================= reductions
// find_HII_bubbles.c:451-477: volume / mass weighted sums and the N_rec
// recombination update (recombinations.c:30-52 lookup).
__global__ void k_fhb_reduce(FhbReduceArgs a, int D, int H, long long N)
{
  double acc[4] = { 0, 0, 0, 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const double cell_xH = (double)a.xH[ir];
    acc[0] += cell_xH;
    if (a.uvb)
      acc[1] += (double)a.J21[ir];
    const double dom = 1.0 + (double)a.deltax[ip];
    acc[2] += cell_xH * dom;
    acc[3] += dom;
    if (a.recomb) {
      const float z_eff = (float)__dsub_rn(__dmul_rn(1. + a.redshift, pow(dom, 1.0 / 3.0)), 1.0);
      const double g12 = (double)a.Gamma12[ir];
      int z_ct = (int)((double)z_eff / (double)RR_DEL_Z + 0.5);
      double lnG = log(g12);
      if (z_ct < 0)
        z_ct = 0;
      else if (z_ct >= RR_Z_NPTS)
        z_ct = RR_Z_NPTS - 1;
      double rr;
      if (lnG < RR_LNG_MIN)
        rr = 0.0;
      else {
        // RR_DEL_LNG * RR_LNG_NPTS is a float product in recombinations.c:46
        const double lng_top = RR_LNG_MIN + (double)(RR_DEL_LNG * (float)RR_LNG_NPTS);
        if (lnG >= lng_top)
          lnG = lng_top - FRACT_FLOAT_ERR;
        rr = spline_eval(a.rr_x, a.rr_y + (long long)z_ct * RR_LNG_NPTS, a.rr_c + (long long)z_ct * RR_LNG_NPTS,
                         RR_LNG_NPTS, lnG);
      }
      const double dNrec = rr * (double)a.fabs_dtdz * (double)a.zstep * (1. - cell_xH);
      a.N_rec[ip] = (float)((double)a.N_rec[ip] + dNrec);
    }
  }
  block_reduce_store<4>(acc, a.partials);
}

void launch_fhb_reduce(const FhbReduceArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_fhb_reduce<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

__global__ void k_finalize(const double* __restrict__ partials, int nvals, double* __restrict__ out)
{
  // one thread per value, fixed summation order over blocks
  const int v = threadIdx.x;
  if (v < nvals) {
    double s = 0.0;
    for (int b = 0; b < RED_BLOCKS; b++)
      s += partials[(long long)b * nvals + v];
    out[v] = s;
  }
}

void launch_finalize(const double* partials, int nvals, double* out, cudaStream_t s)
{
  k_finalize<<<1, 32, 0, s>>>(partials, nvals, out);
  g_launches++;
}

// ============================================================ grid helpers
__global__ void k_fill(float* p, long long n, float v)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}
void launch_fill(float* p, long long n, float v, cudaStream_t s)
{
  k_fill<<<blocks_for(n, 256), 256, 0, s>>>(p, n, v);
  g_launches++;
}
__global__ void k_fill_real_in_padded(float* p, int D, int H, long long N, float v)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x)
    p[pad_of(ir, D, H)] = v;
}
void launch_fill_real_in_padded(float* p, const GridDims& gd, float v, cudaStream_t s)
{
  k_fill_real_in_padded<<<blocks_for(gd.N, 256), 256, 0, s>>>(p, gd.D, gd.H, gd.N, v);
  g_launches++;
}

// =============================================================== ComputeTs
// ComputeTs.c:321-322 / 311-312: the first slab_n_complex floats of the
// padded sfr grid are rescaled or cleared (the reference loops over
// slab_n_complex float elements of a 2*slab_n_complex array).
__global__ void k_sfr_scale_half(float* sfr, long long n, double w)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    sfr[i] = (float)((double)sfr[i] * w);
}
void launch_sfr_scale_half(float* sfr, long long nhalf, double w, cudaStream_t s)
{
  k_sfr_scale_half<<<blocks_for(nhalf, 256), 256, 0, s>>>(sfr, nhalf, w);
  g_launches++;
}
void launch_sfr_zero_half(float* sfr, long long nhalf, cudaStream_t s)
{
  k_fill<<<blocks_for(nhalf, 256), 256, 0, s>>>(sfr, nhalf, 0.0f);
  g_launches++;
}
// load_reion_sfr_grids, reionization.c:1756-1784: the history slice is read
// with REAL indexing and written with PADDED indexing.
__global__ void k_sfr_load(float* sfr, const float* slice, float w, int acc, int D, int H, long long N)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const float v = __fmul_rn(slice[ir], w);
    sfr[ip] = acc ? __fadd_rn(sfr[ip], v) : v;
  }
}
void launch_sfr_load(float* sfr, const float* slice, float w, int accumulate, const GridDims& gd, cudaStream_t s)
{
  k_sfr_load<<<blocks_for(gd.N, 256), 256, 0, s>>>(sfr, slice, w, accumulate, gd.D, gd.H, gd.N);
  g_launches++;
}

__global__ void k_shell_extract(const float* filtered, long long P, int n, int r0, float* shells, int D, int H,
                                long long N)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    for (int r = 0; r < n; r++)
      shells[(long long)(r0 + r) * N + ir] = fmaxf(filtered[(long long)r * P + ip], 0.0f);
  }
}
void launch_shell_extract(const float* filtered, long long P, int n, int r0, float* shells, const GridDims& gd,
                          cudaStream_t s)
{
  k_shell_extract<<<blocks_for(gd.N, 256), 256, 0, s>>>(filtered, P, n, r0, shells, gd.D, gd.H, gd.N);
  g_launches++;
}

// ComputeTs.c:438-475
__global__ void k_cf_xe(CfArgs a, int D, int H, long long N)
{
  double acc[2] = { 0, 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const double dom = 1.0 + a.deltax[ip];
    double cf = a.stars[ip] / (a.RtoM_h2 * dom) * (4.0 / 3.0) * PI_D * a.R3 / a.pixel_volume;
    if (cf > 1.0)
      cf = 1.0;
    acc[0] += cf;
    acc[1] += a.x_e_prev[ip];
  }
  block_reduce_store<2>(acc, a.partials);
}
void launch_cf_xe(const CfArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_cf_xe<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

namespace {
// alpha_A, XRayHeatingFunctions.c:1450-1458
__device__ double d_alpha_A(double T)
{
  const double logT = log(T / (double)1.1604505e4);
  return exp(-28.6130338 - 0.72411256 * logT - 2.02604473e-2 * pow(logT, 2) - 2.38086188e-3 * pow(logT, 3) -
             3.21260521e-4 * pow(logT, 4) - 1.42150291e-5 * pow(logT, 5) + 4.98910892e-6 * pow(logT, 6) +
             5.75561414e-7 * pow(logT, 7) - 1.85676704e-8 * pow(logT, 8) - 3.07113524e-9 * pow(logT, 9));
}

__device__ double d_kappa(const TsDevConst& c, int which, double T)
{
  // kappa_10 (which 0): power law above the table; elec/pH (1,2): linear in logs
  const int n = c.nk[which];
  const double* x = c.kx[which];
  const double* y = c.ky[which];
  double ans;
  if (which == 0) {
    if (log(T) < x[0])
      ans = y[0];
    else if (log(T) > x[n - 1])
      ans = log(exp(y[n - 1]) * pow(T / exp(x[n - 1]), 0.381));
    else
      ans = spline_eval(x, y, c.kc[which], n, log(T));
  } else {
    const double lt = log(T);
    if (lt < x[0])
      ans = y[0];
    else if (lt > x[n - 1])
      ans = y[n - 1] + ((y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]) * (lt - x[n - 1]));
    else
      ans = spline_eval(x, y, c.kc[which], n, lt);
  }
  return exp(ans);
}

// get_Ts, XRayHeatingFunctions.c:1513-1558 (+ xcoll :1560-1600, xalpha_tilde
// / taugp / Salpha_tilde / Tc_eff :1847-1882).  The fixed-point iteration is
// capped; hitting the cap sets bit 0 of *err.
__device__ float d_get_Ts(const TsDevConst& c, float z, float delta, float TK, float xe, float Jalpha, float* curr_xalpha,
                          unsigned int* err)
{
  const double zd = z, TKd = TK, dd = delta, xd = xe;
  const double Trad = TCMB * (1.0 + zd);
  const double p3 = pow(1.0 + zd, 3.0);
  const double nH = (1.0 - xd) * c.no * p3 * (1.0 + dd);
  const double ne = xd * c.n_b0 * p3 * (1.0 + dd);
  const double np = xd * c.no * p3 * (1.0 + dd);
  const double xc = T21 / Trad * nH * d_kappa(c, 0, TKd) / A10 + T21 / Trad * ne * d_kappa(c, 1, TKd) / A10 +
                    T21 / Trad * np * d_kappa(c, 2, TKd) / A10;
  double TS, TSinv, xa = 0;
  if (Jalpha > 1.0e-20) {
    TS = Trad;
    double TSold = 0.0;
    const double tgp = 1.342881e-7 / c.hubble_z * c.no * pow(1 + zd, 3) * (1.0 + dd) * (1.0 - xd);
    const double xi = pow(1.0e-7 * tgp / TKd / TKd, 1.0 / 3.0);
    int it = 0;
    while (fabs(TS - TSold) / TS > 1.0e-3) {
      if (++it > TS_MAX_ITER) {
        atomicOr(err, 1u);
        break;
      }
      TSold = TS;
      double St = 1.0 - 0.0631789 / TKd + 0.115995 / TKd / TKd - 0.401403 / TS / TKd;
      St += 0.336463 / TS / TKd / TKd;
      St /= 1.0 + 2.98394 * xi + 1.53583 * xi * xi + 3.85289 * xi * xi * xi;
      xa = 1.66e11 / (1.0 + zd) * St * (double)Jalpha;
      const double Tceff = 1.0 / (1.0 / TKd + 0.405535 / TKd * (1.0 / TS - 1.0 / TKd));
      TSinv = (1.0 / Trad + xa / Tceff + xc / TKd) / (1.0 + xa + xc);
      TS = 1.0 / TSinv;
    }
    *curr_xalpha = (float)xa;
  } else {
    TSinv = (1.0 / Trad + xc / TKd) / (1.0 + xc);
    TS = 1.0 / TSinv;
    *curr_xalpha = 0;
  }
  if (TS < 0.)
    TS = fabs(TS);
  return (float)TS;
}
}  // namespace

// Per-cell spin-temperature update, ComputeTs.c:743-900 with evolveInt
// (XRayHeatingFunctions.c:1241-1435).  The frequency tables are staged in
// shared memory once per block.
__global__ void k_evolve(EvolveArgs a, int D, int H, long long N)
{
  const TsDevConst& c = *a.cst;
  const int S = c.S;
  extern __shared__ double s_tab[];  // 3 * 14 * S
  for (int i = threadIdx.x; i < 3 * NXHII * S; i += blockDim.x) {
    const int t = i / (NXHII * S), rem = i % (NXHII * S), x = rem / S, r = rem % S;
    s_tab[i] = c.tab[t][x][r];
  }
  __syncthreads();
  const double Conversion = c.conv;
  double acc[4] = { 0, 0, 0, 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const float delta = a.deltax[ip];
    float xe_f = a.x_e_prev[ip];
    float Tk_f = a.Tk[ir];
    const double x_e = xe_f, T = Tk_f;
    double xcall = xe_f;
    if (xcall > c.xhii[NXHII - 1] * 0.999)
      xcall = c.xhii[NXHII - 1] * 0.999;
    else if (xcall < c.xhii[0])
      xcall = 1.001 * c.xhii[0];
    int lo = NXHII - 1;
    while ((float)xcall < c.xhii[lo])
      lo--;
    const int hi = lo + 1;
    const double dxh = (double)(c.xhii[hi] - c.xhii[lo]);
    const double wx = xcall - c.xhii[lo];
    const float zp = c.zp;
    const double n_b = c.n_b0 * c.p3 * (1 + delta);
    double heat = 0, ion = 0, lya = 0, starlya = 0;
    if (!c.no_light) {
      for (int r = 0; r < S; r++) {
        const float sf = a.shells[(long long)r * N + ir];
        const double SFR = ((sf / c.pixel_volume) * c.sfr_a) * c.sfr_b / 1.989e33;
        const double fh = (s_tab[(0 * NXHII + hi) * S + r] - s_tab[(0 * NXHII + lo) * S + r]) / dxh * wx +
                          s_tab[(0 * NXHII + lo) * S + r];
        const double fi = (s_tab[(1 * NXHII + hi) * S + r] - s_tab[(1 * NXHII + lo) * S + r]) / dxh * wx +
                          s_tab[(1 * NXHII + lo) * S + r];
        const double fl = (s_tab[(2 * NXHII + hi) * S + r] - s_tab[(2 * NXHII + lo) * S + r]) / dxh * wx +
                          s_tab[(2 * NXHII + lo) * S + r];
        const double integrand = SFR * c.b[r];
        heat += c.a[r] * integrand * fh;
        ion += c.a[r] * integrand * fi;
        lya += c.a[r] * integrand * fl;
        starlya += SFR * c.p2 * c.zpp1[r] * c.sum_lyn[r] * c.dt_dzpp[r] * c.dzpp[r];
      }
      heat *= c.prefactor;
      ion *= c.prefactor;
      lya *= c.prefactor * n_b;
      starlya *= Conversion;
    }
    const double sink = d_alpha_A(T) * c.clumping * x_e * x_e * c.f_h * n_b;
    const double dxe_dzp = c.dt_dzp * (ion - sink);
    double dadia = 3 / (1.0 + zp);
    if (fabs(delta) > FRACT_FLOAT_ERR)
      dadia += c.dgrowth / (1.0 / delta + c.growth);
    dadia *= (2.0 / 3.0) * T;
    const double dspec = -dxe_dzp * T / (1 + x_e);
    const double Trad = TCMB * (1.0 + zp);
    double dcomp = (-1.51e-4) * (x_e / (1.0 + x_e + c.f_he)) / (c.hubble_z / c.hubble0_h) / c.h * pow(Trad, 4.0) /
                   (1.0 + zp);
    dcomp *= Trad - T;
    const double dxheat_dzp = heat * c.dt_dzp * 2.0 / 3.0 / BOLTZMANN / (1.0 + x_e);
    const double d1 = dxheat_dzp + dcomp + dspec + dadia;
    const double d2 = lya + starlya;
    const double d4 = c.dt_dzp * ion;

    xe_f = (float)((double)xe_f + dxe_dzp * c.dzp);
    if (xe_f > 1)
      xe_f = (float)(1 - FRACT_FLOAT_ERR);
    else if (xe_f < 0)
      xe_f = 0;
    if (Tk_f < MAX_TK)
      Tk_f = (float)((double)Tk_f + d1 * c.dzp);
    if (Tk_f < 0)
      Tk_f = (float)(TCMB * (1 + c.zpd));
    float xalpha;
    const float TS = d_get_Ts(c, zp, delta, Tk_f, xe_f, (float)d2, &xalpha, a.err);
    a.x_e_prev[ip] = xe_f;
    a.Tk[ir] = Tk_f;
    a.TS[ir] = TS;
    acc[0] += d2;
    acc[1] += xalpha;
    acc[2] += dxheat_dzp;
    acc[3] += d4;
  }
  block_reduce_store<4>(acc, a.partials);
}

void launch_evolve(const EvolveArgs& a, const GridDims& gd, cudaStream_t s)
{
  // the constant block lives in device memory; S is read on the host side
  const int S_max = MAX_SHELLS;
  (void)S_max;
  k_evolve<<<RED_BLOCKS, RED_THREADS, 3 * NXHII * MAX_SHELLS * sizeof(double), s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

// Homogeneous branch, ComputeTs.c:189-262
__global__ void k_homog(HomogArgs a, int D, int H, long long N)
{
  const TsDevConst& c = *a.cst;
  double acc[1] = { 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    a.x_e_prev[ip] = a.xe0;
    a.Tk[ir] = a.tk0;
    float xa;
    a.TS[ir] = d_get_Ts(c, c.zp, a.deltax[ip], a.tk0, a.xe0, 0.0f, &xa, a.err);
    const double dom = 1.0 + a.deltax[ip];
    double cf = a.stars[ip] / (a.RtoM_h2 * dom) * (4.0 / 3.0) * PI_D * a.R3 / a.pixel_volume;
    if (cf > 1.0)
      cf = 1.0;
    acc[0] += cf;
  }
  block_reduce_store<1>(acc, a.partials);
}
void launch_homog(const HomogArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_homog<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

__global__ void k_ts_means(const float* TS, const float* Tk, double* partials, long long N)
{
  double acc[2] = { 0, 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    acc[0] += (double)TS[ir];
    acc[1] += (double)Tk[ir];
  }
  block_reduce_store<2>(acc, partials);
}
void launch_ts_means(const float* TS, const float* Tk, double* partials, const GridDims& gd, cudaStream_t s)
{
  k_ts_means<<<RED_BLOCKS, RED_THREADS, 0, s>>>(TS, Tk, partials, gd.N);
  g_launches++;
}

// ================================================== brightness temperature
// BrightnessTemperature.c:84-124 and the mean at :512-535
__global__ void k_delta_T(DeltaTArgs a, int D, int H, long long N)
{
  double acc[1] = { 0 };
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const double pdx = a.deltax[ip];
    const double pxh = a.xH[ir];
    float dT = (float)((double)a.const_factor * pxh * (1.0 + pdx));
    if (a.spin) {
      const float ts = a.TS[ir];
      if (a.pecvel > 1)
        dT = (float)((double)dT * ((1. + (double)a.redshift) / (1000. * (double)ts)));
      else
        dT = (float)((double)dT * (1 - a.T_rad / (double)ts));
    }
    a.delta_T[ir] = dT;
    acc[0] += (double)dT;
  }
  block_reduce_store<1>(acc, a.partials);
}
void launch_delta_T(const DeltaTArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_delta_T<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

}  // namespace mx
