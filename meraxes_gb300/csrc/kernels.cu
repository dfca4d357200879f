// Device kernels of the reionization grid step (see kernels.cuh).
//
// Layouts: PADDED real grids index k + 2H (j + D i); REAL grids k + D (j + D i);
// half spectra k + H (j + D i), H = D/2 + 1 (src/core/misc_tools.c:200-214).
#include <math_constants.h>

#include <cfloat>
#include <cmath>

#include "kernels.cuh"
#include "deposit.cuh"
#include "fft3d.cuh"
#include "lightcone.cuh"
#include "pecvel.cuh"
#include "ps.cuh"

namespace mx {

namespace {
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int g_launches = 0;

constexpr float REL_TOL = 1e-5f;
constexpr float ABS_TOL = 1e-8f;
constexpr double PI_D = 3.14159265358979323846;
constexpr double FRACT_FLOAT_ERR = 1e-7;
constexpr int RR_Z_NPTS = 300;
constexpr int RR_LNG_NPTS = 150;
constexpr float RR_DEL_Z = 0.2f;
constexpr float RR_DEL_LNG = 0.1f;
constexpr double RR_LNG_MIN = -10.0;

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

// cells whose loads a grid-stride loop issues together
constexpr int CELL_BATCH = 4;

__device__ __forceinline__ long long pad_of(long long ir, int D, int H)
{
  const long long row = row_of(ir, D);
  return ir - row * D + row * 2LL * H;
}

}  // namespace

// grad_sfr (PADDED) += alpha_half * (v (PADDED, may be NULL) + u0 (REAL, may be
// NULL)) at the cells; alpha_half = a_first for padded indices below D*D*(D/2+1)
// (the half of the array the SFR-history scalings touch), else a_second.
__global__ void k_adjoint_axpy(float* __restrict__ grad, const float* __restrict__ v, const float* __restrict__ u0,
                               float a_first, float a_second, int D, int H, long long N, long long C)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    const long long ip = row * 2LL * H + (ir - row * D);
    float x = 0.0f;
    if (v)
      x += v[ip];
    if (u0)
      x += u0[ir];
    grad[ip] += (ip < C ? a_first : a_second) * x;
  }
}

void launch_adjoint_axpy(float* grad, const float* v, const float* u0, float a_first, float a_second,
                         const GridDims& gd, cudaStream_t s)
{
  k_adjoint_axpy<<<RED_BLOCKS, RED_THREADS, 0, s>>>(grad, v, u0, a_first, a_second, gd.D, gd.H, gd.N, gd.C);
  g_launches++;
}

int kernel_launch_count()
{
  return g_launches + ts_kernel_launches() + fft_kernel_launches() + ps_kernel_launches() + pecvel_kernel_launches() +
         lightcone_kernel_launches() + deposit_kernel_launches();
}
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
            w = tophat_weight(kR);
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
      float nr = 0.0f, xe = 0.0f;
      if (a.recomb) {
        nr = fmaxf(field(a.idx_nr), 0.0f);
        if (nr < ABS_TOL)
          nr = 0;
      }
      if (a.spin) {
        xe = fmaxf(field(a.idx_xe), 0.0f);
        if (xe < ABS_TOL)
          xe = 0;
        xe = fminf(xe, 0.999f);
      }
      // FP32 evaluation of the criterion f_coll*eff > nf*(1+rec); when the two
      // sides are within 4e-6 of each other (a few float roundings), the
      // decision and the partial xH are recomputed in FP64 as the reference
      // writes them (find_HII_bubbles.c:348-428).
      const float domf = 1.0f + dx;
      const float lhs_f = st * rp.kfc / domf;
      const float nf_f = 1.0f - xe;
      const float rhs_f = nf_f * (1.0f + nr / domf);
      bool ionised;
      float xpart;
      if (fabsf(lhs_f - rhs_f) > 4e-6f * fmaxf(lhs_f, rhs_f)) {
        ionised = lhs_f > rhs_f;
        xpart = nf_f - lhs_f;
      } else {
        const double dom = 1.0 + (double)dx;
        const double rec = a.recomb ? (double)nr / dom : 0.0;
        const double nf = a.spin ? 1.0 - (double)xe : 1.0;
        const double f_coll = (double)st / (rp.M_mean * dom) * (4.0 / 3.0) * PI_D * rp.R_cubed / a.pixel_volume;
        ionised = f_coll * a.eff > nf * (1. + rec);
        xpart = (float)__dsub_rn(nf, __dmul_rn(f_coll, a.eff));
      }
      const float J21_aux = a.uvb ? ws * rp.kj : 0.0f;
      if (ionised) {
        if (xH > REL_TOL) {
          if (a.uvb)
            J21 = J21_aux;
          if (a.recomb)
            G12 = ws * rp.kg;
        }
        xH = 0.0f;
        rb = (float)rp.R;
      } else if (rp.last && (xH > REL_TOL)) {
        xH = xpart;
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
  CSum sum[4];
  // the lnGamma nodes of the recombination table, searched per cell
  __shared__ float rr_x[RR_LNG_NPTS];
  for (int i = threadIdx.x; i < RR_LNG_NPTS; i += blockDim.x)
    rr_x[i] = a.recomb ? a.rr_xf[i] : 0.0f;
  __syncthreads();
  // RR_DEL_LNG * RR_LNG_NPTS is a float product in recombinations.c:46
  const double lng_top = RR_LNG_MIN + (double)(RR_DEL_LNG * (float)RR_LNG_NPTS);
  const float dNfac = a.fabs_dtdz * a.zstep;
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long ip = pad_of(ir, D, H);
    const float xHf = a.xH[ir];
    const float dxf = a.deltax[ip];
    const float j21 = a.uvb ? a.J21[ir] : 0.0f;
    const float g12 = a.recomb ? a.Gamma12[ir] : 0.0f;
    sum[0].add(xHf);
    if (a.uvb)
      sum[1].add(j21);
    const float domf = 1.0f + dxf;
    sum[2].add(xHf * domf);
    sum[3].add(domf);
    // dNrec is exactly zero for neutral cells and for Gamma12 = 0 (log -> -inf)
    if (a.recomb && xHf < 1.0f && g12 > 0.0f) {
      // FP32 lookup of splined_recombination_rate (recombinations.c:30-52);
      // the redshift bin and the lower lnGamma cut are decided in FP64 when
      // FP32 lands within rounding of a bin edge
      const float zf = (1.0f + (float)a.redshift) * cbrtf(1.0f + dxf) - 1.0f;
      const float qf = zf / RR_DEL_Z + 0.5f;
      int z_ct;
      if (fabsf(qf - rintf(qf)) > 2e-4f) {
        z_ct = (int)qf;
      } else {
        const float z_eff = (float)__dsub_rn(__dmul_rn(1. + a.redshift, pow(1.0 + (double)dxf, 1.0 / 3.0)), 1.0);
        z_ct = (int)((double)z_eff / (double)RR_DEL_Z + 0.5);
      }
      z_ct = z_ct < 0 ? 0 : (z_ct >= RR_Z_NPTS ? RR_Z_NPTS - 1 : z_ct);
      float lnG = logf(g12);
      bool below = lnG < (float)RR_LNG_MIN;
      if (fabsf(lnG - (float)RR_LNG_MIN) < 1e-5f)
        below = log((double)g12) < RR_LNG_MIN;
      if (!below) {
        if ((double)lnG >= lng_top)
          lnG = (float)(lng_top - FRACT_FLOAT_ERR);
        const float* x = rr_x;
        const float* y = a.rr_yf + (long long)z_ct * RR_LNG_NPTS;
        const float* c = a.rr_cf + (long long)z_ct * RR_LNG_NPTS;
        float rr;
        if (!(lnG >= x[0] && lnG <= x[RR_LNG_NPTS - 1])) {
          rr = CUDART_NAN_F;  // outside the table (the reference's GSL reports a domain error)
        } else {
          int lo = 0, hi = RR_LNG_NPTS - 1;
          while (hi > lo + 1) {
            const int mid = (lo + hi) >> 1;
            if (x[mid] > lnG)
              hi = mid;
            else
              lo = mid;
          }
          const float h = x[lo + 1] - x[lo], t = lnG - x[lo];
          const float b = (y[lo + 1] - y[lo]) / h - h * (c[lo + 1] + 2.0f * c[lo]) * (1.0f / 3.0f);
          const float d = (c[lo + 1] - c[lo]) / (3.0f * h);
          rr = y[lo] + t * (b + t * (c[lo] + t * d));
        }
        a.N_rec[ip] = a.N_rec[ip] + rr * a.rr_scale_inv * dNfac * (1.0f - xHf);
      }
    }
  }
  double acc[4] = { sum[0].value(), sum[1].value(), sum[2].value(), sum[3].value() };
  block_reduce_store<4>(acc, a.partials);
}

void launch_fhb_reduce(const FhbReduceArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_fhb_reduce<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

__global__ void k_finalize(const double* __restrict__ partials, int nvals, int nblocks, double* __restrict__ out)
{
  // one thread per value, fixed summation order over blocks
  const int v = threadIdx.x;
  if (v < nvals) {
    double s = 0.0;
    for (int b = 0; b < nblocks; b++)
      s += partials[(long long)b * nvals + v];
    out[v] = s;
  }
}

void launch_finalize(const double* partials, int nvals, double* out, cudaStream_t s, int nblocks)
{
  k_finalize<<<1, 32, 0, s>>>(partials, nvals, nblocks, out);
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
  CSum sum[2];
  // per-cell collapse fraction in FP32, volume sums compensated (CSum); the
  // loads of CELL_BATCH cells of a thread's stride are issued together
  const float kcf = (float)((4.0 / 3.0) * PI_D * a.R3 / a.pixel_volume / a.RtoM_h2);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long ir0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir0 < N; ir0 += CELL_BATCH * stride) {
    float st[CELL_BATCH], dx[CELL_BATCH], xe[CELL_BATCH];
#pragma unroll
    for (int u = 0; u < CELL_BATCH; u++) {
      const long long ir = ir0 + u * stride;
      if (ir < N) {
        const long long ip = pad_of(ir, D, H);
        st[u] = a.stars[ip];
        dx[u] = a.deltax[ip];
        xe[u] = a.x_e_prev[ip];
      }
    }
#pragma unroll
    for (int u = 0; u < CELL_BATCH; u++) {
      if (ir0 + u * stride < N) {
        sum[0].add(fminf(st[u] * kcf / (1.0f + dx[u]), 1.0f));
        sum[1].add(xe[u]);
      }
    }
  }
  double acc[2] = { sum[0].value(), sum[1].value() };
  block_reduce_store<2>(acc, a.partials);
}
void launch_cf_xe(const CfArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_cf_xe<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

__global__ void k_ts_means(const float* TS, const float* Tk, double* partials, long long N)
{
  CSum sum[2];
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    sum[0].add(TS[ir]);
    sum[1].add(Tk[ir]);
  }
  double acc[2] = { sum[0].value(), sum[1].value() };
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
  CSum sum;
  // the loads of CELL_BATCH cells of a thread's stride are issued together
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long ir0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir0 < N; ir0 += CELL_BATCH * stride) {
    float xh[CELL_BATCH], dx[CELL_BATCH], ts[CELL_BATCH];
#pragma unroll
    for (int u = 0; u < CELL_BATCH; u++) {
      const long long ir = ir0 + u * stride;
      if (ir < N) {
        xh[u] = a.xH[ir];
        dx[u] = a.deltax[pad_of(ir, D, H)];
        ts[u] = a.spin ? a.TS[ir] : 1.0f;
      }
    }
#pragma unroll
    for (int u = 0; u < CELL_BATCH; u++) {
      const long long ir = ir0 + u * stride;
      if (ir < N) {
        float dT = a.const_factor * xh[u] * (1.0f + dx[u]);
        if (a.spin) {
          if (a.pecvel > 1)
            dT = dT * ((1.0f + a.redshift) / (1000.0f * ts[u]));
          else
            dT = dT * (1.0f - a.T_rad_f / ts[u]);
        }
        a.delta_T[ir] = dT;
        sum.add(dT);
      }
    }
  }
  double acc[1] = { sum.value() };
  block_reduce_store<1>(acc, a.partials);
}
void launch_delta_T(const DeltaTArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_delta_T<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  g_launches++;
}

}  // namespace mx
