// Device kernels of the reionization grid step and their launch helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mx {

// Reduction blocks used by every deterministic two-stage FP64 reduction.
constexpr int RED_BLOCKS = 608;  // 4 x 152 SMs
constexpr int RED_THREADS = 256;

// ir / D for a non-negative cell index: a 32-bit division while the index
// fits in 32 bits (every grid up to 1625^3), which costs a fraction of the
// emulated 64-bit one
// Real-space top-hat weight W(x) of the filter, x = kR > 1e-4 (reionization.c
// :2130-2140): the reference's float expression
// 3 (sinf(x) / powf(x, 3) - cosf(x) / powf(x, 2)).  Both terms are about
// 1/x^2 and their difference about 1/3, so for small x an ulp of sin, cos or
// a power becomes about 3/x^2 ulp of W (at the lowest modes of the smallest
// radii, x ~ 0.01, a relative 1e-3 of W, enough to move near-threshold cells
// by 1e-4 of their ratio).  Below x = 1 the expression is therefore evaluated
// as written, with sin and cos computed in double and rounded once to float
// (the correctly rounded values, which a host libm returns to within its last
// bit) and x^2, x^3 rounded from double; above, where the amplification is
// below 3, one sincosf and a reciprocal.
__device__ __forceinline__ float tophat_weight(float x)
{
  if (x < 1.0f) {
    const double xd = x;
    const float s = (float)sin(xd), c = (float)cos(xd);
    const float p3 = (float)(xd * xd * xd), p2 = (float)(xd * xd);
    return (float)(3.0 * (double)__fsub_rn(__fdiv_rn(s, p3), __fdiv_rn(c, p2)));
  }
  float s, c;
  sincosf(x, &s, &c);
  const float inv = __fdividef(1.0f, x);
  return 3.0f * (s * inv - c) * inv * inv;
}

__device__ __forceinline__ long long row_of(long long ir, int D)
{
  return ir < 4294967296LL ? (long long)((unsigned)ir / (unsigned)D) : ir / D;
}

// A thread's running sum of float terms as an unevaluated pair hi + lo
// (Neumaier's compensated summation, error O(n eps^2) of the sum of |terms|):
// as accurate as an FP64 running sum at these lengths, on the FP32 pipe
// (GB300 issues FP64 at a small fraction of the FP32 rate).  value() is the
// FP64 sum that the block and grid reductions (FP64) take.
struct CSum
{
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x)
  {
    const float t = hi + x;
    lo += fabsf(hi) >= fabsf(x) ? (hi - t) + x : (x - t) + hi;
    hi = t;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
constexpr int MAX_FIELDS = 5;
constexpr int MAX_SHELLS = 64;
constexpr int MAX_RADII = 256;

struct GridDims
{
  int D;       // cells per side
  int H;       // D/2 + 1
  long long C; // complex elements D*D*H
  long long N; // cells D^3
  long long P; // padded reals 2*C
};

// ------------------------------------------------------------ k-space filter
// Per-radius parameters of a filtered batch.
struct FilterBatch
{
  int n;                   // radii in the batch
  int filter_type;         // 0 tophat, 1 sharp-k, 2 Gaussian
  int scale_mode;          // 0: (float)((double)v / N); 1: v / (float)N
  float R[MAX_RADII];      // (float)R per radius
  int apply[MAX_RADII];    // 0 on the unfiltered last step
};

// out[(r*G + g)] = filter_r(scale(in[g])) for every complex element.
void launch_filter(const float2* const* in, int G, float2* out, long long out_field_stride, const FilterBatch& fb,
                   const GridDims& gd, float box_size, cudaStream_t s);

// ---------------------------------------------------------- threshold loop
struct RadiusParams
{
  double R, M_mean, R_cubed, J21_const, Gamma_pref;
  int last;
  // FP32 fast path: f_coll*eff = st * kfc / (1+dx); J21_aux = ws * kj;
  // Gamma12 = ws * kg
  float kfc, kj, kg;
};
struct ThresholdArgs
{
  const float* fields;   // batch base: field (r*G + g) at fields + (r*G+g)*P
  long long P;
  int G;                 // fields per radius: dx, stars, wsfr, [x_e], [N_rec]
  int idx_xe, idx_nr;    // field slot or -1
  int n_r;               // radii in this batch
  const RadiusParams* rp; // device array, n_r entries
  // The unfiltered last step is an identity transform: its fields are read
  // from the input grids (PADDED) instead of a transformed copy.
  const float* direct[MAX_FIELDS];
  float* xH;
  float* z_at_ion;
  float* r_bubble;
  float* J21;
  float* J21_at_ion;
  float* Gamma12;
  double pixel_volume, eff, redshift;
  float gamma_halo_bias;
  int uvb, recomb, spin;
};
void launch_threshold(const ThresholdArgs& a, const GridDims& gd, cudaStream_t s);

// ---------------------------------------------------------------- reductions
struct FhbReduceArgs
{
  const float* xH;
  const float* J21;
  const float* deltax;  // PADDED, unfiltered input
  const float* Gamma12;
  float* N_rec;         // PADDED, updated when recomb
  const float* rr_yf;   // recombination table (device, FP32, values scaled
  const float* rr_cf;   // by rr_scale = 1/rr_scale_inv to O(1))
  const float* rr_xf;
  float rr_scale_inv;
  double redshift;
  float fabs_dtdz, zstep;
  int uvb, recomb;
  double* partials;     // RED_BLOCKS x 4
};
void launch_fhb_reduce(const FhbReduceArgs& a, const GridDims& gd, cudaStream_t s);
// Sums `nvals` columns of a RED_BLOCKS x nvals partials array in fixed order.
// out[v] = sum over the first nblocks blocks' partials (fixed order)
void launch_finalize(const double* partials, int nvals, double* out, cudaStream_t s, int nblocks = RED_BLOCKS);

// ------------------------------------------------------------ grid helpers
void launch_fill(float* p, long long n, float v, cudaStream_t s);
void launch_fill_real_in_padded(float* p, const GridDims& gd, float v, cudaStream_t s);

// ---------------------------------------------------------------- ComputeTs
// SFR-history operations on the PADDED sfr grid (ComputeTs.c:288-377).
void launch_sfr_scale_half(float* sfr, long long nhalf, double w, cudaStream_t s);
void launch_sfr_zero_half(float* sfr, long long nhalf, cudaStream_t s);
void launch_sfr_load(float* sfr, const float* slice, float w, int accumulate, const GridDims& gd, cudaStream_t s);

// Shell value extraction: shells[r*N + real] = max(filtered_real, 0).
void launch_shell_extract(const float* filtered, long long P, int n, int r0, float* shells, const GridDims& gd,
                          cudaStream_t s);

// Collapse fraction and mean x_e of the unsmoothed fields (ComputeTs.c:413-475).
struct CfArgs
{
  const float* stars;
  const float* deltax;
  const float* x_e_prev;
  double RtoM_h2;  // RtoM(R) * h * h
  double R3;       // pow(R, 3.0)
  double pixel_volume;
  double* partials; // RED_BLOCKS x 2
};
void launch_cf_xe(const CfArgs& a, const GridDims& gd, cudaStream_t s);

// Per-cell constants of the spin-temperature update.
struct TsDevConst
{
  int S, no_light;
  float zp;
  double zpd;
  double dzp, dt_dzp, growth, dgrowth, prefactor, conv, p2, p3, n_b0, f_h, f_he, no;
  double pixel_volume, sfr_a, sfr_b, clumping;
  double hubble_z, hubble0_h, h;  // hubble((float)zp), HUBBLE*h, h
  double a[MAX_SHELLS], b[MAX_SHELLS], zpp1[MAX_SHELLS], sum_lyn[MAX_SHELLS], dt_dzpp[MAX_SHELLS],
    dzpp[MAX_SHELLS];
  double tab[3][14][MAX_SHELLS];
  float xhii[14];
  // kappa splines (ln T -> ln kappa)
  int nk[3];
  double kx[3][27], ky[3][27], kc[3][27];

  // FP32 fast path.  The unit and cosmology factors of evolveInt are folded
  // into per-shell coefficients and the frequency tables are rescaled per
  // (table, shell) by powers of two, so that every float stays far from the
  // float range limits:
  //   dxheat_dzp * (1+x_e) = sum_r sf_r * fKH[r] * lerp(ftab[0][.][r], x_e)
  //   dt_dzp * dxion_src   = sum_r sf_r * fKI[r] * lerp(ftab[1][.][r], x_e)
  //   dxlya_dt / (1+delta) = sum_r sf_r * fKL[r] * lerp(ftab[2][.][r], x_e)
  //   dstarlya_dt          = sum_r sf_r * fKS[r]
  float fKH[MAX_SHELLS], fKI[MAX_SHELLS], fKL[MAX_SHELLS], fKS[MAX_SHELLS];
  float ftab[3][14][MAX_SHELLS];
  float fksink;   // dt_dzp * CLUMPING * f_H * N_b0 * (1+zp)^3
  float fadia0;   // 3 / (1+zp)
  float fdgrowth, fgrowth;
  float fccomp;   // dT_comp prefactor without x_e/(1+x_e+f_He) (Trad - T)
  float ftrad, ff_he, fdzp, ftk_floor;
  float fxc[3];   // T21/Trad * {No, N_b0, No} * (1+z)^3 / A10
  float ftgp;     // 1.342881e-7 / H(z) * No * (1+z)^3
  float fxa;      // 1.66e11 / (1+z)
  float fkx[3][27], fky[3][27], fkc[3][27];
};

struct EvolveArgs
{
  const float* shells;  // S x N
  const float* deltax;  // PADDED
  float* x_e_prev;      // PADDED
  float* Tk;            // REAL
  float* TS;            // REAL
  const TsDevConst* cst;  // device copy
  double* partials;       // RED_BLOCKS x 4 (J_alpha, xalpha, Xheat, Xion)
  unsigned int* err;      // error word: bit 1 iteration cap, bit 2 a shell-copy wait timed out
  int n_shells;           // S of *cst (sizes the shared-memory shell ring)
};
// shell_map: 2-D tensor map of the shells (cells x shells, box EV_TILE x S;
// ev_shell_map_ok() says when one applies), or nullptr for one bulk copy per
// shell row
bool ev_shell_map_ok(long long N, int S);
// returns the number of blocks (of partial sums) launched
int launch_evolve(const EvolveArgs& a, const GridDims& gd, const void* shell_map, cudaStream_t s);

// Adjoint of the per-cell spin-temperature update and of the 21cm box.
struct AdjointArgs
{
  float* shells;          // S x N: shell values in, dL/d(shell) out
  const float* deltax;    // PADDED
  const float* x_e_prev;  // PADDED, state before the step
  const float* Tk;        // REAL, state before the step
  const float* x_e_new;   // PADDED, x_e after the step (x_e_box)
  const float* stars;     // PADDED, as find_HII_bubbles read it
  const float* xH;        // REAL, after the step
  const float* TS;        // REAL, after the step
  const float* grad_dT;   // REAL, dL/d(delta_T)
  float* grad_stars;      // PADDED, dL/d(stars) at the cells (padding untouched)
  const TsDevConst* cst;
  const float4* dP_dE0;   // 14 x S: d/dE0 of (K_H tab_H, K_I tab_I, K_L tab_L, -)
  float dT_factor;        // 21cm box constant
  float dT_trad;          // T_CMB (1 + z) of the 21cm box
  float kfc_last;         // f_coll * eff = stars * kfc_last / (1 + dx) at the last step
  double* partials;       // RED_BLOCKS x 2: L_X and E0 terms
  unsigned int* err;
  int n_shells;
};
void launch_evolve_adjoint(const AdjointArgs& a, const GridDims& gd, const void* shell_map, cudaStream_t s);
// grad (PADDED) += alpha * (v (PADDED) + u0 (REAL)) at the cells, alpha = a_first
// on the first D*D*(D/2+1) floats of the padded array, a_second after
void launch_adjoint_axpy(float* grad, const float* v, const float* u0, float a_first, float a_second,
                         const GridDims& gd, cudaStream_t s);

// Homogeneous branch: fill x_e, T_K and compute T_S with J_alpha = 0.
struct HomogArgs
{
  const float* deltax;
  const float* stars;
  float* x_e_prev;
  float* Tk;
  float* TS;
  float xe0, tk0;
  const TsDevConst* cst;
  double RtoM_h2, R3, pixel_volume;
  double* partials;  // RED_BLOCKS x 1 (collapse fraction)
  unsigned int* err;
};
void launch_homog(const HomogArgs& a, const GridDims& gd, cudaStream_t s);

// Means of T_S and T_K (ComputeTs.c:942-974).
void launch_ts_means(const float* TS, const float* Tk, double* partials, const GridDims& gd, cudaStream_t s);

// --------------------------------------------------- brightness temperature
struct DeltaTArgs
{
  const float* deltax;
  const float* xH;
  const float* TS;
  float* delta_T;
  float const_factor;
  float T_rad_f;
  float redshift;
  int spin, pecvel;
  double* partials;  // RED_BLOCKS x 1
};
void launch_delta_T(const DeltaTArgs& a, const GridDims& gd, cudaStream_t s);

int kernel_launch_count();
void reset_kernel_launch_count();
int ts_kernel_launches();
// Sets the poll limit of the evolve kernels' pipeline waits (bulk.cuh).
cudaError_t ts_set_wait_polls(long long polls);

}  // namespace mx
