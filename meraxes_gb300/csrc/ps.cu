// 21 cm power spectrum of delta_T: Compute_PS (ComputePowerSpectrum.c:44-255).
//
//   1. mean of delta_T (two-stage fixed-order FP64 sum);
//   2. the field (delta_T / mean - 1) * V / N * mean into the padded layout,
//      with the reference's double arithmetic per cell;
//   3. R2C (cuFFT, in mx_reion.cu);
//   4. the binned sums over the half spectrum: every mode (kx, ky, kz <= D/2)
//      is counted once, |k| in float as the reference computes it, bins of
//      ratio 1.35 from delta_k (edges computed on the host in float by the
//      reference's recurrence), k^3 |X|^2 / (2 pi^2 V) and |k| summed in FP64.
//
// The binned sums are deterministic: a warp owns whole rows (kx, ky); lane l
// visits kz = l, l + 32, ... whose |k| increases, so its bin index never
// decreases along a row; it accumulates runs in registers and adds each run
// to its private histogram.  Histograms are reduced per block in a fixed
// order, then over blocks in a fixed order.
#include "ps.cuh"

namespace mx {

namespace {
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int ps_launches = 0;

__global__ void k_ps_sum(const float* __restrict__ dT, long long N, double* partials)
{
  __shared__ double sh[RED_THREADS / 32];
  CSum sum;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    sum.add(dT[i]);
  double acc = sum.value();
  for (int o = 16; o > 0; o >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < RED_THREADS / 32; w++)
      s += sh[w];
    partials[blockIdx.x] = s;
  }
}

// sums[v] = sum over blocks of partials[b * nvals + v], fixed order
__global__ void k_ps_finalize(const double* __restrict__ partials, int nblocks, int nvals, double* __restrict__ sums)
{
  const int v = threadIdx.x;
  if (v < nvals) {
    double s = 0.0;
    for (int b = 0; b < nblocks; b++)
      s += partials[(long long)b * nvals + v];
    sums[v] = s;
  }
}

// ComputePowerSpectrum.c:94-110
__global__ void k_ps_field(const float* __restrict__ dT, const double* __restrict__ sum, double n_cells, float volume,
                           float n_cells_f, int D, int H, long long N, float* __restrict__ out)
{
  const double ave = sum[0] / n_cells;
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    const long long ip = row * 2LL * H + (ir - row * D);
    float v = (float)(((double)dT[ir] / ave - 1) * (double)volume / (double)n_cells_f);
    v = (float)((double)v * ave);
    out[ip] = v;
  }
}

__device__ __forceinline__ float kcomp_ps(int n, int D, float delta_k)
{
  return (n > D / 2) ? __fmul_rn((float)(n - D), delta_k) : __fmul_rn((float)n, delta_k);
}

// ComputePowerSpectrum.c:160-215
__global__ void __launch_bounds__(RED_THREADS) k_ps_bin(PsArgs a)
{
  double hp[PS_MAX_BINS], hk[PS_MAX_BINS], hc[PS_MAX_BINS];
  for (int b = 0; b < a.nb; b++)
    hp[b] = hk[b] = hc[b] = 0.0;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (RED_THREADS / 32);
  const int D = a.D, H = D / 2 + 1;
  const long long rows = (long long)D * D;
  const double pdiv = 2.0 * 3.14159265358979323846 * 3.14159265358979323846 * (double)a.volume;
  for (long long row = blockIdx.x * (RED_THREADS / 32) + (threadIdx.x >> 5); row < rows; row += warps) {
    const int nx = (int)(row / D), ny = (int)(row % D);
    const float kx = kcomp_ps(nx, D, a.delta_k), ky = kcomp_ps(ny, D, a.delta_k);
    // k_x*k_x + k_y*k_y + k_z*k_z in the reference's float operations (no
    // fused multiply-add)
    const float kxy = __fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky));
    const float2* __restrict__ spec = a.spec + row * H;
    int cur = -1;
    double sp = 0.0, sk = 0.0, sc = 0.0;
    for (int nz = lane; nz < H; nz += 32) {
      const float kz = __fmul_rn((float)nz, a.delta_k);
      // (float)sqrt((double)s) of the reference equals sqrtf(s): the double
      // square root of a float has enough bits that rounding it again to
      // float gives the correctly rounded float root
      const float kmag = sqrtf(__fadd_rn(kxy, __fmul_rn(kz, kz)));
      int b = -1;
      if (kmag < a.edges[a.nb]) {
        b = 0;
        while (!(kmag < a.edges[b + 1]))
          b++;
      }
      if (b != cur) {
        if (cur >= 0) {
          hp[cur] += sp;
          hk[cur] += sk;
          hc[cur] += sc;
        }
        cur = b;
        sp = sk = sc = 0.0;
      }
      if (b >= 0) {
        const float2 X = spec[nz];
        const double k = (double)kmag;
        const double m2 = (double)X.x * (double)X.x + (double)X.y * (double)X.y;
        sp += k * k * k * m2 / pdiv;
        sk += k;
        sc += 1.0;
      }
    }
    if (cur >= 0) {
      hp[cur] += sp;
      hk[cur] += sk;
      hc[cur] += sc;
    }
  }
  // block reduction per bin, fixed order: lanes by shuffles, warps in order
  __shared__ double sh[3][RED_THREADS / 32];
  const int warp = threadIdx.x >> 5;
  for (int b = 0; b < a.nb; b++) {
    double v[3] = { hp[b], hk[b], hc[b] };
#pragma unroll
    for (int q = 0; q < 3; q++) {
      for (int o = 16; o > 0; o >>= 1)
        v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
      if (lane == 0)
        sh[q][warp] = v[q];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      double s = 0.0;
      for (int w = 0; w < RED_THREADS / 32; w++)
        s += sh[threadIdx.x][w];
      a.partials[(long long)blockIdx.x * 3 * a.nb + threadIdx.x * a.nb + b] = s;
    }
    __syncthreads();
  }
}
// f = dT * scale into the padded layout (the power-spectrum loss field)
__global__ void k_ps_scale(const float* __restrict__ dT, float scale, int D, int H, long long N, float* __restrict__ out)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    out[row * 2LL * H + (ir - row * D)] = dT[ir] * scale;
  }
}

// Gradient spectrum of the binned loss: Y_k = coef[b] k^3 X_k on the modes of
// bin b (the binning of k_ps_bin), times 2 on the kz = 0 and kz = D/2 planes,
// which a C2R counts once where it counts the others twice.  In place.
__global__ void k_ps_loss_grad(PsArgs a, const double* __restrict__ coef, float2* __restrict__ spec)
{
  const int D = a.D, H = D / 2 + 1;
  const long long n = (long long)D * D * H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int nz = (int)(i % H);
    const long long row = i / H;
    const int nx = (int)(row / D), ny = (int)(row % D);
    const float kx = kcomp_ps(nx, D, a.delta_k), ky = kcomp_ps(ny, D, a.delta_k);
    const float kz = __fmul_rn((float)nz, a.delta_k);
    const float kmag = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz)));
    float f = 0.0f;
    if (kmag < a.edges[a.nb]) {
      int b = 0;
      while (!(kmag < a.edges[b + 1]))
        b++;
      const double k = (double)kmag;
      f = (float)(coef[b] * k * k * k * ((nz == 0 || 2 * nz == D) ? 2.0 : 1.0));
    }
    float2 x = spec[i];
    spec[i] = make_float2(x.x * f, x.y * f);
  }
}

// REAL out = PADDED in * scale
__global__ void k_padded_to_real(const float* __restrict__ in, float scale, int D, int H, long long N,
                                 float* __restrict__ out)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    out[ir] = in[row * 2LL * H + (ir - row * D)] * scale;
  }
}
}  // namespace

void launch_ps_mean(const float* dT, long long N, double* partials, double* sum, cudaStream_t s)
{
  k_ps_sum<<<RED_BLOCKS, RED_THREADS, 0, s>>>(dT, N, partials);
  k_ps_finalize<<<1, 32, 0, s>>>(partials, RED_BLOCKS, 1, sum);
  ps_launches += 2;
}

void launch_ps_field(const float* dT, const double* sum, float volume, const GridDims& gd, float* out, cudaStream_t s)
{
  const double n = (double)gd.N;
  k_ps_field<<<RED_BLOCKS, RED_THREADS, 0, s>>>(dT, sum, n, volume, (float)n, gd.D, gd.H, gd.N, out);
  ps_launches++;
}

void launch_ps_bin(const PsArgs& a, double* sums, cudaStream_t s)
{
  k_ps_bin<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a);
  k_ps_finalize<<<1, 3 * PS_MAX_BINS, 0, s>>>(a.partials, RED_BLOCKS, 3 * a.nb, sums);
  ps_launches += 2;
}

void launch_ps_scale(const float* dT, float scale, const GridDims& gd, float* out, cudaStream_t s)
{
  k_ps_scale<<<RED_BLOCKS, RED_THREADS, 0, s>>>(dT, scale, gd.D, gd.H, gd.N, out);
  ps_launches++;
}

void launch_ps_loss_grad(const PsArgs& a, const double* coef, float2* spec, cudaStream_t s)
{
  k_ps_loss_grad<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, coef, spec);
  ps_launches++;
}

void launch_padded_to_real(const float* in, float scale, const GridDims& gd, float* out, cudaStream_t s)
{
  k_padded_to_real<<<RED_BLOCKS, RED_THREADS, 0, s>>>(in, scale, gd.D, gd.H, gd.N, out);
  ps_launches++;
}

int ps_kernel_launches() { return ps_launches; }

}  // namespace mx
