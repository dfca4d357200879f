// Galaxy -> grid deposit: construct_baryon_grids (reionization.c:1353-1615)
// on one rank without mini-haloes; and calculate_Mvir_crit
// (physics/reionization.c:10-59).
//
// The reference adds each galaxy's mass into its nearest-grid-point cell in
// galaxy order, float += double.  For the same float sums the GPU sorts the
// (cell, galaxy) pairs with a stable radix sort (CUB), so that a cell's
// galaxies are adjacent and in their original order; one thread per run of
// equal cells then adds them with the reference's roundings.  A last pass
// writes the padded grids: stars clamped at 0, the SFR grids divided by the
// SFR timescale in double.
#include <cub/device/device_radix_sort.cuh>

#include "deposit.cuh"

namespace mx {

namespace {
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int dep_launches = 0;

int key_bits(long long n_cells)
{
  int b = 1;
  while ((1LL << b) <= n_cells)
    b++;
  return b;  // holds 0 .. n_cells
}

// pos_to_ngp (misc_tools.c:163-173): nearest grid point, the top face wraps
__device__ __forceinline__ int ngp(float x, double side, int nx)
{
  int ind = (int)rint(__dmul_rn(__ddiv_rn((double)x, side), (double)nx));
  if (ind > nx - 1)
    ind = 0;
  return ind;
}

__global__ void k_gal_keys(DepositArgs a, int D, unsigned skip)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n)
    return;
  unsigned key = skip;
  if (a.type[i] <= 2) {
    const int ix = ngp(a.pos[3LL * i], a.box_size, D), iy = ngp(a.pos[3LL * i + 1], a.box_size, D),
              iz = ngp(a.pos[3LL * i + 2], a.box_size, D);
    if (ix < 0 || iy < 0 || iz < 0)
      atomicOr(a.err, DEPOSIT_ERR_BELOW_BOX);
    else
      key = (unsigned)(((long long)ix * D + iy) * D + iz);
  }
  a.keys_in[i] = key;
  a.idx_in[i] = i;
}

// one thread per first galaxy of a run of equal cells in the sorted keys
__global__ void k_cell_sums(DepositArgs a, unsigned skip)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n)
    return;
  const unsigned key = a.keys[j];
  if (key == skip || (j > 0 && a.keys[j - 1] == key))
    return;
  float st = 0.0f, ws = 0.0f, sf = 0.0f;
  for (int q = j; q < a.n && a.keys[q] == key; q++) {
    const int g = a.idx[q];
    const bool bh = a.flag_bh && a.bhm[g] >= a.bh_limit;
    // buffer[ind] += <double>: the float is widened, added, rounded back
    st = (float)__dadd_rn((double)st, a.fesc_gsm[g]);
    if (bh)
      st = (float)__dadd_rn((double)st, a.ebhm[g]);
    ws = (float)__dadd_rn((double)ws, a.fesc_gsm[g]);
    if (bh)
      ws = (float)__dadd_rn((double)ws, __ddiv_rn(__dmul_rn(a.ebhm[g], a.alpha_uv_bh), a.alpha_uv));
    if (a.spin)
      sf = (float)__dadd_rn((double)sf, a.gross_sm[g]);
  }
  a.buf_stars[key] = st;
  a.buf_wsfr[key] = ws;
  if (a.spin)
    a.buf_sfr[key] = sf;
}

// padded outputs from the REAL sums; the padding columns become 0
__global__ void k_deposit_grids(DepositArgs a, int D, int H, long long P)
{
  for (long long ip = blockIdx.x * (long long)blockDim.x + threadIdx.x; ip < P;
       ip += (long long)gridDim.x * blockDim.x) {
    const long long row = ip / (2LL * H);
    const int z = (int)(ip - row * 2LL * H);
    float st = 0.0f, ws = 0.0f, sf = 0.0f;
    if (z < D) {
      const long long ir = row * D + z;
      st = a.buf_stars[ir];
      if (st < 0)
        st = 0;
      double v = (double)a.buf_wsfr[ir];
      ws = (float)((v > 0) ? __ddiv_rn(v, a.sfr_timescale) : 0.0);
      if (a.spin) {
        v = (double)a.buf_sfr[ir];
        sf = (float)((v > 0) ? __ddiv_rn(v, a.sfr_timescale) : 0.0);
      }
    }
    a.stars[ip] = st;
    a.weighted_sfr[ip] = ws;
    if (a.spin) {
      a.sfr[ip] = sf;
      // the reference writes the newest history slice at the cells only
      if (a.sfr_hist0 && z < D)
        a.sfr_hist0[ip] = sf;
    }
  }
}

// physics/reionization.c:38-52, per cell in double
__global__ void k_Mvir_crit(double redshift, double m0, double sa, double sb, double sc, double sd, double hubble_h,
                            const float* __restrict__ J21, const float* __restrict__ zion, float* __restrict__ out,
                            long long N)
{
  const double zfac = pow((1.0 + redshift) / 10.0, sb);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    double cell = 0.0;
    const double zi = (double)zion[i];
    if (zi > redshift) {
      const double j = __dmul_rn(__dmul_rn((double)J21[i], hubble_h), hubble_h);
      cell = __dmul_rn(__dmul_rn(__dmul_rn(m0, pow(j, sa)), zfac),
                       pow(1.0 - pow((1.0 + redshift) / (1.0 + zi), sc), sd));
    }
    out[i] = (float)cell;
  }
}
}  // namespace

size_t deposit_sort_bytes(int n)
{
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const unsigned*)nullptr, (unsigned*)nullptr, (const int*)nullptr,
                                  (int*)nullptr, n > 0 ? n : 1);
  return bytes;
}

cudaError_t launch_deposit(const DepositArgs& a, void* sort_tmp, size_t sort_bytes, const GridDims& gd,
                           cudaStream_t s)
{
  const unsigned skip = (unsigned)gd.N;
  cudaError_t e = cudaMemsetAsync(a.buf_stars, 0, sizeof(float) * gd.N, s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(a.buf_wsfr, 0, sizeof(float) * gd.N, s);
  if (e == cudaSuccess && a.spin)
    e = cudaMemsetAsync(a.buf_sfr, 0, sizeof(float) * gd.N, s);
  if (e != cudaSuccess)
    return e;
  if (a.n > 0) {
    const int blocks = (a.n + 255) / 256;
    k_gal_keys<<<blocks, 256, 0, s>>>(a, gd.D, skip);
    size_t bytes = sort_bytes;
    e = cub::DeviceRadixSort::SortPairs(sort_tmp, bytes, a.keys_in, a.keys, a.idx_in, a.idx, a.n, 0,
                                        key_bits(gd.N), s);
    if (e != cudaSuccess)
      return e;
    k_cell_sums<<<blocks, 256, 0, s>>>(a, skip);
    dep_launches += 2;
  }
  k_deposit_grids<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.P);
  dep_launches++;
  return cudaGetLastError();
}

void launch_Mvir_crit(double redshift, const double sm[5], double hubble_h, const float* J21_at_ion,
                      const float* z_at_ion, float* out, const GridDims& gd, cudaStream_t s)
{
  k_Mvir_crit<<<RED_BLOCKS, RED_THREADS, 0, s>>>(redshift, sm[0], sm[1], sm[2], sm[3], sm[4], hubble_h, J21_at_ion,
                                                 z_at_ion, out, gd.N);
  dep_launches++;
}

int deposit_kernel_launches() { return dep_launches; }

}  // namespace mx
