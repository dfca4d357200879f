// Galaxy -> grid deposit and the Mvir_crit grid (see deposit.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mx {

struct DepositArgs
{
  int n;                 // galaxies
  const float* pos;      // [n][3], Mpc/h
  const int* type;       // galaxies of type > 2 are skipped
  const double* fesc_gsm;
  const double* gross_sm;  // read only with the sfr grid
  const double* bhm;       // read only with BH feedback
  const double* ebhm;
  int flag_bh;
  double bh_limit;
  double alpha_uv_bh;
  double alpha_uv;
  double box_size;
  int spin;              // also deposit the sfr grid and its history slice 0
  double sfr_timescale;  // internal time units
  unsigned* keys_in;     // [n] REAL cell index, or the number of cells (skipped)
  unsigned* keys;        // [n] sorted
  int* idx_in;           // [n]
  int* idx;              // [n] sorted
  float* buf_stars;      // REAL scratch, zeroed by launch_deposit
  float* buf_wsfr;
  float* buf_sfr;
  unsigned* err;         // bit 4: a galaxy below the box
  float* stars;          // PADDED outputs
  float* weighted_sfr;
  float* sfr;
  float* sfr_hist0;      // newest history slice, or NULL
};

constexpr unsigned DEPOSIT_ERR_BELOW_BOX = 4u;

// CUB temporary storage for sorting n galaxies (bytes)
size_t deposit_sort_bytes(int n);
// Zeroes the REAL scratch, sorts, sums and writes the padded grids.
cudaError_t launch_deposit(const DepositArgs& a, void* sort_tmp, size_t sort_bytes, const GridDims& gd,
                           cudaStream_t s);
// sm = {m0, a, b, c, d} of the Sobacchi & Mesinger (2013) fit
void launch_Mvir_crit(double redshift, const double sm[5], double hubble_h, const float* J21_at_ion,
                      const float* z_at_ion, float* out, const GridDims& gd, cudaStream_t s);
int deposit_kernel_launches();

}  // namespace mx
