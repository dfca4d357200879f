// Fused 3-D transforms for power-of-two grids and grids with a factor 3
// (see fft3d.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mx {

// x-pass: filter + 1/N scale + inverse FFT along x for a batch of radii.
struct XPassArgs
{
  const float2* in[MAX_FIELDS];  // unfiltered, unnormalised half spectra, rows of fft_pitch(D)
  int G;                          // fields
  int n;                          // radii in the batch
  float2* out;                    // spectrum (r*G + g) at out + (r*G + g)*C
  long long C;                    // D * D * fft_pitch(D)
  float R[MAX_RADII];
  int apply[MAX_RADII];
  int filter_type;
  float delta_k;
  float scale;       // 1/N (exact for power-of-two N)
  float sharpk_max;  // set by launch_fft_x_filter
};

// Forward R2C of G padded real grids into spectra [kx][ky][kz] with rows of
// fft_pitch(D) complex values (the x-pass's input layout).
struct FwdArgs
{
  const float* src[MAX_FIELDS];  // PADDED real grids (8-byte aligned)
  int G;
  float2* out;  // spectrum g at out + g * C
  long long C;  // D * D * fft_pitch(D)
};

// z-pass fused with the find_HII_bubbles per-cell test.
struct ZThresholdArgs
{
  const float2* spectra;  // batch spectra after the x and y passes
  long long C;
  int G, idx_xe, idx_nr;  // fields deltax, stars, weighted_sfr, [x_e if spin], [N_rec if recomb]
  int n_r;  // radii of the batch
  int n_f;  // of which filtered (spectra r*G + g for r < n_f); a last radius
            // with rp.last set reads the input grids directly
  const RadiusParams* rp;
  const float* direct[MAX_FIELDS];  // PADDED input grids for the unfiltered step
  float* xH;
  float* z_at_ion;
  float* r_bubble;
  float* J21;
  float* J21_at_ion;
  float* Gamma12;
  double pixel_volume, eff, redshift;
  float gamma_halo_bias;
  int uvb, recomb, spin;
  unsigned* err;  // bit 2: a pipeline wait timed out
  // row groups [group0, group0 + n_groups) of fft_z_row_groups(D) (n_groups
  // 0: all), so that a launch can cover a slab of rows
  int group0 = 0, n_groups = 0;
  // register budget of the launch: 2 or 3 resident blocks per SM
  int blocks_per_sm = 2;
};

bool fft3d_supported(int D);
// Row pitch (complex values) of the spectra between the fused passes: D/2 + 1
// rounded up to whole 128-byte lines.  A batch spectrum holds D * D * pitch.
int fft_pitch(int D);
// acc = (first ? 0 : acc) + W(|k| R) * scale * U on a half spectrum (any D);
// the filter of the x-pass
void launch_filter_accumulate(int D, float2* acc, const float2* U, float R, int filter_type, float delta_k,
                              float scale, bool first, cudaStream_t s);
// threads per block of the x- and y-pass: 256 or 512
bool launch_fft_x_filter(int D, const XPassArgs& a, int threads, cudaStream_t s);
bool launch_fft_y(int D, float2* data, long long C, int n_spectra, int threads, cudaStream_t s);
// three launches: z (real rows -> half spectrum), y, x; threads of the y and
// x passes 256 or 512
bool launch_fft_forward(int D, const FwdArgs& a, int threads, cudaStream_t s);
bool launch_fft_z_threshold(int D, const ZThresholdArgs& a, cudaStream_t s);
bool launch_fft_z_store(int D, const float2* spectra, long long C, int n, int r0, float* shells, long long N,
                        unsigned* err, cudaStream_t s);
// row groups of the threshold z-pass and rows (x * D + y) per group
int fft_z_row_groups(int D);
int fft_z_rows_per_group(int D);
int fft_kernel_launches();
// Sets the poll limit of this unit's pipeline waits (bulk.cuh).
cudaError_t fft_set_wait_polls(long long polls);

}  // namespace mx
