// 21 cm power spectrum kernels (see ps.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mx {

constexpr int PS_MAX_BINS = 48;

struct PsArgs
{
  const float2* spec;          // half spectrum [D][D][D/2+1] of the field
  int D;
  int nb;                      // bins
  float edges[PS_MAX_BINS + 1];  // edges[0] = 0, edges[b + 1] = ceiling of bin b
  float delta_k;
  float volume;                // (box / h)^3 in Mpc^3, as float
  double* partials;            // RED_BLOCKS x 3 x nb: sum P, sum |k|, count
};

void launch_ps_mean(const float* dT, long long N, double* partials, double* sum, cudaStream_t s);
void launch_ps_field(const float* dT, const double* sum, float volume, const GridDims& gd, float* out, cudaStream_t s);
void launch_ps_bin(const PsArgs& a, double* sums, cudaStream_t s);
// power-spectrum loss: f = dT * scale (padded), gradient spectrum (in place:
// Y_k = coef[bin] k^3 X_k, doubled on the kz = 0, D/2 planes), REAL = padded * scale
void launch_ps_scale(const float* dT, float scale, const GridDims& gd, float* out, cudaStream_t s);
void launch_ps_loss_grad(const PsArgs& a, const double* coef, float2* spec, cudaStream_t s);
void launch_padded_to_real(const float* in, float scale, const GridDims& gd, float* out, cudaStream_t s);
int ps_kernel_launches();

}  // namespace mx
