// Light-cone slices (see lightcone.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mx {

struct LightconeArgs
{
  const float* delta_T;       // REAL, this snapshot
  const float* delta_T_prev;  // REAL, previous snapshot
  float* out;                 // [D*D columns][pitch] floats; slice s of column c at out[c * pitch + s]
  long long pitch;
  const double* t_slice;      // cosmic time of each slice (n)
  int n;                      // slices of this snapshot
  int iz0;                    // z column of the first slice
  double t1, t2;              // times of this and the previous snapshot
};

void launch_lightcone(const LightconeArgs& a, const GridDims& gd, cudaStream_t s);
int lightcone_kernel_launches();

}  // namespace mx
