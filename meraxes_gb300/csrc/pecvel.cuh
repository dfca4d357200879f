// Peculiar-velocity corrections of the brightness temperature (see pecvel.cu).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mx {

constexpr int RSD_STEPS = 50;  // N_RSD_STEPS, reionization.h:34

struct PecvelArgs
{
  const float* grad;  // dv/dx on the padded layout
  float* delta_T;     // REAL
  const float* TS;    // REAL
  int mode;           // Flag_IncludePecVelsFor21cm
  float H_z;
  float redshift;
  double max_v_deriv;  // fabs(MAX_DVDR * H_z)
  double T_rad;
};

struct RsdArgs
{
  const float* vel;      // converted velocities, padded
  const float* delta_T;  // REAL, read
  const float* xH;       // REAL
  float* los;            // REAL scratch (one column per thread)
  float* delta_T_out;    // REAL, receives the remapped columns
  float x_pos[RSD_STEPS], x_pos_offset[RSD_STEPS];
  double box;            // BoxSize / h [Mpc]
  double subcell_width;
  float H_z;
};

void launch_vel_convert(float* vel, int trees_id, float redshift, const GridDims& gd, cudaStream_t s);
void launch_vel_grad_k(float2* spec, const GridDims& gd, double hubble_h, float delta_k, cudaStream_t s);
void launch_pecvel_cells(const PecvelArgs& a, const GridDims& gd, cudaStream_t s);
void launch_rsd(const RsdArgs& a, const GridDims& gd, cudaStream_t s);
int pecvel_kernel_launches();

}  // namespace mx
