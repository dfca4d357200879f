// Peculiar-velocity corrections of the 21 cm brightness temperature
// (BrightnessTemperature.c:158-509, velocity_gradient reionization.c:2172-2187),
// used when the spin temperature is on and Flag_IncludePecVelsFor21cm is 1-3:
//
//   k_vel_convert    velocity units in place (trees convention, to comoving
//                    Mpc/s), per cell in FP64 like the reference;
//   (cuFFT R2C of vel, in mx_reion.cu)
//   k_vel_grad_k     1/N and h scale, times i k_z (k from BoxSize in Mpc/h);
//   (cuFFT C2R in place: dv/dx on the padded layout)
//   k_pecvel_cells   mode 1: divide by (dv/dx / H + 1) with |dv/dx| capped at
//                    0.2 H; modes 2-3: optical-depth form
//                    (1 - exp(-tau / |dv/dx / H + 1|)) 1000 (T_S - T_CMB) / (1+z);
//   k_rsd_columns    mode 3: the line-of-sight remap along z.  Each z column
//                    is one thread running the reference's sequential sub-cell
//                    loop (50 sub-cells per cell, FP64 positions, the same
//                    float / double accumulation), so the deposits land in the
//                    same order.
#include "pecvel.cuh"

namespace mx {

namespace {
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int pv_launches = 0;
constexpr double FRACT_FLOAT_ERR_D = 1e-7;
constexpr double MPC_CM = 3.086e24;

__global__ void k_vel_convert(float* vel, int trees_id, float redshift, int D, int H, long long N)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    const long long ip = row * 2LL * H + (ir - row * D);
    float v = vel[ip];
    if (trees_id == 1)
      v = (float)(sqrt(1. / (1. + redshift)) * v / 1000.);
    else if (trees_id == 0 || trees_id == 2)
      v = (float)((1. + redshift) * v);
    v = (float)((double)v * (1000. * 100. / MPC_CM));
    v = (float)(v / (1. / (1. + redshift)));
    vel[ip] = v;
  }
}

// c /= N; c *= h (each in double, rounded to float); c *= (0 + i k_z) as a
// float complex product
__global__ void k_vel_grad_k(float2* spec, int H, long long C, double n_cells, double hubble_h, float delta_k)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < C; i += (long long)gridDim.x * blockDim.x) {
    float2 v = spec[i];
    v.x = (float)((double)v.x / n_cells);
    v.y = (float)((double)v.y / n_cells);
    v.x = (float)((double)v.x * hubble_h);
    v.y = (float)((double)v.y * hubble_h);
    const int nz = (int)(i % H);
    const float kz = __fmul_rn((float)nz, delta_k);
    // (a + i b)(0 + i k): real a*0 - b*k, imaginary a*k + b*0
    const float re = __fsub_rn(__fmul_rn(v.x, 0.0f), __fmul_rn(v.y, kz));
    const float im = __fadd_rn(__fmul_rn(v.x, kz), __fmul_rn(v.y, 0.0f));
    spec[i] = make_float2(re, im);
  }
}

__global__ void k_pecvel_cells(PecvelArgs a, int D, int H, long long N)
{
  for (long long ir = blockIdx.x * (long long)blockDim.x + threadIdx.x; ir < N; ir += (long long)gridDim.x * blockDim.x) {
    const long long row = row_of(ir, D);
    const long long ip = row * 2LL * H + (ir - row * D);
    const double g = (double)a.grad[ip];
    if (a.mode == 1) {
      double dvdx = g;
      if (fabs(dvdx) > a.max_v_deriv)
        dvdx = dvdx < 0 ? -a.max_v_deriv : a.max_v_deriv;
      a.delta_T[ir] = (float)((double)a.delta_T[ir] / (dvdx / (double)a.H_z + 1.0));
    } else {
      const double gc = fabs(g / (double)a.H_z + 1.0);
      const double ts = (double)a.TS[ir];
      if (gc < FRACT_FLOAT_ERR_D)
        a.delta_T[ir] = (float)(1000. * (ts - a.T_rad) / (1. + (double)a.redshift));
      else
        a.delta_T[ir] = (float)((1. - exp(-(double)a.delta_T[ir] / gc)) * 1000. * (ts - a.T_rad) /
                                (1. + (double)a.redshift));
    }
  }
}

// Target cell index of a deposit.  The reference's index arithmetic assumes
// a displacement below one box length; wrapping keeps every access inside the
// column in any case and is the identity whenever the reference's index is
// valid.
__device__ __forceinline__ int wrap(int t, int D) { return ((t % D) + D) % D; }

// BrightnessTemperature.c:325-499 for one z column per thread
__global__ void k_rsd_columns(RsdArgs a, int D, int H)
{
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= (long long)D * D)
    return;
  const float* vel = a.vel + col * 2LL * H;
  const float* dTc = a.delta_T + col * D;
  const float* xHc = a.xH + col * D;
  float* los = a.los + col * D;
  const int NS = RSD_STEPS;
  const double cw = a.box / (float)D;  // BoxSize / (float)ReionGridDim
  const double sw = a.subcell_width;
  const float H_z = a.H_z;
  for (int kk = 0; kk < D; kk++)
    los[kk] = 0.0f;
  for (int kk = 0; kk < D; kk++) {
    const float dT = dTc[kk];
    if (!((fabs((double)dT) >= FRACT_FLOAT_ERR_D) && ((double)xHc[kk] >= FRACT_FLOAT_ERR_D)))
      continue;
    // displacements: float divisions assigned to doubles, as in the reference
    double d1_low, d2_low, d1_high, d2_high;
    if (kk == 0) {
      d1_low = __fdiv_rn(vel[D - 1], H_z);
      d2_low = __fdiv_rn(vel[kk], H_z);
    } else {
      d1_low = __fdiv_rn(vel[kk - 1], H_z);
      d2_low = __fdiv_rn(vel[kk], H_z);
    }
    if (kk == D - 1) {
      d1_high = __fdiv_rn(vel[kk], H_z);
      d2_high = __fdiv_rn(vel[0], H_z);
    } else {
      d1_high = __fdiv_rn(vel[kk], H_z);
      d2_high = __fdiv_rn(vel[kk + 1], H_z);
    }
    const float share = __fdiv_rn(dT, (float)NS);  // delta_T / (float)N_RSD_STEPS
    for (int iii = 0; iii < NS; iii++) {
      const float xp = a.x_pos[iii];
      double disp;
      if (xp <= 0.5f)
        disp = d1_low + (((double)xp + 0.5) - 0.) * (d2_low - d1_low) / (1. - 0.);
      else
        disp = d1_high + (((double)xp - 0.5) - 0.) * (d2_high - d1_high) / (1. - 0.);
      const double pos = ((double)a.x_pos_offset[iii] + disp) / cw;
      const double lo = pos - (sw / 2.) / cw;
      const double hi = pos + (sw / 2.) / cw;
      if (lo >= 0.0 && hi < 1.0) {
        los[kk] = __fadd_rn(los[kk], share);
      } else if (lo < 0.0 && hi < 0.0) {
        const double cell_distance = ceil(fabs(lo)) - 1.;
        const int cd = (int)cell_distance;
        if (fabs(hi) > cell_distance) {
          const int t = wrap(kk < cd + 1 ? kk - (cd + 1) + D : kk - (cd + 1), D);
          los[t] = __fadd_rn(los[t], share);
        } else {
          const double fo = (fabs(lo) - cell_distance) / (sw / cw);
          const double fw = 1. - fo;
          const int t1 = wrap(kk < cd ? kk - cd + D : kk - cd, D);
          los[t1] = (float)((double)los[t1] + fw * (double)dT / (double)(float)NS);
          const int t2 = wrap(kk < cd + 1 ? kk - (cd + 1) + D : kk - (cd + 1), D);
          los[t2] = (float)((double)los[t2] + fo * (double)dT / (double)(float)NS);
        }
      } else if (lo < 0.0 && (hi > 0.0 && hi < 1.0)) {
        const double fw = hi / (sw / cw);
        const double fo = 1. - fw;
        const int t1 = kk == 0 ? D - 1 : kk - 1;
        los[t1] = (float)((double)los[t1] + fo * (double)dT / (double)(float)NS);
        los[kk] = (float)((double)los[kk] + fw * (double)dT / (double)(float)NS);
      } else if ((lo >= 0.0 && lo < 1.0) && (hi >= 1.0)) {
        const double fo = (hi - 1.) / (sw / cw);
        const double fw = 1. - fo;
        const int t2 = kk == D - 1 ? 0 : kk + 1;
        los[kk] = (float)((double)los[kk] + fw * (double)dT / (double)(float)NS);
        los[t2] = (float)((double)los[t2] + fo * (double)dT / (double)(float)NS);
      } else {
        const double cell_distance = floor(fabs(hi));
        const int cd = (int)cell_distance;
        if (lo >= cell_distance) {
          const int t = wrap(kk > D - 1 - cd ? kk + cd - D : kk + cd, D);
          los[t] = __fadd_rn(los[t], share);
        } else {
          const double fo = (hi - cell_distance) / (sw / cw);
          const double fw = 1. - fo;
          const int t1 = wrap(kk > D - 1 - (cd - 1) ? kk + cd - 1 - D : kk + cd - 1, D);
          los[t1] = (float)((double)los[t1] + fw * (double)dT / (double)(float)NS);
          const int t2 = wrap(kk > D - 1 - cd ? kk + cd - D : kk + cd, D);
          los[t2] = (float)((double)los[t2] + fo * (double)dT / (double)(float)NS);
        }
      }
    }
  }
}

__global__ void k_copy_grid(const float* __restrict__ src, float* __restrict__ dst, long long N)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
}  // namespace

void launch_vel_convert(float* vel, int trees_id, float redshift, const GridDims& gd, cudaStream_t s)
{
  k_vel_convert<<<RED_BLOCKS, RED_THREADS, 0, s>>>(vel, trees_id, redshift, gd.D, gd.H, gd.N);
  pv_launches++;
}

void launch_vel_grad_k(float2* spec, const GridDims& gd, double hubble_h, float delta_k, cudaStream_t s)
{
  k_vel_grad_k<<<RED_BLOCKS, RED_THREADS, 0, s>>>(spec, gd.H, gd.C, (double)gd.N, hubble_h, delta_k);
  pv_launches++;
}

void launch_pecvel_cells(const PecvelArgs& a, const GridDims& gd, cudaStream_t s)
{
  k_pecvel_cells<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D, gd.H, gd.N);
  pv_launches++;
}

void launch_rsd(const RsdArgs& a, const GridDims& gd, cudaStream_t s)
{
  const long long cols = (long long)gd.D * gd.D;
  k_rsd_columns<<<(unsigned)((cols + 127) / 128), 128, 0, s>>>(a, gd.D, gd.H);
  k_copy_grid<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a.los, a.delta_T_out, gd.N);
  pv_launches += 2;
}

int pecvel_kernel_launches() { return pv_launches; }

}  // namespace mx
