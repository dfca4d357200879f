// Light-cone construction (ConstructLightcone.c:69-166): slice s of this
// snapshot takes the z column iz0 + s (mod D) of the co-eval boxes,
// interpolated linearly in cosmic time between the previous snapshot's
// delta_T and this one's, in double like the reference.  A thread per
// (column, slice) with the slice fastest: each column's run of slices is one
// contiguous write, as in the reference's [i][j][slice] layout.
#include "lightcone.cuh"

namespace mx {

namespace {
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int lc_launches = 0;

__global__ void k_lightcone(LightconeArgs a, int D)
{
  const long long total = (long long)D * D * a.n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(i % a.n);
    const long long col = i / a.n;
    const int iz = (a.iz0 + s) % D;
    const double fz1 = a.delta_T[col * D + iz], fz2 = a.delta_T_prev[col * D + iz];
    // (fz2 - fz1) / (t2 - t1) * (t - t1) + fz1 with separate roundings (no
    // fused multiply-add), as the reference evaluates it
    const double q = __ddiv_rn(__dsub_rn(fz2, fz1), __dsub_rn(a.t2, a.t1));
    a.out[col * a.pitch + s] = (float)__dadd_rn(__dmul_rn(q, __dsub_rn(a.t_slice[s], a.t1)), fz1);
  }
}
}  // namespace

void launch_lightcone(const LightconeArgs& a, const GridDims& gd, cudaStream_t s)
{
  if (a.n > 0) {
    k_lightcone<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, gd.D);
    lc_launches++;
  }
}

int lightcone_kernel_launches() { return lc_launches; }

}  // namespace mx
