// The 21cm brightness-temperature box with its volume average, for callers
// that cannot allocate device memory.
//
// Who cannot allocate, and why: a galaxy-formation host that keeps every
// reionization grid resident has usually handed the rest of the device to its
// own pool, so the work buffers mx_create reserves are not available to it;
// and a host thread that must not stall cannot call cudaMalloc or cudaFree,
// which may synchronise the whole device.  This entry point needs no context.
// It takes the caller's device grids, and its only scratch is a file-scope
// __device__ array of fixed size.
//
// Per-cell arithmetic: BrightnessTemperature.c:48-53 (constants) and :82-124
// (the cell formula without peculiar velocities), in float: the reference
// forms const_factor * xH * (1.0 + deltax) in double and rounds once, this
// kernel rounds after each float product (a few ulp, well inside the 1e-4
// relative tolerance of delta_T); the same float operations as k_delta_T in
// kernels.cu.  The volume sum (:530-545) is deterministic.
// Block b reduces cells [b * CELLS_PER_BLOCK, (b+1) * CELLS_PER_BLOCK) in a
// fixed order and stores its partial.  The block that finishes last (by an
// atomic ticket) sums the partials in index order and writes the mean.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "host_physics.h"
#include "mx_reion.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 64;
constexpr long long NA_CELLS_PER_BLOCK = (long long)NA_THREADS * NA_CELLS_PER_THREAD;
constexpr int NA_MAX_PARTIALS = MX_NOALLOC_MAX_CELLS / NA_CELLS_PER_BLOCK;
static_assert(MX_NOALLOC_MAX_CELLS % NA_CELLS_PER_BLOCK == 0, "partials cover the maximum grid");

// Scratch: the ticket (must be 0 when a launch starts; every call zeroes it
// on its stream before launching), then one double per block.
constexpr size_t NA_TICKET_BYTES = 256;
constexpr size_t NA_SCRATCH_BYTES = NA_TICKET_BYTES + sizeof(double) * NA_MAX_PARTIALS;
static_assert(NA_SCRATCH_BYTES == MX_NOALLOC_SCRATCH_BYTES, "header states the scratch size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

struct NaArgs
{
  const float* deltax;  // PADDED
  const float* xH;
  const float* TS;
  float* delta_T;
  float const_factor, T_rad_f;
  int spin;
  int D, H;
  long long N;
  double inv_N;
  unsigned char* scratch;
  double* mean;
};

__global__ void __launch_bounds__(NA_THREADS) k_delta_T_noalloc(NaArgs a)
{
  unsigned int* ticket = reinterpret_cast<unsigned int*>(a.scratch);
  double* partials = reinterpret_cast<double*>(a.scratch + NA_TICKET_BYTES);
  __shared__ double red[NA_THREADS];
  __shared__ bool last;
  const long long c0 = (long long)blockIdx.x * NA_CELLS_PER_BLOCK;
  double acc = 0.0;
  for (int j = 0; j < NA_CELLS_PER_THREAD; j++) {
    const long long ir = c0 + (long long)j * NA_THREADS + threadIdx.x;
    if (ir >= a.N)
      break;
    const long long row = ir / a.D;
    const long long ip = row * 2LL * a.H + (ir - row * a.D);
    float dT = a.const_factor * a.xH[ir] * (1.0f + a.deltax[ip]);
    if (a.spin)
      dT = dT * (1.0f - a.T_rad_f / a.TS[ir]);
    a.delta_T[ir] = dT;
    acc += (double)dT;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last)
    return;
  __threadfence();
  double t = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += NA_THREADS)
    t += __ldcg(&partials[b]);
  red[threadIdx.x] = t;
  __syncthreads();
  for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    *a.mean = red[0] * a.inv_N;
}

// The scratch address per device, as last looked up outside stream capture
// (calls made while their stream is capturing use it).
std::mutex g_mu;
void* g_scratch_addr[256] = {};

void set_error(char* errbuf, size_t errlen, const char* msg)
{
  if (errbuf && errlen > 0) {
    std::strncpy(errbuf, msg, errlen - 1);
    errbuf[errlen - 1] = '\0';
  }
}

}  // namespace

extern "C" int mx_brightness_temperature_noalloc(const mx_params* params,
                                                 double redshift,
                                                 const float* deltax,
                                                 const float* xH,
                                                 const float* TS_box,
                                                 float* delta_T,
                                                 double* volume_ave_Tb,
                                                 void* stream,
                                                 char* errbuf,
                                                 size_t errlen)
{
  if (!params || params->abi_version != MX_ABI_VERSION) {
    set_error(errbuf, errlen, "invalid parameters or ABI version");
    return MX_EINVAL;
  }
  const mx_params& p = *params;
  const int D = p.grid_dim;
  if (D < 2 || (D & 1)) {
    set_error(errbuf, errlen, "invalid grid_dim (must be even and >= 2)");
    return MX_EINVAL;
  }
  const long long N = (long long)D * D * D;
  if (N > (long long)MX_NOALLOC_MAX_CELLS) {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "grid_dim %d needs %lld cells; the no-allocation scratch holds partial sums for at most %d cells",
                  D, N, MX_NOALLOC_MAX_CELLS);
    set_error(errbuf, errlen, msg);
    return MX_EINVAL;
  }
  if (p.flag_spin_temp && p.flag_pecvel > 0) {
    set_error(errbuf, errlen, "peculiar-velocity modes of the brightness temperature are not built");
    return MX_ENOTSUP;
  }
  if (!deltax || !xH || !delta_T || !volume_ave_Tb || (p.flag_spin_temp && !TS_box)) {
    set_error(errbuf, errlen, "a required device pointer is NULL");
    return MX_EINVAL;
  }
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    set_error(errbuf, errlen, "no current CUDA device");
    return MX_ECUDA;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) {
    set_error(errbuf, errlen, "invalid stream");
    return MX_ECUDA;
  }
  void* scratch = nullptr;
  {
    // The array's device address, looked up with the device current.  A call
    // outside stream capture looks it up again, so that a context created
    // anew on the device (after cudaDeviceReset) gets its own address; a
    // call on a capturing stream uses the address of the last call outside
    // capture.
    std::lock_guard<std::mutex> lock(g_mu);
    if (capture == cudaStreamCaptureStatusNone) {
      void* addr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
      if (e != cudaSuccess) {
        set_error(errbuf, errlen, cudaGetErrorString(e));
        return MX_ECUDA;
      }
      g_scratch_addr[dev] = addr;
    } else if (!g_scratch_addr[dev]) {
      set_error(errbuf, errlen, "the first call on a device must come before any stream capture");
      return MX_ESTATE;
    }
    scratch = g_scratch_addr[dev];
  }
  // constants of BrightnessTemperature.c:495-510
  const float z = (float)redshift;
  const float Hubble_h = (float)p.hubble_h;
  const float OmegaM = (float)p.omega_m;
  const float OmegaB = (float)(OmegaM * p.baryon_frac);
  NaArgs a;
  a.const_factor = (float)(27.0 * (OmegaB * Hubble_h * Hubble_h / 0.023) *
                           std::sqrt((0.15 / OmegaM / Hubble_h / Hubble_h) * (1.0 + z) / 10.0));
  a.T_rad_f = (float)(mx::k::TCMB * (1. + z));
  a.deltax = deltax;
  a.xH = xH;
  a.TS = TS_box;
  a.delta_T = delta_T;
  a.spin = p.flag_spin_temp;
  a.D = D;
  a.H = D / 2 + 1;
  a.N = N;
  a.inv_N = 1.0 / (double)N;
  a.scratch = static_cast<unsigned char*>(scratch);
  a.mean = volume_ave_Tb;
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    const unsigned blocks = (unsigned)((N + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK);
    k_delta_T_noalloc<<<blocks, NA_THREADS, 0, s>>>(a);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_error(errbuf, errlen, cudaGetErrorString(e));
    return MX_ECUDA;
  }
  return MX_OK;
}
