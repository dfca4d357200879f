// Fused inverse 3-D transforms for power-of-two grids (D = 32 ... 512).
//
// The reference inverse-transforms every filtered field at every radius with
// FFTW (find_HII_bubbles.c:254-269, ComputeTs.c:405-409) and then makes
// separate passes for the aliasing clamps and the per-cell test.  Here the
// inverse C2R of a batch of (radius, field) spectra is three passes:
//
//   x-pass   filter W(kR) (reionization.c:2110-2170) and the 1/N scale fused
//            into the load; the unfiltered spectrum tile is reused from L2 for
//            every radius of the batch; inverse FFT along x.
//   y-pass   inverse FFT along y, in place.
//   z-pass   Hermitian-extended inverse FFT along z (FFTW c2r semantics: the
//            imaginary parts of kz = 0 and kz = D/2 are ignored) fused with
//            the consumer: either the clamps + ionisation test + bookkeeping
//            of find_HII_bubbles for every radius with the cell state kept on
//            chip, or the clamped store of ComputeTs shells.
//
// Each 1-D transform of length D = D1 * D2 is a two-step (Cooley-Tukey
// "four-step") transform over a tile of T columns: D1-point DFTs in
// registers, twiddles, a transpose through shared memory, D2-point DFTs in
// registers.  Twiddles come from a shared-memory table filled with sincospi.
#include <cmath>
#include <cstdint>

#include "fft3d.cuh"

namespace mx {

namespace {
constexpr int FFT_THREADS = 256;
constexpr int TX = 16;  // columns (kz) per x/y tile
constexpr int TZ = 4;   // rows (y) per z tile
constexpr float REL_TOL_F = 1e-5f;
constexpr float ABS_TOL_F = 1e-8f;
constexpr double PI_D = 3.14159265358979323846;
int fft_launches = 0;

template <int D>
struct Split;
template <>
struct Split<32>
{
  static constexpr int D1 = 4, D2 = 8;
};
template <>
struct Split<64>
{
  static constexpr int D1 = 8, D2 = 8;
};
template <>
struct Split<128>
{
  static constexpr int D1 = 8, D2 = 16;
};
template <>
struct Split<256>
{
  static constexpr int D1 = 16, D2 = 16;
};
template <>
struct Split<512>
{
  static constexpr int D1 = 16, D2 = 32;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

__host__ __device__ constexpr int ilog2(int m) { return m <= 1 ? 0 : 1 + ilog2(m / 2); }
__host__ __device__ constexpr int brev(int i, int bits)
{
  int r = 0;
  for (int b = 0; b < bits; b++)
    r |= ((i >> b) & 1) << (bits - 1 - b);
  return r;
}

// tw[j] = exp(+2 pi i j / D) for j < D
template <int D>
__device__ void fill_twiddles(float2* tw)
{
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    float s, c;
    sincospif(2.0f * (float)j / (float)D, &s, &c);
    tw[j] = make_float2(c, s);
  }
}

// In-register backward DFT of M points (radix-2, decimation in time);
// tw is the D-point table, so exp(+2 pi i a / M) = tw[a * D / M].
template <int M, int D>
__device__ __forceinline__ void dft_bwd(float2 (&v)[M], const float2* __restrict__ tw)
{
  constexpr int LOG = ilog2(M);
#pragma unroll
  for (int i = 0; i < M; i++) {
    const int j = brev(i, LOG);
    if (j > i) {
      const float2 t = v[i];
      v[i] = v[j];
      v[j] = t;
    }
  }
#pragma unroll
  for (int half = 1; half < M; half <<= 1) {
#pragma unroll
    for (int i = 0; i < M; i += 2 * half) {
#pragma unroll
      for (int j = 0; j < half; j++) {
        float2 b = v[i + j + half];
        if (j != 0)
          b = cmul(b, tw[j * (D / (2 * half))]);
        v[i + j + half] = csub(v[i + j], b);
        v[i + j] = cadd(v[i + j], b);
      }
    }
  }
}

// k-space filter of reionization.c:2110-2170 in single precision only:
//  * real-space top-hat 3 (sin kR / kR^3 - cos kR / kR^2): sin and cos from one
//    sincosf, the powers from products (within an ulp of powf).  The
//    reference's test (double)kR > 1e-4 is the same predicate as kR > 1e-4f
//    (1e-4f is the largest float below 1e-4), and (float)(3.0 * (double)w) is
//    3.0f * w rounded once, as the double product of a float and 3 is exact;
//  * k-space top-hat: a mode is zeroed when (float)((double)kR * 0.413566994)
//    > 1, i.e. when kR exceeds the float threshold sharpk_max computed on the
//    host from that expression;
//  * Gaussian: the reference's operations.
__device__ __forceinline__ float filter_weight(int filter_type, float kmag, float R, float sharpk_max, bool* zero)
{
  float kR = __fmul_rn(kmag, R);
  *zero = false;
  if (filter_type == 0) {
    if (kR > 1e-4f) {
      float s, c;
      sincosf(kR, &s, &c);
      const float kR2 = __fmul_rn(kR, kR);
      const float kR3 = __fmul_rn(kR2, kR);
      return __fmul_rn(3.0f, __fsub_rn(__fdiv_rn(s, kR3), __fdiv_rn(c, kR2)));
    }
    return 1.0f;
  }
  if (filter_type == 1) {
    *zero = kR > sharpk_max;
    return 1.0f;
  }
  kR = (float)((double)kR * 0.643);
  return powf((float)2.71828182845904523536, (float)((double)__fmul_rn(-kR, kR) / 2.0));
}

__device__ __forceinline__ float kcomp(int n, int D, float delta_k)
{
  return (n > D / 2) ? __fmul_rn((float)(n - D), delta_k) : __fmul_rn((float)n, delta_k);
}
}  // namespace

int fft_kernel_launches() { return fft_launches; }

// ------------------------------------------------------------------ x-pass
// Grid: one block per (ky, kz tile).  For every radius of the batch and every
// field: load the unfiltered column tile (HBM on the first radius, L2 after),
// scale by 1/N, multiply by W(|k| R), inverse FFT along x, store to
// out[(r*G + g) * C + (x*D + ky)*H + kz].
template <int D>
__global__ void __launch_bounds__(FFT_THREADS) k_fft_x_filter(XPassArgs a)
{
  constexpr int D1 = Split<D>::D1, D2 = Split<D>::D2, H = D / 2 + 1;
  constexpr int NT = (H + TX - 1) / TX;
  constexpr int ITEMS_A = TX * D2, ITEMS_B = TX * D1;
  constexpr int PER_A = (ITEMS_A + FFT_THREADS - 1) / FFT_THREADS;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + D;
  float* wsm = reinterpret_cast<float*>(buf + D * TX);
  fill_twiddles<D>(tw);
  const int ky = blockIdx.x / NT;
  const int kz0 = (blockIdx.x % NT) * TX;
  const float kyv = kcomp(ky, D, a.delta_k);
  __syncthreads();
  for (int r = 0; r < a.n; r++) {
    // filter weights of the tile for radius r, wsm[kx * TX + t]; a zeroed
    // sharp-k mode is a weight of 0
    for (int i = threadIdx.x; i < D * TX; i += FFT_THREADS) {
      const int kx = i / TX, kz = kz0 + i % TX;
      float wv = 1.0f;
      if (a.apply[r]) {
        const float kxv = kcomp(kx, D, a.delta_k);
        const float kzv = __fmul_rn((float)kz, a.delta_k);
        const float kmag =
          sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(kyv, kyv)), __fmul_rn(kzv, kzv)));
        bool zero = false;
        wv = filter_weight(a.filter_type, kmag, a.R[r], a.sharpk_max, &zero);
        if (zero)
          wv = 0.0f;
      }
      wsm[i] = wv;
    }
    __syncthreads();
    for (int g = 0; g < a.G; g++) {
      const float2* __restrict__ src = a.in[g];
      // step A: D1-point DFTs along n1, twiddle, to shared memory
#pragma unroll
      for (int q = 0; q < PER_A; q++) {
        const int item = threadIdx.x + q * FFT_THREADS;
        if (item < ITEMS_A) {
          const int t = item % TX, n2 = item / TX;
          const int kz = kz0 + t;
          float2 v[D1];
#pragma unroll
          for (int n1 = 0; n1 < D1; n1++) {
            const int kx = n2 + D2 * n1;
            float2 x = make_float2(0.f, 0.f);
            if (kz < H) {
              x = src[((long long)kx * D + ky) * H + kz];
              const float wv = wsm[kx * TX + t];
              x.x = __fmul_rn(__fmul_rn(x.x, a.scale), wv);
              x.y = __fmul_rn(__fmul_rn(x.y, a.scale), wv);
            }
            v[n1] = x;
          }
          dft_bwd<D1, D>(v, tw);
#pragma unroll
          for (int k1 = 0; k1 < D1; k1++) {
            const float2 t2 = k1 == 0 || n2 == 0 ? v[k1] : cmul(v[k1], tw[(n2 * k1) % D]);
            buf[(k1 * D2 + n2) * TX + t] = t2;
          }
        }
      }
      __syncthreads();
      // step B: D2-point DFTs along n2, natural-order store
      float2* __restrict__ dst = a.out + (long long)(r * a.G + g) * a.C;
      for (int item = threadIdx.x; item < ITEMS_B; item += FFT_THREADS) {
        const int t = item % TX, k1 = item / TX;
        const int kz = kz0 + t;
        float2 u[D2];
#pragma unroll
        for (int n2 = 0; n2 < D2; n2++)
          u[n2] = buf[(k1 * D2 + n2) * TX + t];
        dft_bwd<D2, D>(u, tw);
        if (kz < H) {
#pragma unroll
          for (int k2 = 0; k2 < D2; k2++) {
            const int x = k1 + D1 * k2;
            dst[((long long)x * D + ky) * H + kz] = u[k2];
          }
        }
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------------------ y-pass
// Grid: (spectrum, x, kz tile).  In-place inverse FFT along y.
template <int D>
__global__ void __launch_bounds__(FFT_THREADS) k_fft_y(float2* data, long long C, int n_spectra)
{
  constexpr int D1 = Split<D>::D1, D2 = Split<D>::D2, H = D / 2 + 1;
  constexpr int NT = (H + TX - 1) / TX;
  constexpr int ITEMS_A = TX * D2, ITEMS_B = TX * D1;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + D;
  fill_twiddles<D>(tw);
  const long long blk = blockIdx.x;
  const int tile = (int)(blk % NT);
  const int x = (int)((blk / NT) % D);
  const long long s = blk / ((long long)NT * D);
  const int kz0 = tile * TX;
  float2* plane = data + s * C + (long long)x * D * H;
  __syncthreads();
  for (int item = threadIdx.x; item < ITEMS_A; item += FFT_THREADS) {
    const int t = item % TX, n2 = item / TX;
    const int kz = kz0 + t;
    float2 v[D1];
#pragma unroll
    for (int n1 = 0; n1 < D1; n1++)
      v[n1] = kz < H ? plane[(long long)(n2 + D2 * n1) * H + kz] : make_float2(0.f, 0.f);
    dft_bwd<D1, D>(v, tw);
#pragma unroll
    for (int k1 = 0; k1 < D1; k1++)
      buf[(k1 * D2 + n2) * TX + t] = k1 == 0 || n2 == 0 ? v[k1] : cmul(v[k1], tw[(n2 * k1) % D]);
  }
  __syncthreads();
  for (int item = threadIdx.x; item < ITEMS_B; item += FFT_THREADS) {
    const int t = item % TX, k1 = item / TX;
    const int kz = kz0 + t;
    float2 u[D2];
#pragma unroll
    for (int n2 = 0; n2 < D2; n2++)
      u[n2] = buf[(k1 * D2 + n2) * TX + t];
    dft_bwd<D2, D>(u, tw);
    if (kz < H) {
#pragma unroll
      for (int k2 = 0; k2 < D2; k2++)
        plane[(long long)(k1 + D1 * k2) * H + kz] = u[k2];
    }
  }
}

// ------------------------------------------------------------------ z-pass
// The z-pass reads, per block, TZ consecutive rows (x, y0 .. y0+TZ-1) of every
// spectrum of the batch: TZ*H contiguous complex values.  These row groups are
// streamed into shared memory by bulk asynchronous copies (cp.async.bulk,
// completion on an mbarrier) through a ZSTAGES-deep ring, so that the copies
// of the next spectra are in flight while the current one is transformed.
namespace {
constexpr int ZSTAGES = 4;
constexpr unsigned ERR_PIPELINE_TIMEOUT = 2u;
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;  // 2 s
constexpr long long WAIT_LIMIT_ITERS = 1LL << 26;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arms the barrier for `bytes` and issues one bulk copy global -> shared.
// dst, src and bytes are multiples of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
    "l"(src), "r"(bytes), "r"(smem_addr(bar))
    : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity)
{
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_addr(bar)), "r"(parity)
    : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase `parity` of the barrier; false after about WAIT_LIMIT_NS.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity)
{
  if (mbar_test(bar, parity))
    return true;
  const unsigned long long t0 = global_ns();
  for (long long it = 1; it < WAIT_LIMIT_ITERS; it++) {
    if (mbar_test(bar, parity))
      return true;
    if ((it & 255) == 0 && global_ns() - t0 > WAIT_LIMIT_NS)
      return false;
  }
  return false;
}

// Shared-memory plan of a z-pass block.
template <int D>
struct ZPlan
{
  static constexpr int D1 = Split<D>::D1, D2 = Split<D>::D2, H = D / 2 + 1;
  static constexpr int STAGE = TZ * H;          // complex values per stage
  static constexpr int BT = D1 * (D2 + 1);      // padded transpose buffer per row
  static constexpr int OS = D + D1;             // padded real output row
  static constexpr size_t OFF_TW = 64;          // after the barriers
  static constexpr size_t OFF_STAGE = OFF_TW + sizeof(float2) * D;
  static constexpr size_t OFF_BUF = OFF_STAGE + sizeof(float2) * (size_t)ZSTAGES * STAGE;
  static constexpr size_t OFF_FLD = OFF_BUF + sizeof(float2) * (size_t)TZ * BT;
  static constexpr size_t bytes(int fields) { return OFF_FLD + sizeof(float) * (size_t)fields * TZ * OS; }
  static_assert((sizeof(float2) * STAGE) % 16 == 0, "bulk copy size");
  static_assert(OFF_STAGE % 16 == 0, "bulk copy destination");
};

// The producer side of the ring: thread 0 issues item `it` into stage
// it % ZSTAGES.  Item it is spectrum it (of C complex values), rows row0 ..
template <int D>
__device__ __forceinline__ void z_issue(char* smem, const float2* spectra, long long C, long long row0, int it)
{
  using P = ZPlan<D>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  float2* st = reinterpret_cast<float2*>(smem + P::OFF_STAGE) + (size_t)(it % ZSTAGES) * P::STAGE;
  bulk_load(st, spectra + (long long)it * C + row0 * P::H, (unsigned)(sizeof(float2) * P::STAGE),
            &bars[it % ZSTAGES]);
}

// Inverse C2R along z of the TZ staged rows of item `it` into out[t*OS + z].
// Returns false (for every thread of the block) if the copy did not arrive.
// Thread 0 refills the stage with item it + ZSTAGES (< n_items) as soon as
// every thread has read it.
template <int D>
__device__ __forceinline__ bool z_c2r(char* smem, int it, int n_items, const float2* spectra, long long C,
                                      long long row0, float* out)
{
  using P = ZPlan<D>;
  constexpr int D1 = P::D1, D2 = P::D2, H = P::H;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  const float2* tw = reinterpret_cast<const float2*>(smem + P::OFF_TW);
  const float2* st = reinterpret_cast<const float2*>(smem + P::OFF_STAGE) + (size_t)(it % ZSTAGES) * P::STAGE;
  float2* buf = reinterpret_cast<float2*>(smem + P::OFF_BUF);
  const bool arrived = mbar_wait(&bars[it % ZSTAGES], (unsigned)(it / ZSTAGES) & 1u);
  // step A: D1-point DFTs along n1 (Hermitian-extended input), twiddles
  for (int item = threadIdx.x; item < TZ * D2; item += FFT_THREADS) {
    const int n2 = item % D2, t = item / D2;
    const float2* row = st + t * H;
    float2 v[D1];
#pragma unroll
    for (int n1 = 0; n1 < D1; n1++) {
      const int k = n2 + D2 * n1;
      float2 x;
      if (k < H) {
        x = row[k];
        if (k == 0 || k == D / 2)
          x.y = 0.0f;
      } else {
        const float2 c = row[D - k];
        x = make_float2(c.x, -c.y);
      }
      v[n1] = x;
    }
    dft_bwd<D1, D>(v, tw);
#pragma unroll
    for (int k1 = 0; k1 < D1; k1++)
      buf[t * P::BT + k1 * (D2 + 1) + n2] = k1 == 0 || n2 == 0 ? v[k1] : cmul(v[k1], tw[(n2 * k1) % D]);
  }
  if (__syncthreads_or(!arrived))
    return false;
  if (threadIdx.x == 0 && it + ZSTAGES < n_items)
    z_issue<D>(smem, spectra, C, row0, it + ZSTAGES);
  // step B: D2-point DFTs along n2, real parts in natural order
  for (int item = threadIdx.x; item < TZ * D1; item += FFT_THREADS) {
    const int k1 = item % D1, t = item / D1;
    float2 u[D2];
#pragma unroll
    for (int n2 = 0; n2 < D2; n2++)
      u[n2] = buf[t * P::BT + k1 * (D2 + 1) + n2];
    dft_bwd<D2, D>(u, tw);
#pragma unroll
    for (int k2 = 0; k2 < D2; k2++)
      out[t * P::OS + k1 + D1 * k2] = u[k2].x;
  }
  __syncthreads();
  return true;
}

// Ring setup: barriers, twiddles, the first ZSTAGES copies.
template <int D>
__device__ __forceinline__ void z_setup(char* smem, const float2* spectra, long long C, long long row0, int n_items)
{
  using P = ZPlan<D>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  if (threadIdx.x == 0) {
    for (int s = 0; s < ZSTAGES; s++)
      mbar_init(&bars[s], 1);
    mbar_init_fence();
  }
  fill_twiddles<D>(reinterpret_cast<float2*>(smem + P::OFF_TW));
  __syncthreads();
  if (threadIdx.x == 0)
    for (int it = 0; it < ZSTAGES && it < n_items; it++)
      z_issue<D>(smem, spectra, C, row0, it);
}

// After a timed-out wait: record the error and wait (bounded) for the copies
// still in flight into this block's shared memory before it exits.
template <int D>
__device__ void z_abort(char* smem, int it, int n_items, unsigned* err)
{
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  if (threadIdx.x != 0)
    return;
  atomicOr(err, ERR_PIPELINE_TIMEOUT);
  // items it .. min(it + ZSTAGES, n_items) - 1 may have been issued
  for (int j = it; j < n_items && j < it + ZSTAGES; j++)
    mbar_wait(&bars[j % ZSTAGES], (unsigned)(j / ZSTAGES) & 1u);
}
}  // namespace

// z-pass fused with the per-cell test of find_HII_bubbles (clamps
// :271-311, criterion and bookkeeping :342-443) for every radius of the batch.
// Grid: one block per (x, y tile of TZ rows).  The cell state lives in
// registers for all radii; the G fields of a radius are transformed into
// shared memory, then every cell is tested.
template <int D>
__global__ void __launch_bounds__(FFT_THREADS, 2) k_fft_z_threshold(ZThresholdArgs a)
{
  using P = ZPlan<D>;
  constexpr int CELLS = TZ * D;
  constexpr int CPT = (CELLS + FFT_THREADS - 1) / FFT_THREADS;
  extern __shared__ __align__(128) unsigned char zsmem[];
  char* smem = reinterpret_cast<char*>(zsmem);
  float* fldbase = reinterpret_cast<float*>(smem + P::OFF_FLD);
  const int ny = D / TZ;
  const int x = blockIdx.x / ny;
  const int y0 = (blockIdx.x % ny) * TZ;
  const long long row0 = (long long)x * D + y0;  // first row index
  const int n_items = a.n_f * a.G;
  z_setup<D>(smem, a.spectra, a.C, row0, n_items);
  float xH[CPT], zion[CPT], rb[CPT], J21[CPT], J21i[CPT], G12[CPT];
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = threadIdx.x + j * FFT_THREADS;
    const long long ir = row0 * D + c;
    if (c < CELLS) {
      xH[j] = a.xH[ir];
      zion[j] = a.z_at_ion[ir];
      rb[j] = a.r_bubble[ir];
      J21[j] = a.uvb ? a.J21[ir] : 0.0f;
      J21i[j] = a.uvb ? a.J21_at_ion[ir] : 0.0f;
      G12[j] = a.recomb ? a.Gamma12[ir] : 0.0f;
    }
  }
  int it = 0;
  for (int r = 0; r < a.n_r; r++) {
    const RadiusParams rp = a.rp[r];
    const bool direct = rp.last != 0;
    if (!direct) {
      for (int g = 0; g < a.G; g++, it++)
        if (!z_c2r<D>(smem, it, n_items, a.spectra, a.C, row0, fldbase + g * TZ * P::OS)) {
          z_abort<D>(smem, it, n_items, a.err);
          return;
        }
    }
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      const int c = threadIdx.x + j * FFT_THREADS;
      if (c >= CELLS)
        continue;
      const int t = c / D, zc = c % D;
      float f[MAX_FIELDS];
      if (direct) {
        const long long ip = (row0 + t) * 2LL * P::H + zc;
        for (int g = 0; g < a.G; g++)
          f[g] = a.direct[g][ip];
      } else {
        for (int g = 0; g < a.G; g++)
          f[g] = fldbase[g * TZ * P::OS + t * P::OS + zc];
      }
      const float dx = fmaxf(f[0], -1 + REL_TOL_F);
      float st = fmaxf(f[1], 0.0f);
      if (st < ABS_TOL_F)
        st = 0;
      float ws = fmaxf(f[2], 0.0f);
      if (ws < ABS_TOL_F)
        ws = 0;
      float nr = 0.0f, xe = 0.0f;
      if (a.recomb) {
        nr = fmaxf(f[a.idx_nr], 0.0f);
        if (nr < ABS_TOL_F)
          nr = 0;
      }
      if (a.spin) {
        xe = fmaxf(f[a.idx_xe], 0.0f);
        if (xe < ABS_TOL_F)
          xe = 0;
        xe = fminf(xe, 0.999f);
      }
      const float domf = 1.0f + dx;
      const float lhs_f = st * rp.kfc / domf;
      const float nf_f = 1.0f - xe;
      const float rhs_f = nf_f * (1.0f + nr / domf);
      bool ionised;
      float xpart;
      if (fabsf(lhs_f - rhs_f) > 4e-6f * fmaxf(lhs_f, rhs_f)) {
        ionised = lhs_f > rhs_f;
        xpart = nf_f - lhs_f;
      } else {
        const double dom = 1.0 + (double)dx;
        const double rec = a.recomb ? (double)nr / dom : 0.0;
        const double nf = a.spin ? 1.0 - (double)xe : 1.0;
        const double f_coll = (double)st / (rp.M_mean * dom) * (4.0 / 3.0) * PI_D * rp.R_cubed / a.pixel_volume;
        ionised = f_coll * a.eff > nf * (1. + rec);
        xpart = (float)__dsub_rn(nf, __dmul_rn(f_coll, a.eff));
      }
      const float J21_aux = a.uvb ? ws * rp.kj : 0.0f;
      if (ionised) {
        if (xH[j] > REL_TOL_F) {
          if (a.uvb)
            J21[j] = J21_aux;
          if (a.recomb)
            G12[j] = ws * rp.kg;
        }
        xH[j] = 0.0f;
        rb[j] = (float)rp.R;
      } else if (rp.last && (xH[j] > REL_TOL_F)) {
        xH[j] = fminf(fmaxf(xpart, 0.0f), 1.0f);
      }
      if ((xH[j] < REL_TOL_F) && (zion[j] < 0)) {
        zion[j] = (float)a.redshift;
        if (a.uvb)
          J21i[j] = J21_aux * a.gamma_halo_bias;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = threadIdx.x + j * FFT_THREADS;
    const long long ir = row0 * D + c;
    if (c < CELLS) {
      a.xH[ir] = xH[j];
      a.z_at_ion[ir] = zion[j];
      a.r_bubble[ir] = rb[j];
      if (a.uvb) {
        a.J21[ir] = J21[j];
        a.J21_at_ion[ir] = J21i[j];
      }
      if (a.recomb)
        a.Gamma12[ir] = G12[j];
    }
  }
}

// z-pass storing clamped real values (ComputeTs shells, ComputeTs.c:476-500):
// shells[(r0 + r) * N + cell] = max(value, 0) for every spectrum of the batch.
template <int D>
__global__ void __launch_bounds__(FFT_THREADS, 2) k_fft_z_store(const float2* spectra, long long C, int n, int r0,
                                                                   float* shells, long long N, unsigned* err)
{
  using P = ZPlan<D>;
  constexpr int CELLS = TZ * D;
  extern __shared__ __align__(128) unsigned char zsmem[];
  char* smem = reinterpret_cast<char*>(zsmem);
  float* fld = reinterpret_cast<float*>(smem + P::OFF_FLD);
  const int ny = D / TZ;
  const int x = blockIdx.x / ny;
  const int y0 = (blockIdx.x % ny) * TZ;
  const long long row0 = (long long)x * D + y0;
  z_setup<D>(smem, spectra, C, row0, n);
  for (int r = 0; r < n; r++) {
    if (!z_c2r<D>(smem, r, n, spectra, C, row0, fld)) {
      z_abort<D>(smem, r, n, err);
      return;
    }
    float* dst = shells + (long long)(r0 + r) * N + row0 * D;
    for (int c = threadIdx.x; c < CELLS; c += FFT_THREADS)
      dst[c] = fmaxf(fld[(c / D) * P::OS + c % D], 0.0f);
    __syncthreads();
  }
}

// ----------------------------------------------------------------- launch
bool fft3d_supported(int D) { return D == 32 || D == 64 || D == 128 || D == 256 || D == 512; }

template <int D>
constexpr size_t smem_xy()
{
  return sizeof(float2) * (D + (size_t)D * TX);
}
template <int D>
constexpr size_t smem_x()
{
  return smem_xy<D>() + sizeof(float) * (size_t)D * TX;
}
template <int D>
static void launch_x(const XPassArgs& a, cudaStream_t s)
{
  constexpr int H = D / 2 + 1;
  constexpr int NT = (H + TX - 1) / TX;
  cudaFuncSetAttribute(k_fft_x_filter<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x<D>());
  k_fft_x_filter<D><<<D * NT, FFT_THREADS, smem_x<D>(), s>>>(a);
}
template <int D>
static void launch_y(float2* data, long long C, int n_spectra, cudaStream_t s)
{
  constexpr int H = D / 2 + 1;
  constexpr int NT = (H + TX - 1) / TX;
  const long long blocks = (long long)n_spectra * D * NT;
  cudaFuncSetAttribute(k_fft_y<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_xy<D>());
  k_fft_y<D><<<(unsigned)blocks, FFT_THREADS, smem_xy<D>(), s>>>(data, C, n_spectra);
}
template <int D>
static void launch_zt(const ZThresholdArgs& a, cudaStream_t s)
{
  const size_t bytes = ZPlan<D>::bytes(MAX_FIELDS);
  cudaFuncSetAttribute(k_fft_z_threshold<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_fft_z_threshold<D><<<D * (D / TZ), FFT_THREADS, bytes, s>>>(a);
}
template <int D>
static void launch_zs(const float2* spectra, long long C, int n, int r0, float* shells, long long N, unsigned* err,
                      cudaStream_t s)
{
  const size_t bytes = ZPlan<D>::bytes(1);
  cudaFuncSetAttribute(k_fft_z_store<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_fft_z_store<D><<<D * (D / TZ), FFT_THREADS, bytes, s>>>(spectra, C, n, r0, shells, N, err);
}

// Largest float kR with (float)((double)kR * 0.413566994) <= 1, the last mode
// the k-space top-hat of reionization.c:2150-2153 keeps.
static float sharpk_threshold()
{
  const double c = 0.413566994;
  float x = (float)(1.0 / c);
  while ((float)((double)x * c) > 1.0f)
    x = std::nextafter(x, 0.0f);
  while ((float)((double)std::nextafter(x, INFINITY) * c) <= 1.0f)
    x = std::nextafter(x, INFINITY);
  return x;
}

bool launch_fft_x_filter(int D, const XPassArgs& args, cudaStream_t s)
{
  static const float kmax = sharpk_threshold();
  XPassArgs a = args;
  a.sharpk_max = kmax;
  switch (D) {
    case 32: launch_x<32>(a, s); break;
    case 64: launch_x<64>(a, s); break;
    case 128: launch_x<128>(a, s); break;
    case 256: launch_x<256>(a, s); break;
    case 512: launch_x<512>(a, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

bool launch_fft_y(int D, float2* data, long long C, int n_spectra, cudaStream_t s)
{
  switch (D) {
    case 32: launch_y<32>(data, C, n_spectra, s); break;
    case 64: launch_y<64>(data, C, n_spectra, s); break;
    case 128: launch_y<128>(data, C, n_spectra, s); break;
    case 256: launch_y<256>(data, C, n_spectra, s); break;
    case 512: launch_y<512>(data, C, n_spectra, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

bool launch_fft_z_threshold(int D, const ZThresholdArgs& a, cudaStream_t s)
{
  switch (D) {
    case 32: launch_zt<32>(a, s); break;
    case 64: launch_zt<64>(a, s); break;
    case 128: launch_zt<128>(a, s); break;
    case 256: launch_zt<256>(a, s); break;
    case 512: launch_zt<512>(a, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

bool launch_fft_z_store(int D, const float2* spectra, long long C, int n, int r0, float* shells, long long N,
                        unsigned* err, cudaStream_t s)
{
  switch (D) {
    case 32: launch_zs<32>(spectra, C, n, r0, shells, N, err, s); break;
    case 64: launch_zs<64>(spectra, C, n, r0, shells, N, err, s); break;
    case 128: launch_zs<128>(spectra, C, n, r0, shells, N, err, s); break;
    case 256: launch_zs<256>(spectra, C, n, r0, shells, N, err, s); break;
    case 512: launch_zs<512>(spectra, C, n, r0, shells, N, err, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

}  // namespace mx
