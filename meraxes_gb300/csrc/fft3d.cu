// Fused 3-D transforms for power-of-two grids (D = 32 ... 512) and for the
// grids 24, 48, 96 and 192 (a factor 3).
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
// The x- and y-passes run a three-step Cooley-Tukey transform over a tile of
// 16 columns (radix-8 or radix-4 DFTs in registers with compile-time
// twiddles, inter-step twiddles from a shared table filled with sincospi,
// transposes through the shared tile).  The z-pass computes each row's C2R as a
// half-length complex transform split over 4-lane groups (see below).
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "bulk.cuh"
#include "fft3d.cuh"

namespace mx {

using namespace bulk;

// Compile-time cos and sin of 2 pi j / n, by Taylor series on [-pi, pi] (30
// terms; the truncation error is far below double rounding).  Used only to
// initialise constexpr twiddle factors.
__host__ __device__ constexpr double cx_cos_sin(int j, int n, bool want_sin)
{
  j = ((j % n) + n) % n;
  if (2 * j > n)
    j -= n;  // angle in [-pi, pi]
  const double x = 2.0 * 3.14159265358979323846 * (double)j / (double)n;
  double term = want_sin ? x : 1.0, sum = term;
  for (int k = 1; k < 30; k++) {
    const double a = want_sin ? (2.0 * k) * (2.0 * k + 1.0) : (2.0 * k - 1.0) * (2.0 * k);
    term *= -x * x / a;
    sum += term;
  }
  return sum;
}


namespace {
constexpr int FFT_THREADS = 256;
constexpr float REL_TOL_F = 1e-5f;
constexpr float ABS_TOL_F = 1e-8f;
constexpr double PI_D = 3.14159265358979323846;
// per host thread: a call counts its own launches when contexts run concurrently
thread_local int fft_launches = 0;

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

// b * exp(+2 pi i J / N) with the factor known at compile time; the eighth
// roots of unity take their exact forms.
template <int J, int N>
__device__ __forceinline__ float2 mul_tw(float2 b)
{
  constexpr int j = ((J % N) + N) % N;
  constexpr float h = 0.70710678118654752440f;  // 1/sqrt(2)
  if constexpr (j == 0) {
    return b;
  } else if constexpr (4 * j == N) {
    return make_float2(-b.y, b.x);
  } else if constexpr (2 * j == N) {
    return make_float2(-b.x, -b.y);
  } else if constexpr (4 * j == 3 * N) {
    return make_float2(b.y, -b.x);
  } else if constexpr (8 * j == N) {
    return make_float2(h * (b.x - b.y), h * (b.x + b.y));
  } else if constexpr (8 * j == 3 * N) {
    return make_float2(-h * (b.x + b.y), h * (b.x - b.y));
  } else if constexpr (8 * j == 5 * N) {
    return make_float2(h * (b.y - b.x), -h * (b.x + b.y));
  } else if constexpr (8 * j == 7 * N) {
    return make_float2(h * (b.x + b.y), h * (b.y - b.x));
  } else {
    constexpr float c = (float)cx_cos_sin(J, N, false);
    constexpr float s = (float)cx_cos_sin(J, N, true);
    return make_float2(c * b.x - s * b.y, c * b.y + s * b.x);
  }
}

// Butterflies of a radix-2 decimation-in-time DFT, stage HALF, group I,
// butterfly J, unrolled by template recursion so every twiddle is a constant.
template <int M, int HALF, int I, int J>
__device__ __forceinline__ void dft_stage(float2 (&v)[M])
{
  if constexpr (HALF < M) {
    if constexpr (I < M) {
      if constexpr (J < HALF) {
        const float2 b = mul_tw<J, 2 * HALF>(v[I + J + HALF]);
        const float2 a = v[I + J];
        v[I + J] = cadd(a, b);
        v[I + J + HALF] = csub(a, b);
        dft_stage<M, HALF, I, J + 1>(v);
      } else {
        dft_stage<M, HALF, I + 2 * HALF, 0>(v);
      }
    } else {
      dft_stage<M, 2 * HALF, 0, 0>(v);
    }
  }
}

// In-register backward DFT of M points: v[k] <- sum_n v[n] exp(+2 pi i nk/M).
template <int M>
__device__ __forceinline__ void dft_bwd(float2 (&v)[M])
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
  dft_stage<M, 1, 0, 0>(v);
}

// Backward DFT of 3 points, v_k <- sum_n v_n w^{nk} with w = exp(2 pi i / 3)
// = -1/2 + i sqrt(3)/2: v_0 = a + (b + d), v_{1,2} = a - (b + d)/2 +- i
// (sqrt(3)/2)(b - d).
__device__ __forceinline__ void dft3_bwd(float2 (&v)[3])
{
  constexpr float s = 0.86602540378443864676f;
  const float2 a = v[0], t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
  const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
  const float2 su = make_float2(-s * u.y, s * u.x);  // i s u
  v[0] = cadd(a, t);
  v[1] = cadd(m, su);
  v[2] = csub(m, su);
}

// In-register backward DFT of M points, M a power of two or 3.
template <int M>
__device__ __forceinline__ void dft_any(float2 (&v)[M])
{
  if constexpr (M == 3)
    dft3_bwd(v);
  else
    dft_bwd<M>(v);
}

// k-space filter of reionization.c:2110-2170:
//  * real-space top-hat: tophat_weight (kernels.cuh), the reference's float
//    expression below kR = 1, where it cancels, and one sincosf and a
//    reciprocal above.  The reference's test (double)kR > 1e-4 is the same
//    predicate as kR > 1e-4f (1e-4f is the largest float below 1e-4);
//  * k-space top-hat: a mode is zeroed when (float)((double)kR * 0.413566994)
//    > 1, i.e. when kR exceeds the float threshold sharpk_max computed on the
//    host from that expression;
//  * Gaussian: the reference's operations.
__device__ __forceinline__ float filter_weight(int filter_type, float kmag, float R, float sharpk_max, bool* zero)
{
  float kR = __fmul_rn(kmag, R);
  *zero = false;
  if (filter_type == 0)
    return kR > 1e-4f ? tophat_weight(kR) : 1.0f;
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

// Weight of the x-pass at (kx <= D/2, ky, kz) with kyv = kcomp(ky): the
// filter W(|k| R) times the 1/N scale (a power of two, so x * (scale * W) ==
// (x * scale) * W exactly); a zeroed sharp-k mode is a weight of 0.
__device__ __forceinline__ float x_weight(int kx, float kyv, int kz, int D, float delta_k, int filter_type, float R,
                                          float sharpk_max, float scale)
{
  const float kxv = kcomp(kx, D, delta_k);
  const float kzv = __fmul_rn((float)kz, delta_k);
  const float kmag = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(kyv, kyv)), __fmul_rn(kzv, kzv)));
  bool zero = false;
  float wv = filter_weight(filter_type, kmag, R, sharpk_max, &zero);
  if (zero)
    wv = 0.0f;
  return wv * scale;
}
}  // namespace

int fft_kernel_launches() { return fft_launches; }

cudaError_t fft_set_wait_polls(long long polls) { return set_consumer_wait_polls(polls); }

// ---------------------------------------------------- column-tile engine
// The x- and y-passes transform TXC adjacent columns (kz) of D points along
// a slow axis.  D = R1 * R2 * R3; with n = n' + M n1 (M = R2 R3) and
// n' = n3 + R3 n2, the three steps are
//   A: per (column, n'): DFT_R1 over n1 from global memory, twiddle
//      w_D^{n' k1}, into the shared tile at line k1 M + n';
//   B: per (column, k1, n3): DFT_R2 over n2 in place (lines n3 + R3 n2),
//      twiddle w_M^{n3 k2};
//   C: per (column, k1, k2): DFT_R3 over n3, output k = k1 + R1 (k2 + R2 k3).
// Every work item holds R points (R <= 8), so a block of 256 threads keeps
// few registers and a 64 KB tile at D = 512.
//
// Sixteen columns are 128 bytes: a half-warp moves one aligned 128-byte run
// per access.  The spectra between the passes are stored with rows of
// HP = D/2 + 1 rounded up to 16 complex values (272 at D = 512).  Every
// x-pass store is then one whole aligned 128-byte line at a 1 MB stride.
// Stores of that kind run at the HBM copy rate, whereas the unaligned
// 64-byte runs of 257-value rows ran at a third of it.  Rows are also 128-byte
// aligned for the y-pass and for the bulk copies of the z-pass.
constexpr int TXC = 16;  // columns per tile

// row pitch (complex values) of the spectra between the passes
template <int D>
struct Pitch
{
  static constexpr int H = D / 2 + 1;
  static constexpr int HP = (H + TXC - 1) / TXC * TXC;
};

template <int D>
struct Split3;
template <>
struct Split3<12>
{
  static constexpr int R1 = 4, R2 = 3, R3 = 1;
};
template <>
struct Split3<16>
{
  static constexpr int R1 = 4, R2 = 2, R3 = 2;
};
template <>
struct Split3<24>
{
  static constexpr int R1 = 4, R2 = 2, R3 = 3;
};
template <>
struct Split3<48>
{
  static constexpr int R1 = 4, R2 = 4, R3 = 3;
};
template <>
struct Split3<96>
{
  static constexpr int R1 = 8, R2 = 4, R3 = 3;
};
template <>
struct Split3<192>
{
  static constexpr int R1 = 8, R2 = 8, R3 = 3;
};
template <>
struct Split3<32>
{
  static constexpr int R1 = 4, R2 = 4, R3 = 2;
};
template <>
struct Split3<64>
{
  static constexpr int R1 = 4, R2 = 4, R3 = 4;
};
template <>
struct Split3<128>
{
  static constexpr int R1 = 8, R2 = 4, R3 = 4;
};
template <>
struct Split3<256>
{
  static constexpr int R1 = 8, R2 = 8, R3 = 4;
};
template <>
struct Split3<512>
{
  static constexpr int R1 = 8, R2 = 8, R3 = 8;
};

template <int D>
__host__ __device__ constexpr bool is_pow2()
{
  return (D & (D - 1)) == 0;
}
// Threads per block of the tile engine for a grid with a factor 3: 24 slots
// of 16 columns, a multiple of the radix-3 step and of the radix-2/4/8 steps.
constexpr int TILE_THREADS_3 = 384;
template <int D>
constexpr int gen_threads()
{
  return is_pow2<D>() ? FFT_THREADS : TILE_THREADS_3;
}

template <int D>
struct TilePlan
{
  static constexpr int R1 = Split3<D>::R1, R2 = Split3<D>::R2, R3 = Split3<D>::R3, M = R2 * R3;
  static constexpr int BUF = D * TXC;         // float2
  static constexpr int NT = Pitch<D>::HP / TXC;  // tiles over kz
  static_assert(R1 * R2 * R3 == D, "split");
  // position of (line, column) in the tile: a half-warp always reads or
  // writes the 16 columns of one line, 128 bytes over all 32 banks, so no
  // padding is needed
  static __device__ __forceinline__ int at(int line, int t) { return line * TXC + t; }
};

// Inverse DFT of the tile's columns in three steps, each a member of
// TileSteps; the caller puts a barrier between them and after the last one
// before it reuses buf.  tile_dft() runs all three.
//
// Thread roles are fixed: column t = tid % TXC and slot s = tid / TXC of
// S = NTHR / TXC slots (NTHR threads in the block).  A half-warp is the 16 columns of one slot,
// so every shared and global access of a half-warp is one 128-byte line.
// Slot s takes the work items s, s + S, s + 2S, ... of each step; the loops
// over them are unrolled, so their index arithmetic is constant offsets.
template <int D, int NTHR>
struct TileSteps
{
  using P = TilePlan<D>;
  static constexpr int R1 = P::R1, R2 = P::R2, R3 = P::R3, M = P::M;
  static constexpr int S = NTHR / TXC;
  static_assert(S % R2 == 0 && S % R3 == 0, "slot split");
  static constexpr int JA = (M + S - 1) / S;  // step-A items per thread
  static constexpr int NPTS = JA * R1;        // input points per thread

  // f(n, i) for every input point n this thread reads in step A, i its
  // index 0..NPTS-1 (a compile-time constant once the loops are unrolled,
  // so a register array indexed by i stays in registers)
  template <class F>
  static __device__ __forceinline__ void for_each_input(F f)
  {
    const int s = threadIdx.x / TXC;
#pragma unroll
    for (int j = 0; j < JA; j++) {
      const int np = s + S * j;
      if (M % S == 0 || np < M) {
#pragma unroll
        for (int n1 = 0; n1 < R1; n1++)
          f(np + M * n1, j * R1 + n1);
      }
    }
  }

  // step A: items n' = s + S j; load(n, t, i) returns input point n of
  // column t (i as in for_each_input)
  template <class Load>
  static __device__ __forceinline__ void a(float2* buf, const float2* tw, Load load)
  {
    const int t = threadIdx.x % TXC, s = threadIdx.x / TXC;
    float2* col = buf + t;
#pragma unroll
    for (int j = 0; j < JA; j++) {
      const int np = s + S * j;
      if (M % S == 0 || np < M) {
        float2 v[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; n1++)
          v[n1] = load(np + M * n1, t, j * R1 + n1);
        dft_any<R1>(v);
        col[np * TXC] = v[0];
#pragma unroll
        for (int k1 = 1; k1 < R1; k1++)
          col[(k1 * M + np) * TXC] = cmul(v[k1], tw[(np * k1) % D]);
      }
    }
  }

  // step B: items (n3, k1) with n3 = s % R3 fixed
  static __device__ __forceinline__ void b(float2* buf, const float2* tw)
  {
    const int t = threadIdx.x % TXC, s = threadIdx.x / TXC;
    float2* col = buf + t;
    const int n3 = s % R3;
#pragma unroll
    for (int j = 0; j < (R1 * R3 + S - 1) / S; j++) {
      const int k1 = s / R3 + (S / R3) * j;
      if ((R1 * R3) % S == 0 || k1 < R1) {
        float2* line = col + (k1 * M + n3) * TXC;
        float2 v[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; n2++)
          v[n2] = line[R3 * n2 * TXC];
        dft_any<R2>(v);
        line[0] = v[0];
#pragma unroll
        for (int k2 = 1; k2 < R2; k2++)
          line[R3 * k2 * TXC] = cmul(v[k2], tw[(R1 * n3 * k2) % D]);
      }
    }
  }

  // step C: items (k2, k1) with k2 = s % R2 fixed; output k = k1 + R1 (k2 + R2 k3)
  // goes to store(k, t, v)
  template <class Store>
  static __device__ __forceinline__ void c(const float2* buf, Store store)
  {
    const int t = threadIdx.x % TXC, s = threadIdx.x / TXC;
    const float2* col = buf + t;
    const int k2 = s % R2;
#pragma unroll
    for (int j = 0; j < (R1 * R2 + S - 1) / S; j++) {
      const int k1 = s / R2 + (S / R2) * j;
      if ((R1 * R2) % S == 0 || k1 < R1) {
        const float2* line = col + (k1 * M + R3 * k2) * TXC;
        float2 v[R3];
#pragma unroll
        for (int n3 = 0; n3 < R3; n3++)
          v[n3] = line[n3 * TXC];
        dft_any<R3>(v);
#pragma unroll
        for (int k3 = 0; k3 < R3; k3++)
          store(k1 + R1 * (k2 + R2 * k3), t, v[k3]);
      }
    }
  }
};

template <int D, int NTHR, class Load, class Store>
__device__ __forceinline__ void tile_dft(float2* buf, const float2* tw, Load load, Store store)
{
  using T = TileSteps<D, NTHR>;
  T::a(buf, tw, load);
  __syncthreads();
  T::b(buf, tw);
  __syncthreads();
  T::c(buf, store);
}

// ------------------------------------------------------------------ x-pass
// Grid: one block per (|ky| <= D/2, tile of TXC kz columns, radius), the
// radius fastest, so that the blocks of all radii of a tile run together and
// its unfiltered columns are read from HBM once and from L2 by the others.  A
// block computes the filter weights of its tile for its radius (shared by all
// fields and by the rows ky and D - ky, which have the same |k|), then for
// each of the two rows and every field loads the unfiltered columns (rows of
// HP, the forward transform's layout; columns past H are not read), scales by 1/N, multiplies by W(|k| R), inverse-DFTs along x and stores
// to out[(r*G + g) * C + (x*D + ky)*HP + kz], all HP columns (those past H
// are zero in, zero out).
//
// Per-radius weight tables built once per context (read instead of the
// sincosf) measured slower: the table read before the block's barrier is a
// DRAM wait that the weights' arithmetic is not (a 28-radius one-field batch
// at 512^3 took 8.75 ms with tables, 5.90 ms without).
// XTHREADS threads per block: 256 or 512 (the context's autotuner picks).
template <int D, int XTHREADS>
__global__ void __launch_bounds__(XTHREADS, XTHREADS == 256 && D < 512 ? 3 : 2) k_fft_x_filter(const __grid_constant__ XPassArgs a)
{
  using P = TilePlan<D>;
  constexpr int H = D / 2 + 1;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + D;
  float* wsm = reinterpret_cast<float*>(buf + P::BUF);
  fill_twiddles<D>(tw);
  const int r = blockIdx.x % a.n;
  const int tile = blockIdx.x / a.n;
  const int kyp = tile / P::NT;  // |ky|: the block transforms rows ky = kyp and D - kyp
  const int kz0 = (tile % P::NT) * TXC;
  // the weights depend on ky only through kyv^2, the same for both rows
  const float kyv = kcomp(kyp, D, a.delta_k);
  // this thread's column: kz = kz0 + t, the same in every step
  const int t0 = threadIdx.x % TXC;
  const bool live = kz0 + t0 < H;
  // the unfiltered points of step A, read into registers before the step
  using T = TileSteps<D, XTHREADS>;
  float2 pts[T::NPTS];
  auto read_points = [&](int ky, int g) {
    const float2* __restrict__ src = a.in[g] + (long long)ky * Pitch<D>::HP + kz0 + t0;
    T::for_each_input([&](int kx, int i) {
      pts[i] = live ? src[(long long)kx * (D * Pitch<D>::HP)] : make_float2(0.f, 0.f);
    });
  };
  // filter weights of the tile, wsm[|kx| * TXC + t] for |kx| = min(kx, D -
  // kx) <= D/2, then the first field's points (read after the weights, whose
  // sincosf would otherwise push them out of registers; the reads are in
  // flight across the barrier)
  for (int i = threadIdx.x; i < H * TXC; i += XTHREADS) {
    const int kx = i / TXC, t = i % TXC;
    wsm[i] = a.apply[r] ? x_weight(kx, kyv, kz0 + t, D, a.delta_k, a.filter_type, a.R[r], a.sharpk_max, a.scale)
                        : a.scale;
  }
  const float* wcol = wsm + t0;
  const int n_rows = (kyp == 0 || kyp == D / 2) ? 1 : 2;
  for (int h = 0; h < n_rows; h++) {
    const int ky = h == 0 ? kyp : D - kyp;
    read_points(ky, 0);
    if (h == 0)
      __syncthreads();
    // steps B and C of field g after its step A
    auto finish = [&](int g) {
      __syncthreads();
      T::b(buf, tw);
      __syncthreads();
      float2* __restrict__ dst =
        a.out + (long long)(r * a.G + g) * a.C + (long long)ky * Pitch<D>::HP + kz0 + t0;
      T::c(buf, [&](int x, int, float2 v) { dst[(long long)x * (D * Pitch<D>::HP)] = v; });
      __syncthreads();
    };
    auto step_a = [&]() {
      T::a(buf, tw, [&](int kx, int, int i) {
        float2 x = pts[i];
        const float wv = wcol[(kx <= D / 2 ? kx : D - kx) * TXC];
        x.x *= wv;
        x.y *= wv;
        return x;
      });
    };
    step_a();
    finish(0);
    for (int g = 1; g < a.G; g++) {
      read_points(ky, g);
      step_a();
      finish(g);
    }
  }
}

// ------------------------------------------------------------------ y-pass
// Grid: (spectrum, x, tile of TXC kz columns).  In-place inverse DFT along y
// over all HP columns of the pitch.
template <int D, int YTHREADS>
__global__ void __launch_bounds__(YTHREADS, YTHREADS == 256 ? 3 : 2) k_fft_y(float2* data, long long C, int n_spectra)
{
  using P = TilePlan<D>;
  constexpr int HP = Pitch<D>::HP;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + D;
  const long long blk = blockIdx.x;
  const int tile = (int)(blk % P::NT);
  const int x = (int)((blk / P::NT) % D);
  const long long s = blk / ((long long)P::NT * D);
  const int kz0 = tile * TXC;
  float2* col = data + s * C + (long long)x * D * HP + kz0 + threadIdx.x % TXC;
  // the points of step A are read first, so that the reads are in flight
  // while the twiddle table is filled
  using T = TileSteps<D, YTHREADS>;
  float2 pts[T::NPTS];
  T::for_each_input([&](int ky, int i) { pts[i] = col[ky * HP]; });
  fill_twiddles<D>(tw);
  __syncthreads();
  T::a(buf, tw, [&](int, int, int i) { return pts[i]; });
  __syncthreads();
  T::b(buf, tw);
  __syncthreads();
  T::c(buf, [&](int y, int, float2 v) { col[y * HP] = v; });
}

// ------------------------------------------------------------------ z-pass
// The z-pass reads, per block, TZ consecutive rows (row = x * D + y) of every
// spectrum of the batch: TZ rows at the pitch HP, TZ*HP contiguous complex
// values.  These row groups are
// streamed into shared memory by bulk asynchronous copies (cp.async.bulk,
// completion on an mbarrier) through a ZSTAGES-deep ring, so that the copies
// of the next spectra are in flight while the current one is transformed.
namespace {
constexpr int ZSTAGES = 4;
// Geometry of the z-pass.  A block of 256 threads owns TZ = 2048 / D rows
// (2048 cells, 8 per thread).  Each row's C2R of D points is computed as one
// complex inverse DFT of D/2 points: with w = exp(2 pi i / D),
//   Z[k] = E[k] + i O[k],  E[k] = X[k] + conj(X[D/2-k]),
//   O[k] = (X[k] - conj(X[D/2-k])) w^k,        k < D/2,
// and z = IDFT_{D/2}(Z) gives x[2m] = Re z[m], x[2m+1] = Im z[m].
// The D/2 points split as P1 x P2 (four-step); each P-point DFT is done by
// P/4 consecutive lanes holding 4 points each: a 4-point DFT in registers,
// twiddles, then a P/4-point DFT across the lanes (shuffles).  Every thread
// has exactly one lane-part in each of the two steps.
template <int D>
struct ZS;
template <>
struct ZS<32>
{
  static constexpr int P1 = 4, P2 = 4, PAD = 1;
};
template <>
struct ZS<64>
{
  static constexpr int P1 = 8, P2 = 4, PAD = 1;
};
template <>
struct ZS<128>
{
  static constexpr int P1 = 8, P2 = 8, PAD = 2;
};
template <>
struct ZS<256>
{
  static constexpr int P1 = 8, P2 = 16, PAD = 2;
};
template <>
struct ZS<512>
{
  static constexpr int P1 = 16, P2 = 16, PAD = 4;
};

template <int D>
struct ZPlan
{
  static constexpr int H = D / 2 + 1, DH = D / 2;
  static constexpr int TZ = 2048 / D;  // rows per block
  static constexpr int P1 = ZS<D>::P1, P2 = ZS<D>::P2;
  static constexpr int L1 = P1 / 4, L2 = P2 / 4;
  static constexpr int RS = P2 + ZS<D>::PAD;  // padded row of the transpose buffer
  static constexpr int BROW = P1 * RS;
  static constexpr int HP = Pitch<D>::HP;
  static constexpr int STAGE = TZ * HP;  // complex values per stage
  static constexpr int BUF = TZ * BROW;
  static constexpr size_t OFF_STAGE = 64;  // after the barriers
  static constexpr size_t OFF_BUF = OFF_STAGE + sizeof(float2) * (size_t)ZSTAGES * STAGE;
  static constexpr size_t OFF_XS = OFF_BUF + sizeof(float2) * 2 * (size_t)BUF;
  static constexpr int XS_WARP = 4 * 33;  // float2 of lane-transpose scratch per warp
  static constexpr size_t BYTES = OFF_XS + sizeof(float2) * (size_t)XS_WARP * (FFT_THREADS / 32);
  static constexpr size_t BYTES_NO_XS = OFF_XS;  // shuffles instead of the warp scratch
  static_assert(P1 * P2 == DH, "split");
  static_assert(TZ * P2 * L1 == FFT_THREADS && TZ * P1 * L2 == FFT_THREADS, "one lane-part per thread");
  static_assert((sizeof(float2) * STAGE) % 16 == 0, "bulk copy size");
  static_assert(OFF_STAGE % 16 == 0, "bulk copy destination");
  static_assert(D % TZ == 0 || TZ % D == 0, "rows");
};

// index of the output held in slot e by lane-part l of an L-lane DFT
__device__ __forceinline__ int lane_out(int L, int e, int l) { return L == 4 ? l + 4 * e : e + 4 * l; }

__device__ __forceinline__ void dft4_bwd(float2 (&v)[4])
{
  const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  const float2 t2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
  const float2 t3 = make_float2(-d.y, d.x);  // i (v1 - v3)
  v[0] = cadd(t0, t2);
  v[1] = cadd(t1, t3);
  v[2] = csub(t0, t2);
  v[3] = csub(t1, t3);
}

__device__ __forceinline__ float2 shfl_xor2(float2 v, int m)
{
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// The L-point DFT across the L lane-parts (lane l holds u[c] = U_l[c]); on
// return slot e holds output lane_out(L, e, l).
template <int L>
__device__ __forceinline__ void cross_lane(float2 (&u)[4], int l)
{
  if constexpr (L == 2) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float2 p = shfl_xor2(u[c], 1);
      u[c] = l == 0 ? cadd(u[c], p) : csub(p, u[c]);
    }
  } else if constexpr (L == 4) {
    // 4 x 4 transpose across the lanes: slot m of lane q becomes U_m[q]
#pragma unroll
    for (int s = 1; s < 4; s++) {
      const int j = l ^ s;
      const float2 lo = (j & 1) ? u[1] : u[0], hi = (j & 1) ? u[3] : u[2];
      const float2 r = shfl_xor2((j & 2) ? hi : lo, s);
      u[0] = j == 0 ? r : u[0];
      u[1] = j == 1 ? r : u[1];
      u[2] = j == 2 ? r : u[2];
      u[3] = j == 3 ? r : u[3];
    }
    dft4_bwd(u);
  }
}

// The 4-lane step of cross_lane<4> through the warp's shared scratch xs
// (4 rows of 33 float2): lane l of 4-lane group g writes slot c at
// xs[33 c + 4 g + l] and reads slot m from xs[33 l + 4 g + m].  Both are one
// conflict-free pass over the banks (the row pad of one float2 separates the
// four lanes of a group); eight memory operations replace three rounds of
// shuffles and selects.
__device__ __forceinline__ void cross_lane4_smem(float2 (&u)[4], float2* xs)
{
  const int lane = threadIdx.x & 31;
  const int g4 = lane & ~3, l = lane & 3;
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 4; c++)
    xs[33 * c + lane] = u[c];
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 4; m++)
    u[m] = xs[33 * l + g4 + m];
  dft4_bwd(u);
}

// One 4-point lane-part of a P-point DFT whose 4 points (stride L = P/4) are
// in v: 4-point DFT, twiddles exp(2 pi i l c / P) = w1^c (w1 = exp(2 pi i l /
// P)), cross-lane step (through the warp scratch xs for 4 lanes).
template <int P, bool XS>
__device__ __forceinline__ void lane_dft(float2 (&v)[4], int l, const float2 (&w)[3], float2* xs)
{
  dft4_bwd(v);
  if (P > 4) {
    v[1] = cmul(v[1], w[0]);
    v[2] = cmul(v[2], w[1]);
    v[3] = cmul(v[3], w[2]);
  }
  if constexpr (P / 4 == 4 && XS)
    cross_lane4_smem(v, xs);
  else
    cross_lane<P / 4>(v, l);
}

__device__ __forceinline__ float2 unit(int j, int n)
{
  float s, c;
  sincospif(2.0f * (float)j / (float)n, &s, &c);
  return make_float2(c, s);
}

// Per-thread twiddle factors of the z-pass.  A thread's step-A and step-B
// roles are fixed for the whole kernel, so its twiddles are a few base values
// kept in registers; the others follow by complex products.
template <int D>
struct ZTw
{
  float2 kb, kr;  // w_D^k for the 4 points: kb * kr^i
  float2 fb, fs;  // four-step w_{D/2}^{n2 k1} for slot e: fb * fs^e
  float2 la[3], lb[3];  // lane twiddles w, w^2, w^3 of steps A and B
  __device__ __forceinline__ void init()
  {
    constexpr int P1 = ZS<D>::P1, P2 = ZS<D>::P2, L1 = P1 / 4, L2 = P2 / 4, DH = D / 2;
    const int l = threadIdx.x % L1, n2 = (threadIdx.x / L1) % P2;
    kb = unit(n2 + P2 * l, D);
    kr = unit(P2 * L1, D);
    const int k10 = lane_out(L1, 0, l), dk1 = lane_out(L1, 1, l) - k10;
    fb = unit((n2 * k10) % DH, DH);
    fs = unit((n2 * dk1) % DH, DH);
    const int l2 = threadIdx.x % L2;
#pragma unroll
    for (int c = 1; c <= 3; c++) {
      la[c - 1] = unit((l * c) % P1, P1);
      lb[c - 1] = unit((l2 * c) % P2, P2);
    }
  }
};

// Spectrum of ring item `it` when a radius has G fields (spectrum r*G + g):
// the items of a radius take field 2 (weighted_sfr, which the threshold
// reads only for its J_21 / Gamma12 bookkeeping) last.
__device__ __forceinline__ int z_item_spectrum(int it, int G)
{
  if (G <= 3)
    return it;
  const int j = it % G;
  return it - j + (j < 2 ? j : (j < G - 1 ? j + 1 : 2));
}

// Producer side of the ring: thread 0 issues item `it` into stage it % ZSTAGES.
template <int D>
__device__ __forceinline__ void z_issue(char* smem, const float2* spectra, long long C, long long row0, int it,
                                        int G = 1)
{
  using P = ZPlan<D>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  float2* st = reinterpret_cast<float2*>(smem + P::OFF_STAGE) + (size_t)(it % ZSTAGES) * P::STAGE;
  bulk_load(st, spectra + (long long)z_item_spectrum(it, G) * C + row0 * P::HP, (unsigned)(sizeof(float2) * P::STAGE),
            &bars[it % ZSTAGES]);
}

// C2R along z of the TZ staged rows of item `it`.  On return z[e] holds
// (x[2m], x[2m+1]) of row (threadIdx.x / (L2 * P1)) for
// m = k1 + P1 * lane_out(L2, e, l), k1 = (threadIdx.x / L2) % P1,
// l = threadIdx.x % L2.  Returns false (for every thread) if the copy did not
// arrive.  One block barrier per call: the transpose buffer alternates.
template <int D, bool XS>
__device__ __forceinline__ bool z_c2r(char* smem, int it, int n_items, const float2* spectra, long long C,
                                      long long row0, const ZTw<D>& w, float2 (&z)[4], int G = 1)
{
  using P = ZPlan<D>;
  constexpr int H = P::H, DH = P::DH, P1 = P::P1, P2 = P::P2, L1 = P::L1, L2 = P::L2;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  const float2* st = reinterpret_cast<const float2*>(smem + P::OFF_STAGE) + (size_t)(it % ZSTAGES) * P::STAGE;
  float2* buf = reinterpret_cast<float2*>(smem + P::OFF_BUF) + (size_t)(it & 1) * P::BUF;
  float2* xs = reinterpret_cast<float2*>(smem + P::OFF_XS) + (threadIdx.x / 32) * P::XS_WARP;
  const bool arrived = mbar_wait(&bars[it % ZSTAGES], (unsigned)(it / ZSTAGES) & 1u);
  {
    // step A: row t, column n2, lane-part l of the P1-point DFT over n1
    const int l = threadIdx.x % L1, n2 = (threadIdx.x / L1) % P2, t = threadIdx.x / (L1 * P2);
    const float2* row = st + t * P::HP;
    float2 v[4];
    float2 tk = w.kb;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int k = n2 + P2 * (l + L1 * i);
      float2 A = row[k];
      float2 B = row[DH - k];
      if (i == 0 && k == 0) {
        A.y = 0.0f;  // imaginary parts of kz = 0 and kz = D/2 are ignored
        B.y = 0.0f;
      }
      B.y = -B.y;
      const float2 E = cadd(A, B);
      const float2 O = cmul(csub(A, B), tk);
      v[i] = make_float2(E.x - O.y, E.y + O.x);
      if (i < 3)
        tk = cmul(tk, w.kr);
    }
    lane_dft<P1, XS>(v, l, w.la, xs);
    float2 tf = w.fb;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int k1 = lane_out(L1, e, l);
      buf[t * P::BROW + k1 * P::RS + n2] = cmul(v[e], tf);
      if (e < 3)
        tf = cmul(tf, w.fs);
    }
  }
  if (__syncthreads_or(!arrived))
    return false;
  if (threadIdx.x == 0 && it + ZSTAGES < n_items)
    z_issue<D>(smem, spectra, C, row0, it + ZSTAGES, G);
  {
    // step B: row t, k1, lane-part l of the P2-point DFT over n2
    const int l = threadIdx.x % L2, k1 = (threadIdx.x / L2) % P1, t = threadIdx.x / (L2 * P1);
#pragma unroll
    for (int i = 0; i < 4; i++)
      z[i] = buf[t * P::BROW + k1 * P::RS + l + L2 * i];
    lane_dft<P2, XS>(z, l, w.lb, xs);
  }
  return true;
}

// Consumes ring item `it` without transforming it: waits for its copy, then
// (after a block barrier, which also keeps the transpose buffers'
// alternation safe) refills its stage.  Returns false if the copy did not
// arrive.
template <int D>
__device__ __forceinline__ bool z_skip(char* smem, int it, int n_items, const float2* spectra, long long C,
                                       long long row0, int G)
{
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  const bool arrived = mbar_wait(&bars[it % ZSTAGES], (unsigned)(it / ZSTAGES) & 1u);
  if (__syncthreads_or(!arrived))
    return false;
  if (threadIdx.x == 0 && it + ZSTAGES < n_items)
    z_issue<D>(smem, spectra, C, row0, it + ZSTAGES, G);
  return true;
}

// Ring setup: barriers, the first ZSTAGES copies.
template <int D>
__device__ __forceinline__ void z_setup(char* smem, const float2* spectra, long long C, long long row0, int n_items,
                                        int G = 1)
{
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  if (threadIdx.x == 0) {
    for (int s = 0; s < ZSTAGES; s++)
      mbar_init(&bars[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int it = 0; it < ZSTAGES && it < n_items; it++)
      z_issue<D>(smem, spectra, C, row0, it, G);
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
    mbar_drain(&bars[j % ZSTAGES], (unsigned)(j / ZSTAGES) & 1u);
}

// The FP64 decision of the threshold for a cell whose FP32 sides lie within
// 4e-6 of each other, as the reference writes it (find_HII_bubbles.c:348-
// 428): returns whether the cell is ionised and sets the partial xH.  Out of
// line, so that the rare FP64 path does not weigh on the registers and the
// schedule of the per-cell loop.
__device__ __noinline__ bool threshold_fp64(float dx, float stv, float nr, float xe, bool recomb, bool spin,
                                            double M_mean, double R_cubed, double pixel_volume, double eff,
                                            float* xpart)
{
  const double dom = 1.0 + (double)dx;
  const double rec = recomb ? (double)nr / dom : 0.0;
  const double nf = spin ? 1.0 - (double)xe : 1.0;
  const double f_coll = (double)stv / (M_mean * dom) * (4.0 / 3.0) * PI_D * R_cubed / pixel_volume;
  *xpart = (float)__dsub_rn(nf, __dmul_rn(f_coll, eff));
  return f_coll * eff > nf * (1. + rec);
}

// cell state bits of the threshold z-pass
constexpr unsigned ST_ION = 1u;      // ionised at some radius of this launch
constexpr unsigned ST_XHIGH = 2u;    // xH at launch start > REL_TOL
constexpr unsigned ST_XLOW = 4u;     // xH at launch start < REL_TOL
constexpr unsigned ST_ZUNSET = 8u;   // z_at_ionization < 0
constexpr int ST_RB_SHIFT = 8;       // radius index of the last ionising radius
}  // namespace

// z-pass fused with the per-cell test of find_HII_bubbles (clamps
// :271-311, criterion and bookkeeping :342-443) for every radius of the batch.
// Grid: one block per TZ rows.  A thread transforms, for each field of a
// radius, the 8 cells it then tests, so the fields of a cell meet in
// registers.  The cell state is a few bits per cell: whether it is ionised,
// the xH and z_at_ionization tests at launch start, and the index of the last
// ionising radius.  J_21, Gamma12, z_at_ionization and J_21_at_ionization
// change at most once per cell per launch (at the first crossing) and are
// stored when that happens; xH and r_bubble are stored at the end.
//
// SPIN and RECOMB fix the fields at compile time: deltax, stars,
// weighted_sfr, then x_e with the spin temperature, then N_rec with
// recombinations (the order find_HII_bubbles transforms them in).
// MINB: resident blocks per SM the registers are budgeted for (2: 128
// registers; 3: 80, with a few spills); the context picks one.
template <int D, bool SPIN, bool RECOMB, int MINB>
__global__ void __launch_bounds__(FFT_THREADS, MINB) k_fft_z_threshold(ZThresholdArgs a)
{
  using P = ZPlan<D>;
  constexpr int G = 3 + (SPIN ? 1 : 0) + (RECOMB ? 1 : 0);
  constexpr int IXE = 3, INR = SPIN ? 4 : 3;
  extern __shared__ __align__(128) unsigned char zsmem[];
  char* smem = reinterpret_cast<char*>(zsmem);
  const long long row0 = ((long long)blockIdx.x + a.group0) * P::TZ;
  const int n_items = a.n_f * G;
  z_setup<D>(smem, a.spectra, a.C, row0, n_items, G);
  ZTw<D> w;
  w.init();
  // this thread's cells: row t, z = 2 m_e + {0, 1}
  const int l = threadIdx.x % P::L2, k1 = (threadIdx.x / P::L2) % P::P1, t = threadIdx.x / (P::L2 * P::P1);
  const long long rowc = row0 + t;
  int zc[4];
#pragma unroll
  for (int e = 0; e < 4; e++)
    zc[e] = 2 * (k1 + P::P1 * lane_out(P::L2, e, l));
  unsigned st[8];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const long long ir = rowc * D + zc[e];
    const float2 x0 = *reinterpret_cast<const float2*>(a.xH + ir);
    const float2 z0 = *reinterpret_cast<const float2*>(a.z_at_ion + ir);
    st[2 * e] = (x0.x > REL_TOL_F ? ST_XHIGH : 0u) | (x0.x < REL_TOL_F ? ST_XLOW : 0u) | (z0.x < 0 ? ST_ZUNSET : 0u);
    st[2 * e + 1] = (x0.y > REL_TOL_F ? ST_XHIGH : 0u) | (x0.y < REL_TOL_F ? ST_XLOW : 0u) | (z0.y < 0 ? ST_ZUNSET : 0u);
  }
  // weighted_sfr (field 2) enters only the J_21 / Gamma12 values of a cell
  // ionised for the first time at this radius and J_21_at_ionization where
  // z_at_ionization is first set; its transform is skipped for a block with
  // no such cell (its ring item is still consumed)
  const bool need_ws = a.uvb || RECOMB;
  int it = 0;
  for (int r = 0; r < a.n_r; r++) {
    const RadiusParams rp = a.rp[r];
    const bool direct = rp.last != 0;
    float2 f[G][4];
    if (!direct) {
#pragma unroll
      for (int j = 0; j < G - 1; j++) {
        const int g = j < 2 ? j : j + 1;
        if (!z_c2r<D, true>(smem, it, n_items, a.spectra, a.C, row0, w, f[g], G)) {
          z_abort<D>(smem, it, n_items, a.err);
          return;
        }
        it++;
      }
    } else {
#pragma unroll
      for (int g = 0; g < G; g++)
#pragma unroll
        for (int e = 0; e < 4; e++)
          f[g][e] = *reinterpret_cast<const float2*>(a.direct[g] + rowc * 2LL * P::H + zc[e]);
    }
    // the test and the state update; bit c of first_ion / first_z marks a
    // cell whose J_21 / Gamma12 resp. J_21_at_ionization is written below
    unsigned first_ion = 0, first_z = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int e = c >> 1;
      const bool hi = c & 1;
      const float v0 = hi ? f[0][e].y : f[0][e].x;
      const float v1 = hi ? f[1][e].y : f[1][e].x;
      const float dx = fmaxf(v0, -1 + REL_TOL_F);
      float stv = fmaxf(v1, 0.0f);
      if (stv < ABS_TOL_F)
        stv = 0;
      float nr = 0.0f, xe = 0.0f;
      if constexpr (RECOMB) {
        nr = hi ? f[INR][e].y : f[INR][e].x;
        nr = fmaxf(nr, 0.0f);
        if (nr < ABS_TOL_F)
          nr = 0;
      }
      if constexpr (SPIN) {
        xe = hi ? f[IXE][e].y : f[IXE][e].x;
        xe = fmaxf(xe, 0.0f);
        if (xe < ABS_TOL_F)
          xe = 0;
        xe = fminf(xe, 0.999f);
      }
      // FP32 estimate of the test (a 2-ulp reciprocal is well inside the
      // 4e-6 margin below which the FP64 comparison decides)
      const float inv_dom = __fdividef(1.0f, 1.0f + dx);
      const float lhs_f = stv * rp.kfc * inv_dom;
      const float nf_f = 1.0f - xe;
      const float rhs_f = nf_f * (1.0f + nr * inv_dom);
      bool ionised;
      float xpart;
      if (fabsf(lhs_f - rhs_f) > 4e-6f * fmaxf(lhs_f, rhs_f)) {
        ionised = lhs_f > rhs_f;
        xpart = nf_f - lhs_f;
      } else {
        ionised = threshold_fp64(dx, stv, nr, xe, RECOMB, SPIN, rp.M_mean, rp.R_cubed, a.pixel_volume, a.eff, &xpart);
      }
      const long long ir = rowc * D + zc[e] + (hi ? 1 : 0);
      unsigned s = st[c];
      const bool xr_high = !(s & ST_ION) && (s & ST_XHIGH);  // running xH > REL_TOL
      bool xr_low = (s & ST_ION) || (s & ST_XLOW);            // running xH < REL_TOL
      if (ionised) {
        if (xr_high)
          first_ion |= 1u << c;
        s = (s & ((1u << ST_RB_SHIFT) - 1)) | ST_ION | ((unsigned)r << ST_RB_SHIFT);
        xr_low = true;
      } else if (rp.last && xr_high) {
        const float xn = fminf(fmaxf(xpart, 0.0f), 1.0f);
        a.xH[ir] = xn;
        xr_low = xn < REL_TOL_F;
      }
      if (xr_low && (s & ST_ZUNSET)) {
        a.z_at_ion[ir] = (float)a.redshift;
        first_z |= 1u << c;
        s &= ~ST_ZUNSET;
      }
      st[c] = s;
    }
    if (!need_ws)
      first_ion = first_z = 0;
    if (!a.uvb)
      first_z = 0;
    if (!direct) {
      // field 2 of this radius: transformed if a cell of the block needs it
      const bool any = __syncthreads_or((first_ion | first_z) != 0);
      const bool ok = any ? z_c2r<D, true>(smem, it, n_items, a.spectra, a.C, row0, w, f[2], G)
                          : z_skip<D>(smem, it, n_items, a.spectra, a.C, row0, G);
      if (!ok) {
        z_abort<D>(smem, it, n_items, a.err);
        return;
      }
      it++;
    }
#pragma unroll
    for (int c = 0; c < 8; c++) {
      if (!((first_ion | first_z) >> c & 1u))
        continue;
      const int e = c >> 1;
      const bool hi = c & 1;
      const long long ir = rowc * D + zc[e] + (hi ? 1 : 0);
      float ws = fmaxf(hi ? f[2][e].y : f[2][e].x, 0.0f);
      if (ws < ABS_TOL_F)
        ws = 0;
      const float J21_aux = a.uvb ? ws * rp.kj : 0.0f;
      if (first_ion >> c & 1u) {
        if (a.uvb)
          a.J21[ir] = J21_aux;
        if (RECOMB)
          a.Gamma12[ir] = ws * rp.kg;
      }
      if (first_z >> c & 1u)
        a.J21_at_ion[ir] = J21_aux * a.gamma_halo_bias;
    }
  }
#pragma unroll
  for (int c = 0; c < 8; c++) {
    if (st[c] & ST_ION) {
      const long long ir = rowc * D + zc[c >> 1] + (c & 1);
      a.xH[ir] = 0.0f;
      a.r_bubble[ir] = (float)a.rp[st[c] >> ST_RB_SHIFT].R;
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
  extern __shared__ __align__(128) unsigned char zsmem[];
  char* smem = reinterpret_cast<char*>(zsmem);
  const long long row0 = (long long)blockIdx.x * P::TZ;
  z_setup<D>(smem, spectra, C, row0, n);
  ZTw<D> w;
  w.init();
  const int l = threadIdx.x % P::L2, k1 = (threadIdx.x / P::L2) % P::P1, t = threadIdx.x / (P::L2 * P::P1);
  const long long base = (row0 + t) * D;
  for (int r = 0; r < n; r++) {
    float2 z[4];
    if (!z_c2r<D, false>(smem, r, n, spectra, C, row0, w, z)) {
      z_abort<D>(smem, r, n, err);
      return;
    }
    float* dst = shells + (long long)(r0 + r) * N + base;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int zc = 2 * (k1 + P::P1 * lane_out(P::L2, e, l));
      *reinterpret_cast<float2*>(dst + zc) = make_float2(fmaxf(z[e].x, 0.0f), fmaxf(z[e].y, 0.0f));
    }
  }
}


// ------------------------------------------------------- forward transform
// Forward R2C of G padded real grids (the FFTW r2c of find_HII_bubbles.c:
// 118-163 and ComputeTs.c:379-389: unnormalised, exp(-2 pi i jk / n)) in
// three passes, written as spectra [kx][ky][kz] with rows of HP complex
// values (kz >= D/2 + 1 zero), the layout the x-pass reads:
//
//   z-pass   16 rows of a grid per block, read with coalesced loads into
//            shared memory; each row's D real points as D/2 complex points
//            z_m = x_2m + i x_2m+1, transformed by the tile engine (forward
//            as conj(backward(conj))), then X_k = E_k + w_D^-k O_k with
//            E_k = (Z_k + conj Z_{D/2-k}) / 2 and O_k = (Z_k - conj Z_{D/2-k}) / 2i;
//   y-pass, x-pass   forward DFT along y, then x, in place (tiles of 16 kz
//            columns, as the inverse y-pass).
namespace {
constexpr int FWD_ROWS = TXC;  // rows per z-pass block, one per tile column
}

template <int D>
struct FwdZPlan
{
  static constexpr int L = D / 2, H = D / 2 + 1, HP = Pitch<D>::HP;
  // shared memory (float2): twiddles of the L-point engine, w_D^-k for
  // k <= D/2, the engine's tile, and the 16 rows (H float2 each: the padded
  // input row, later the row's Z_k); a row pitch of H = 1 mod 16 float2 puts
  // the 16 rows of a column access on distinct banks
  static constexpr int OFF_TW = 0, OFF_POST = L, OFF_TILE = OFF_POST + H, OFF_ROWS = OFF_TILE + L * TXC;
  static constexpr size_t BYTES = sizeof(float2) * (size_t)(OFF_ROWS + FWD_ROWS * H);
};

template <int D, int T>
__global__ void __launch_bounds__(T) k_fft_z_r2c(const __grid_constant__ FwdArgs a)
{
  using P = FwdZPlan<D>;
  constexpr int L = P::L, H = P::H, HP = P::HP;
  extern __shared__ float2 smem[];
  float2* tw = smem + P::OFF_TW;
  float2* post = smem + P::OFF_POST;
  float2* tile = smem + P::OFF_TILE;
  float2* rows = smem + P::OFF_ROWS;
  constexpr long long GROUPS = (long long)D * D / FWD_ROWS;
  const int g = (int)(blockIdx.x / GROUPS);
  const long long r0 = (blockIdx.x % GROUPS) * FWD_ROWS;
  // the 16 padded rows are contiguous: FWD_ROWS * H float2, all of a
  // thread's loads in flight while the twiddle tables are filled
  const float2* __restrict__ src = reinterpret_cast<const float2*>(a.src[g]) + r0 * H;
  constexpr int NV = (FWD_ROWS * H + T - 1) / T;
  float2 v[NV];
#pragma unroll
  for (int j = 0; j < NV; j++) {
    const int i = threadIdx.x + j * T;
    if (i < FWD_ROWS * H)
      v[j] = __ldg(src + i);
  }
  fill_twiddles<L>(tw);
  for (int k = threadIdx.x; k < H; k += T) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)D, &sn, &cs);
    post[k] = make_float2(cs, -sn);
  }
#pragma unroll
  for (int j = 0; j < NV; j++) {
    const int i = threadIdx.x + j * T;
    if (i < FWD_ROWS * H)
      rows[i] = v[j];
  }
  __syncthreads();
  // forward DFT of each row's L points: conj in, backward engine, conj out
  tile_dft<L, T>(
    tile, tw,
    [&](int n, int t, int) {
      const float2 v = rows[t * H + n];
      return make_float2(v.x, -v.y);
    },
    [&](int k, int t, float2 v) { rows[t * H + k] = make_float2(v.x, -v.y); });
  __syncthreads();
  float2* __restrict__ dst = a.out + (long long)g * a.C + r0 * HP;
  for (int i = threadIdx.x; i < FWD_ROWS * HP; i += T) {
    const int t = i / HP, k = i - t * HP;
    float2 X = make_float2(0.f, 0.f);
    if (k < H) {
      const float2 zk = rows[t * H + (k < L ? k : 0)];
      const float2 zm = rows[t * H + (k > 0 ? L - k : 0)];
      const float2 A = make_float2(zk.x + zm.x, zk.y - zm.y);  // Z_k + conj Z_{L-k}
      const float2 B = make_float2(zk.x - zm.x, zk.y + zm.y);  // Z_k - conj Z_{L-k}
      const float2 C = cmul(B, post[k]);                       // w_D^-k B
      X = make_float2(0.5f * (A.x + C.y), 0.5f * (A.y - C.x)); // (A - i C) / 2
    }
    dst[i] = X;
  }
}

// Forward DFT along y (AXIS 1) or x (AXIS 0) of n spectra [D][D][HP], in
// place, tiles of 16 kz columns; the inverse y-pass's engine with conjugated
// input and output.
template <int D, int T, int AXIS>
__global__ void __launch_bounds__(T, T == 256 ? 3 : 2) k_fft_fwd_cols(float2* data, long long C, int n_spectra)
{
  using P = TilePlan<D>;
  constexpr int HP = Pitch<D>::HP;
  constexpr long long LINE = AXIS == 1 ? HP : (long long)D * HP;   // between the points of a column
  constexpr long long OUTER = AXIS == 1 ? (long long)D * HP : HP;  // between the columns' rows
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + D;
  const long long blk = blockIdx.x;
  const int tile = (int)(blk % P::NT);
  const int o = (int)((blk / P::NT) % D);
  const long long s = blk / ((long long)P::NT * D);
  float2* col = data + s * C + (long long)o * OUTER + tile * TXC + threadIdx.x % TXC;
  using TS = TileSteps<D, T>;
  float2 pts[TS::NPTS];
  TS::for_each_input([&](int n, int i) { pts[i] = col[n * LINE]; });
  fill_twiddles<D>(tw);
  __syncthreads();
  TS::a(buf, tw, [&](int, int, int i) { return make_float2(pts[i].x, -pts[i].y); });
  __syncthreads();
  TS::b(buf, tw);
  __syncthreads();
  TS::c(buf, [&](int y, int, float2 v) { col[y * LINE] = make_float2(v.x, -v.y); });
}


// ------------------------------------------ z-pass for grids with a factor 3
// D = 24, 48, 96, 192.  A block of TILE_THREADS_3 threads owns 16 rows
// (row = x * D + y) and, per spectrum, reads the rows (HP complex values each)
// with coalesced loads into shared memory, forms the D/2-point complex
// sequence Z_k = E_k + i O_k with E_k = X_k + conj X_{D/2-k} and O_k =
// (X_k - conj X_{D/2-k}) w_D^k (the imaginary parts of X_0 and X_{D/2}
// ignored, FFTW c2r), transforms it with the tile engine (16 rows = the 16
// columns of a tile) and keeps x_2m = Re z_m, x_2m+1 = Im z_m of every row in
// shared memory.  The consumer then reads the real rows in cell order.  Shared
// rows are padded to an odd number of words, so that the 16 rows of one tile
// column fall on distinct banks.
namespace {
constexpr int ZG_ROWS = TXC;
}

template <int D>
struct ZGPlan
{
  static constexpr int L = D / 2, H = D / 2 + 1, HP = Pitch<D>::HP;
  static constexpr int RP = HP + 1;  // float2 row pitch of the staged rows
  static constexpr int RD = D + 1;   // float row pitch of the real rows
  static constexpr int OFF_TW = 0, OFF_POST = L, OFF_TILE = OFF_POST + L, OFF_ROWS = OFF_TILE + L * TXC;
  static constexpr int END2 = OFF_ROWS + ZG_ROWS * RP;  // float2
  static constexpr int REAL = ZG_ROWS * RD;              // floats per field
  static constexpr size_t bytes(int fields) { return sizeof(float2) * (size_t)END2 + sizeof(float) * (size_t)fields * REAL; }
};

// Twiddles of the engine (length L) and w_D^k, k < L.
template <int D>
__device__ __forceinline__ void zg_tables(float2* s2)
{
  using P = ZGPlan<D>;
  fill_twiddles<P::L>(s2 + P::OFF_TW);
  for (int k = threadIdx.x; k < P::L; k += TILE_THREADS_3) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)D, &sn, &cs);
    s2[P::OFF_POST + k] = make_float2(cs, sn);
  }
}

// C2R along z of the 16 rows starting at row0 of one spectrum into real
// (16 rows of RD floats).  Starts and ends with a block barrier.
template <int D>
__device__ void zg_c2r(const float2* __restrict__ spectrum, long long row0, float2* s2, float* real)
{
  using P = ZGPlan<D>;
  constexpr int L = P::L, HP = P::HP, RP = P::RP, RD = P::RD;
  float2* rows = s2 + P::OFF_ROWS;
  const float2* post = s2 + P::OFF_POST;
  const float2* __restrict__ src = spectrum + row0 * HP;
  __syncthreads();  // the previous consumer of rows / real is done
  for (int i = threadIdx.x; i < ZG_ROWS * HP; i += TILE_THREADS_3) {
    const int t = i / HP;
    rows[t * RP + (i - t * HP)] = __ldg(src + i);
  }
  __syncthreads();
  tile_dft<L, TILE_THREADS_3>(
    s2 + P::OFF_TILE, s2 + P::OFF_TW,
    [&](int k, int t, int) {
      float2 A = rows[t * RP + k];
      float2 B = rows[t * RP + (L - k)];
      if (k == 0) {
        A.y = 0.0f;
        B.y = 0.0f;
      }
      B.y = -B.y;
      const float2 E = cadd(A, B);
      const float2 O = cmul(csub(A, B), post[k]);
      return make_float2(E.x - O.y, E.y + O.x);
    },
    [&](int m, int t, float2 v) {
      real[t * RD + 2 * m] = v.x;
      real[t * RD + 2 * m + 1] = v.y;
    });
  __syncthreads();
}

// The per-cell test of find_HII_bubbles (find_HII_bubbles.c:342-428) on the
// clamped values of one cell: FP32 with the FP64 decision within 4e-6 of
// threshold, as in k_fft_z_threshold.
template <bool SPIN, bool RECOMB>
__device__ __forceinline__ bool zg_test(float dx, float stv, float nr, float xe, const RadiusParams& rp,
                                        double pixel_volume, double eff, float* xpart)
{
  const float inv_dom = __fdividef(1.0f, 1.0f + dx);
  const float lhs_f = stv * rp.kfc * inv_dom;
  const float nf_f = 1.0f - xe;
  const float rhs_f = nf_f * (1.0f + nr * inv_dom);
  if (fabsf(lhs_f - rhs_f) > 4e-6f * fmaxf(lhs_f, rhs_f)) {
    *xpart = nf_f - lhs_f;
    return lhs_f > rhs_f;
  }
  return threshold_fp64(dx, stv, nr, xe, RECOMB, SPIN, rp.M_mean, rp.R_cubed, pixel_volume, eff, xpart);
}

// z-pass fused with the per-cell test for grids with a factor 3: every field
// of a radius is transformed into shared memory, then each thread tests its
// cells (cell c = threadIdx.x + j * TILE_THREADS_3 of the block's 16 rows).
// Same state, bookkeeping and stores as k_fft_z_threshold.
template <int D, bool SPIN, bool RECOMB>
__global__ void __launch_bounds__(TILE_THREADS_3) k_fft_z_threshold_gen(const __grid_constant__ ZThresholdArgs a)
{
  using P = ZGPlan<D>;
  constexpr int G = 3 + (SPIN ? 1 : 0) + (RECOMB ? 1 : 0);
  constexpr int IXE = 3, INR = SPIN ? 4 : 3;
  constexpr int CELLS = ZG_ROWS * D, CPT = (CELLS + TILE_THREADS_3 - 1) / TILE_THREADS_3;
  extern __shared__ __align__(16) unsigned char zgsm[];
  float2* s2 = reinterpret_cast<float2*>(zgsm);
  float* real = reinterpret_cast<float*>(zgsm + sizeof(float2) * P::END2);
  zg_tables<D>(s2);
  const long long row0 = ((long long)blockIdx.x + a.group0) * ZG_ROWS;
  unsigned st[CPT];
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = threadIdx.x + j * TILE_THREADS_3;
    st[j] = 0;
    if (c < CELLS) {
      const long long ir = row0 * D + c;
      const float x0 = a.xH[ir], z0 = a.z_at_ion[ir];
      st[j] = (x0 > REL_TOL_F ? ST_XHIGH : 0u) | (x0 < REL_TOL_F ? ST_XLOW : 0u) | (z0 < 0 ? ST_ZUNSET : 0u);
    }
  }
  for (int r = 0; r < a.n_r; r++) {
    const RadiusParams rp = a.rp[r];
    const bool direct = rp.last != 0;
    if (!direct) {
      for (int g = 0; g < G; g++)
        zg_c2r<D>(a.spectra + (long long)(r * G + g) * a.C, row0, s2, real + g * P::REAL);
    }
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      const int c = threadIdx.x + j * TILE_THREADS_3;
      if (c >= CELLS)
        continue;
      const int t = c / D, z = c - t * D;
      const long long ir = row0 * D + c;
      float f[G];
#pragma unroll
      for (int g = 0; g < G; g++)
        f[g] = direct ? a.direct[g][(row0 + t) * 2LL * P::H + z] : real[g * P::REAL + t * P::RD + z];
      const float dx = fmaxf(f[0], -1 + REL_TOL_F);
      float stv = fmaxf(f[1], 0.0f);
      if (stv < ABS_TOL_F)
        stv = 0;
      float nr = 0.0f, xe = 0.0f;
      if constexpr (RECOMB) {
        nr = fmaxf(f[INR], 0.0f);
        if (nr < ABS_TOL_F)
          nr = 0;
      }
      if constexpr (SPIN) {
        xe = fmaxf(f[IXE], 0.0f);
        if (xe < ABS_TOL_F)
          xe = 0;
        xe = fminf(xe, 0.999f);
      }
      float xpart;
      const bool ionised = zg_test<SPIN, RECOMB>(dx, stv, nr, xe, rp, a.pixel_volume, a.eff, &xpart);
      unsigned s = st[j];
      const bool xr_high = !(s & ST_ION) && (s & ST_XHIGH);
      bool xr_low = (s & ST_ION) || (s & ST_XLOW);
      bool first_ion = false, first_z = false;
      if (ionised) {
        first_ion = xr_high;
        s = (s & ((1u << ST_RB_SHIFT) - 1)) | ST_ION | ((unsigned)r << ST_RB_SHIFT);
        xr_low = true;
      } else if (rp.last && xr_high) {
        const float xn = fminf(fmaxf(xpart, 0.0f), 1.0f);
        a.xH[ir] = xn;
        xr_low = xn < REL_TOL_F;
      }
      if (xr_low && (s & ST_ZUNSET)) {
        a.z_at_ion[ir] = (float)a.redshift;
        first_z = true;
        s &= ~ST_ZUNSET;
      }
      st[j] = s;
      if ((a.uvb || RECOMB) && (first_ion || (a.uvb && first_z))) {
        float ws = fmaxf(f[2], 0.0f);
        if (ws < ABS_TOL_F)
          ws = 0;
        const float J21_aux = a.uvb ? ws * rp.kj : 0.0f;
        if (first_ion) {
          if (a.uvb)
            a.J21[ir] = J21_aux;
          if (RECOMB)
            a.Gamma12[ir] = ws * rp.kg;
        }
        if (a.uvb && first_z)
          a.J21_at_ion[ir] = J21_aux * a.gamma_halo_bias;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int c = threadIdx.x + j * TILE_THREADS_3;
    if (c < CELLS && (st[j] & ST_ION)) {
      const long long ir = row0 * D + c;
      a.xH[ir] = 0.0f;
      a.r_bubble[ir] = (float)a.rp[st[j] >> ST_RB_SHIFT].R;
    }
  }
}

// Clamped store of ComputeTs shells for grids with a factor 3 (as
// k_fft_z_store): shells[(r0 + r) * N + cell] = max(value, 0).
template <int D>
__global__ void __launch_bounds__(TILE_THREADS_3) k_fft_z_store_gen(const float2* spectra, long long C, int n, int r0,
                                                                     float* shells, long long N)
{
  using P = ZGPlan<D>;
  constexpr int CELLS = ZG_ROWS * D;
  extern __shared__ __align__(16) unsigned char zgsm[];
  float2* s2 = reinterpret_cast<float2*>(zgsm);
  float* real = reinterpret_cast<float*>(zgsm + sizeof(float2) * P::END2);
  zg_tables<D>(s2);
  const long long row0 = (long long)blockIdx.x * ZG_ROWS;
  for (int r = 0; r < n; r++) {
    zg_c2r<D>(spectra + (long long)r * C, row0, s2, real);
    float* dst = shells + (long long)(r0 + r) * N + row0 * D;
    for (int c = threadIdx.x; c < CELLS; c += TILE_THREADS_3) {
      const int t = c / D;
      dst[c] = fmaxf(real[t * P::RD + (c - t * D)], 0.0f);
    }
  }
}

// ------------------------------------------------- adjoint filter (k-space)
// acc = (first ? 0 : acc) + W(|k| R) * scale * U over a half spectrum [D][D][D/2+1]
// with the weights of the x-pass (the filtered shells are a real, symmetric
// convolution, so their adjoint is the same filter).
__global__ void k_filter_accumulate(float2* __restrict__ acc, const float2* __restrict__ U, int D, float R,
                                    int filter_type, float delta_k, float scale, float sharpk_max, int first)
{
  const int H = D / 2 + 1;
  const long long n = (long long)D * D * H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % H);
    const long long row = i / H;
    const int kx = (int)(row / D), ky = (int)(row % D);
    const float kxv = kcomp(kx, D, delta_k), kyv = kcomp(ky, D, delta_k);
    const float kzv = __fmul_rn((float)kz, delta_k);
    const float kmag = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(kyv, kyv)), __fmul_rn(kzv, kzv)));
    bool zero = false;
    float wv = filter_weight(filter_type, kmag, R, sharpk_max, &zero);
    if (zero)
      wv = 0.0f;
    wv *= scale;
    const float2 u = U[i];
    float2 v = first ? make_float2(0.f, 0.f) : acc[i];
    v.x += u.x * wv;
    v.y += u.y * wv;
    acc[i] = v;
  }
}

// ----------------------------------------------------------------- launch
// powers of two from 32 to 512, and 3 x 8, 3 x 16, 3 x 32, 3 x 64 (radix-3
// tile steps, the 384-thread engine and the factor-3 z-pass)
static bool fft3d_factor3(int D) { return D == 24 || D == 48 || D == 96 || D == 192; }
bool fft3d_supported(int D)
{
  return D == 32 || D == 64 || D == 128 || D == 256 || D == 512 || fft3d_factor3(D);
}

int fft_pitch(int D) { return (D / 2 + 1 + TXC - 1) / TXC * TXC; }


template <int D>
constexpr size_t smem_y()
{
  return sizeof(float2) * (D + (size_t)TilePlan<D>::BUF);
}
template <int D>
constexpr size_t smem_x()
{
  return smem_y<D>() + sizeof(float) * (size_t)(D / 2 + 1) * TXC;
}

template <int D, int T>
static void launch_x_t(const XPassArgs& a, cudaStream_t s)
{
  cudaFuncSetAttribute(k_fft_x_filter<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x<D>());
  const long long blocks = (long long)(D / 2 + 1) * TilePlan<D>::NT * a.n;
  k_fft_x_filter<D, T><<<(unsigned)blocks, T, smem_x<D>(), s>>>(a);
}
template <int D>
static void launch_x(const XPassArgs& a, int threads, cudaStream_t s)
{
  if (threads == 256)
    launch_x_t<D, 256>(a, s);
  else
    launch_x_t<D, 512>(a, s);
}
template <int D, int T>
static void launch_y_t(float2* data, long long C, int n_spectra, cudaStream_t s)
{
  const long long blocks = (long long)n_spectra * D * TilePlan<D>::NT;
  cudaFuncSetAttribute(k_fft_y<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y<D>());
  k_fft_y<D, T><<<(unsigned)blocks, T, smem_y<D>(), s>>>(data, C, n_spectra);
}
template <int D>
static void launch_y(float2* data, long long C, int n_spectra, int threads, cudaStream_t s)
{
  if (threads == 512)
    launch_y_t<D, 512>(data, C, n_spectra, s);
  else
    launch_y_t<D, 256>(data, C, n_spectra, s);
}
template <int D, bool SPIN, bool RECOMB, int MINB>
static void launch_zt_minb(const ZThresholdArgs& a, cudaStream_t s)
{
  const size_t bytes = ZPlan<D>::BYTES;
  cudaFuncSetAttribute(k_fft_z_threshold<D, SPIN, RECOMB, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)bytes);
  const int groups = a.n_groups > 0 ? a.n_groups : D * D / ZPlan<D>::TZ;
  k_fft_z_threshold<D, SPIN, RECOMB, MINB><<<groups, FFT_THREADS, bytes, s>>>(a);
}
template <int D, bool SPIN, bool RECOMB>
static void launch_zt_cfg(const ZThresholdArgs& a, cudaStream_t s)
{
  if (a.blocks_per_sm == 3)
    launch_zt_minb<D, SPIN, RECOMB, 3>(a, s);
  else
    launch_zt_minb<D, SPIN, RECOMB, 2>(a, s);
}
template <int D>
static void launch_zt(const ZThresholdArgs& a, cudaStream_t s)
{
  if (a.spin)
    a.recomb ? launch_zt_cfg<D, true, true>(a, s) : launch_zt_cfg<D, true, false>(a, s);
  else
    a.recomb ? launch_zt_cfg<D, false, true>(a, s) : launch_zt_cfg<D, false, false>(a, s);
}
template <int D>
static void launch_zs(const float2* spectra, long long C, int n, int r0, float* shells, long long N, unsigned* err,
                      cudaStream_t s)
{
  const size_t bytes = ZPlan<D>::BYTES_NO_XS;
  cudaFuncSetAttribute(k_fft_z_store<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_fft_z_store<D><<<D * D / ZPlan<D>::TZ, FFT_THREADS, bytes, s>>>(spectra, C, n, r0, shells, N, err);
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

void launch_filter_accumulate(int D, float2* acc, const float2* U, float R, int filter_type, float delta_k,
                              float scale, bool first, cudaStream_t s)
{
  static const float kmax = sharpk_threshold();
  k_filter_accumulate<<<RED_BLOCKS, RED_THREADS, 0, s>>>(acc, U, D, R, filter_type, delta_k, scale, kmax, first ? 1 : 0);
  fft_launches++;
}

bool launch_fft_x_filter(int D, const XPassArgs& args, int threads, cudaStream_t s)
{
  static const float kmax = sharpk_threshold();
  XPassArgs a = args;
  a.sharpk_max = kmax;
  switch (D) {
    case 32: launch_x<32>(a, threads, s); break;
    case 64: launch_x<64>(a, threads, s); break;
    case 128: launch_x<128>(a, threads, s); break;
    case 256: launch_x<256>(a, threads, s); break;
    case 512: launch_x<512>(a, threads, s); break;
    case 24: launch_x_t<24, TILE_THREADS_3>(a, s); break;
    case 48: launch_x_t<48, TILE_THREADS_3>(a, s); break;
    case 96: launch_x_t<96, TILE_THREADS_3>(a, s); break;
    case 192: launch_x_t<192, TILE_THREADS_3>(a, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

bool launch_fft_y(int D, float2* data, long long C, int n_spectra, int threads, cudaStream_t s)
{
  switch (D) {
    case 32: launch_y<32>(data, C, n_spectra, threads, s); break;
    case 64: launch_y<64>(data, C, n_spectra, threads, s); break;
    case 128: launch_y<128>(data, C, n_spectra, threads, s); break;
    case 256: launch_y<256>(data, C, n_spectra, threads, s); break;
    case 512: launch_y<512>(data, C, n_spectra, threads, s); break;
    case 24: launch_y_t<24, TILE_THREADS_3>(data, C, n_spectra, s); break;
    case 48: launch_y_t<48, TILE_THREADS_3>(data, C, n_spectra, s); break;
    case 96: launch_y_t<96, TILE_THREADS_3>(data, C, n_spectra, s); break;
    case 192: launch_y_t<192, TILE_THREADS_3>(data, C, n_spectra, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

int fft_z_rows_per_group(int D) { return fft3d_factor3(D) ? ZG_ROWS : 2048 / D; }

template <int D, int T, int AXIS>
static void launch_fwd_cols_t(float2* data, long long C, int n, cudaStream_t s)
{
  const long long blocks = (long long)n * D * TilePlan<D>::NT;
  cudaFuncSetAttribute(k_fft_fwd_cols<D, T, AXIS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y<D>());
  k_fft_fwd_cols<D, T, AXIS><<<(unsigned)blocks, T, smem_y<D>(), s>>>(data, C, n);
}
template <int D>
static void launch_fwd(const FwdArgs& a, int threads, cudaStream_t s)
{
  const size_t bytes = FwdZPlan<D>::BYTES;
  cudaFuncSetAttribute(k_fft_z_r2c<D, gen_threads<D>()>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  const long long blocks = (long long)a.G * D * D / FWD_ROWS;
  k_fft_z_r2c<D, gen_threads<D>()><<<(unsigned)blocks, gen_threads<D>(), bytes, s>>>(a);
  if constexpr (!is_pow2<D>()) {
    launch_fwd_cols_t<D, TILE_THREADS_3, 1>(a.out, a.C, a.G, s);
    launch_fwd_cols_t<D, TILE_THREADS_3, 0>(a.out, a.C, a.G, s);
  } else if (threads == 512) {
    launch_fwd_cols_t<D, 512, 1>(a.out, a.C, a.G, s);
    launch_fwd_cols_t<D, 512, 0>(a.out, a.C, a.G, s);
  } else {
    launch_fwd_cols_t<D, 256, 1>(a.out, a.C, a.G, s);
    launch_fwd_cols_t<D, 256, 0>(a.out, a.C, a.G, s);
  }
}

bool launch_fft_forward(int D, const FwdArgs& a, int threads, cudaStream_t s)
{
  if (a.G < 1 || a.G > MAX_FIELDS)
    return false;
  switch (D) {
    case 32: launch_fwd<32>(a, threads, s); break;
    case 64: launch_fwd<64>(a, threads, s); break;
    case 128: launch_fwd<128>(a, threads, s); break;
    case 256: launch_fwd<256>(a, threads, s); break;
    case 512: launch_fwd<512>(a, threads, s); break;
    case 24: launch_fwd<24>(a, threads, s); break;
    case 48: launch_fwd<48>(a, threads, s); break;
    case 96: launch_fwd<96>(a, threads, s); break;
    case 192: launch_fwd<192>(a, threads, s); break;
    default: return false;
  }
  fft_launches += 3;
  return true;
}
int fft_z_row_groups(int D) { return D * D / fft_z_rows_per_group(D); }

template <int D, bool SPIN, bool RECOMB>
static void launch_ztg_cfg(const ZThresholdArgs& a, cudaStream_t s)
{
  const size_t bytes = ZGPlan<D>::bytes(3 + (SPIN ? 1 : 0) + (RECOMB ? 1 : 0));
  cudaFuncSetAttribute(k_fft_z_threshold_gen<D, SPIN, RECOMB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)bytes);
  const int groups = a.n_groups > 0 ? a.n_groups : D * D / ZG_ROWS;
  k_fft_z_threshold_gen<D, SPIN, RECOMB><<<groups, TILE_THREADS_3, bytes, s>>>(a);
}
template <int D>
static void launch_ztg(const ZThresholdArgs& a, cudaStream_t s)
{
  if (a.spin)
    a.recomb ? launch_ztg_cfg<D, true, true>(a, s) : launch_ztg_cfg<D, true, false>(a, s);
  else
    a.recomb ? launch_ztg_cfg<D, false, true>(a, s) : launch_ztg_cfg<D, false, false>(a, s);
}
template <int D>
static void launch_zsg(const float2* spectra, long long C, int n, int r0, float* shells, long long N, cudaStream_t s)
{
  const size_t bytes = ZGPlan<D>::bytes(1);
  cudaFuncSetAttribute(k_fft_z_store_gen<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_fft_z_store_gen<D><<<D * D / ZG_ROWS, TILE_THREADS_3, bytes, s>>>(spectra, C, n, r0, shells, N);
}

bool launch_fft_z_threshold(int D, const ZThresholdArgs& a, cudaStream_t s)
{
  if (a.n_groups < 0 || a.group0 < 0 || (a.n_groups == 0 && a.group0 != 0) ||
      (long long)a.group0 + a.n_groups > fft_z_row_groups(D))
    return false;
  // the kernel's fixed field order
  if (a.G != 3 + (a.spin ? 1 : 0) + (a.recomb ? 1 : 0) || a.idx_xe != (a.spin ? 3 : -1) ||
      a.idx_nr != (a.recomb ? (a.spin ? 4 : 3) : -1))
    return false;
  switch (D) {
    case 32: launch_zt<32>(a, s); break;
    case 64: launch_zt<64>(a, s); break;
    case 128: launch_zt<128>(a, s); break;
    case 256: launch_zt<256>(a, s); break;
    case 512: launch_zt<512>(a, s); break;
    case 24: launch_ztg<24>(a, s); break;
    case 48: launch_ztg<48>(a, s); break;
    case 96: launch_ztg<96>(a, s); break;
    case 192: launch_ztg<192>(a, s); break;
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
    case 24: launch_zsg<24>(spectra, C, n, r0, shells, N, s); break;
    case 48: launch_zsg<48>(spectra, C, n, r0, shells, N, s); break;
    case 96: launch_zsg<96>(spectra, C, n, r0, shells, N, s); break;
    case 192: launch_zsg<192>(spectra, C, n, r0, shells, N, s); break;
    default: return false;
  }
  fft_launches++;
  return true;
}

}  // namespace mx
