// C ABI of the GB300 reionization grid step (include/mx_reion.h):
// context, device memory plan, cuFFT plans and the orchestration of
// find_HII_bubbles, ComputeTs and the brightness-temperature box.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <future>
#include <map>
#include <mutex>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "bulk.cuh"
#include "deposit.cuh"
#include "fft3d.cuh"
#include "lightcone.cuh"
#include "pecvel.cuh"
#include "ps.cuh"
#include "host_physics.h"
#include "bulk.cuh"
#include "kernels.cuh"
#include "mx_reion.h"

using namespace mx;

namespace {
thread_local std::string g_create_error;

struct CudaError
{
  int code;
  std::string msg;
};

#define MX_CUDA(call)                                                                                                  \
  do {                                                                                                                 \
    cudaError_t e_ = (call);                                                                                           \
    if (e_ != cudaSuccess)                                                                                             \
      throw CudaError{ MX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_) };                                \
  } while (0)
#define MX_CUFFT(call)                                                                                                 \
  do {                                                                                                                 \
    cufftResult r_ = (call);                                                                                           \
    if (r_ != CUFFT_SUCCESS)                                                                                           \
      throw CudaError{ MX_ECUDA, std::string(#call) + ": cufft status " + std::to_string((int)r_) };                  \
  } while (0)

int hw_threads()
{
  unsigned n = std::thread::hardware_concurrency();
  return n ? (int)n : 4;
}
}  // namespace

struct mx_ctx
{
  mx_params p;
  Derived d;
  GridDims gd;
  std::string err;
  std::string tables_dir;
  std::vector<double> zz;
  int n_hist = 0;
  double stored_fcoll[1000];
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host-pointer mx_step: copies that overlap the compute
  // host-pointer mx_step: ComputeTs's collapse fraction and <x_e> beside the
  // shells (they wait for other uploads); ev_cf marks their sums on the host
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t ev_cf = nullptr;
  bool early_shells = true;  // MX_TS_EARLY_SHELLS=0: the collapse fraction first
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;
  // host-pointer mx_step: ComputeTs inputs arriving on the copy stream
  // (TsUploads)
  cudaEvent_t ev_ts_first = nullptr, ev_ts_sfr = nullptr, ev_ts_tk = nullptr;
  cudaEvent_t ev_state = nullptr;  // find_HII_bubbles state grids uploaded
  std::vector<cudaEvent_t> ev_slices;
  int device = 0;
  int nthreads = 4;
  // inverse transforms: fused three-pass kernels for power-of-two grids
  // (fft3d.cu), cuFFT otherwise or when MX_TRANSFORM=cufft
  bool fused_fft = false;
  // threads per block of the fused x- and y-pass, chosen by tune_fft()
  int x_threads = 512, y_threads = 256;
  // register budget of the threshold z-pass: 2 or 3 resident blocks per SM
  int z_blocks = 2;
  // 2-D tensor map of d_shells (cells x shells) for the evolve kernel's tile
  // copies (make_shell_map), when one applies
  bulk::TensorMap shell_map{};
  bool has_shell_map = false;

  RecombTable rr;
  HeatTables ht;
  float *d_rr_x = nullptr, *d_rr_y = nullptr, *d_rr_c = nullptr;  // FP32 copies, values scaled by rr_scale
  double rr_scale = 1.0;

  // scratch
  float2* d_unf = nullptr;      // MAX_FIELDS x C
  float2* d_work = nullptr;     // batch x work_C
  long long work_fields = 0;    // capacity in spectra
  size_t work_cap_bytes = 0;    // cap on d_work (0: 45% of free memory)
  long long work_C = 0;         // complex values per batch spectrum: D*D*fft_pitch(D) fused, C otherwise
  long long unf_C = 0;          // complex values per unfiltered spectrum in d_unf (same rule)
  float2** d_in_ptrs = nullptr; // device array of MAX_FIELDS pointers
  // light cone (Initialise_ConstructLightcone / ConstructLightcone state)
  long long lc_length = -1, lc_pos = 0;
  int lc_end_snapshot = 0;
  double* d_lc_times = nullptr;  // slice times of one snapshot
  float* d_lc_scratch = nullptr; // host-pointer calls: D*D x max slices per snapshot
  long long lc_max_slices = 0;
  void* d_gal = nullptr;          // galaxy sort keys, indices, CUB scratch, host-copy arrays
  size_t gal_bytes = 0;
  double* d_ps_partials = nullptr; // RED_BLOCKS x 3 x PS_MAX_BINS
  double* d_ps_sums = nullptr;     // 3 x PS_MAX_BINS + 1
  double* h_ps_sums = nullptr;     // pinned copy
  double* d_partials = nullptr; // RED_BLOCKS x 8
  double* d_sums = nullptr;     // 16
  double* h_sums = nullptr;     // pinned, 16
  RadiusParams* d_rp = nullptr;
  TsDevConst* d_tsc = nullptr;
  TsDevConst* h_tsc = nullptr;  // pinned
  float* d_shells = nullptr;    // S x N (spin temperature)
  unsigned int* d_err = nullptr;
  float* d_xe_last = nullptr;
  // device mirror used by the host-pointer entry points
  mx_grids mirror{};
  std::vector<void*> mirror_allocs;
  std::map<long long, cufftHandle> c2r_plans;  // keyed by batch
  cufftHandle r2c_plan = 0;
  // adjoint scratch (allocated by the first adjoint call)
  cufftHandle r2c_real_plan = 0;  // R2C of a REAL-layout grid
  float* d_adj_sfr = nullptr;     // PADDED copy of the SFR grid
  float4* d_adj_dp = nullptr;     // 14 x MAX_SHELLS d/dE0 tables
  double* d_adj_coef = nullptr;   // loss coefficients per bin
  int launches = 0;

  // per-kernel event timing (mx_profile_enable / mx_profile_read)
  struct ProfRec
  {
    const char* name;
    double bytes;
    int ev;  // index of the start event; the stop event is ev + 1
  };
  bool prof_on = false;
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> prof_events;

  // Whole-step CUDA graph (mx_set_step_graph): mx_step_device captures
  // ComputeTs -> find_HII_bubbles -> 21cm box on the context stream and
  // launches the step as one graph.  While capturing, values read back from
  // the device land in pinned slots of h_stage and the code that uses them
  // (`finishers`) runs after the graph has completed; host data uploaded by
  // the step is staged in h_stage too, so that it outlives the capture.
  // ComputeTs's frequency tables are built by a host node of the graph.
  bool graph_on = false;
  bool capturing = false;
  unsigned char* h_stage = nullptr;  // pinned, STAGE_BYTES
  size_t stage_used = 0;
  std::vector<std::function<void()>> finishers;
  std::vector<std::shared_ptr<void>> graph_keep;  // host-node payloads of the step being captured

  ~mx_ctx();
  void alloc_scratch();
  void make_shell_map();
  cufftHandle c2r_plan(long long batch);
  void ensure_mirror();
};

// Records CUDA events around one kernel (or cuFFT execution) on its stream
// when profiling is on; `bytes` is the launch's algorithmic HBM traffic.
class Prof
{
 public:
  Prof(mx_ctx* c, const char* name, double bytes, cudaStream_t s) : c_(c), s_(s)
  {
    if (!c->prof_on)
      return;
    const int ev = (int)c->prof.size() * 2;
    while ((int)c->prof_events.size() < ev + 2) {
      cudaEvent_t e;
      MX_CUDA(cudaEventCreate(&e));
      c->prof_events.push_back(e);
    }
    c->prof.push_back({ name, bytes, ev });
    idx_ = ev;
    MX_CUDA(record(c->prof_events[ev]));
  }
  ~Prof()
  {
    if (idx_ >= 0)
      record(c_->prof_events[idx_ + 1]);
  }

 private:
  // inside a captured step the record is an event node of the graph
  cudaError_t record(cudaEvent_t e)
  {
    return c_->capturing ? cudaEventRecordWithFlags(e, s_, cudaEventRecordExternal) : cudaEventRecord(e, s_);
  }

 public:

 private:
  mx_ctx* c_;
  cudaStream_t s_;
  int idx_ = -1;
};

// pinned staging of a step: read-back slots and uploads (graph capture)
constexpr size_t STAGE_BYTES = 1 << 20;

static void* stage(mx_ctx* c, size_t bytes)
{
  const size_t b = (bytes + 255) & ~(size_t)255;
  if (c->stage_used + b > STAGE_BYTES)
    throw CudaError{ MX_ENOTSUP, "step staging area exhausted" };
  void* q = c->h_stage + c->stage_used;
  c->stage_used += b;
  return q;
}

// n values of type T read back from device memory into a pinned slot; the
// slot is valid in the code passed to after()
template <class T>
static const T* readback(mx_ctx* c, const T* dsrc, int n, cudaStream_t s)
{
  T* h = static_cast<T*>(stage(c, sizeof(T) * (size_t)n));
  MX_CUDA(cudaMemcpyAsync(h, dsrc, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost, s));
  return h;
}

// Runs f once the work queued on s so far has completed: now (after a
// synchronize) outside a capture, after the graph's completion inside one.
template <class F>
static void after(mx_ctx* c, cudaStream_t s, F&& f)
{
  if (c->capturing) {
    c->finishers.emplace_back(std::forward<F>(f));
    return;
  }
  MX_CUDA(cudaStreamSynchronize(s));
  c->stage_used = 0;
  f();
}

// Host -> device copy of data that the caller may overwrite after the call
// returns: staged in pinned memory while capturing.
static void upload(mx_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s)
{
  if (c->capturing) {
    void* q = stage(c, bytes);
    std::memcpy(q, src, bytes);
    src = q;
  }
  MX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
}

mx_ctx::~mx_ctx()
{
  cudaFreeHost(h_stage);
  for (cudaEvent_t e : prof_events)
    cudaEventDestroy(e);
  for (auto& kv : c2r_plans)
    cufftDestroy(kv.second);
  if (r2c_plan)
    cufftDestroy(r2c_plan);
  if (r2c_real_plan)
    cufftDestroy(r2c_real_plan);
  cudaFree(d_adj_sfr);
  cudaFree(d_adj_dp);
  cudaFree(d_adj_coef);
  cudaFree(d_unf);
  cudaFree(d_work);
  cudaFree(d_in_ptrs);
  cudaFree(d_lc_times);
  cudaFree(d_lc_scratch);
  cudaFree(d_gal);
  cudaFree(d_ps_partials);
  cudaFree(d_ps_sums);
  cudaFreeHost(h_ps_sums);
  cudaFree(d_partials);
  cudaFree(d_sums);
  cudaFreeHost(h_sums);
  cudaFree(d_rp);
  cudaFree(d_tsc);
  cudaFreeHost(h_tsc);
  cudaFree(d_shells);
  cudaFree(d_err);
  cudaFree(d_xe_last);
  cudaFree(d_rr_x);
  cudaFree(d_rr_y);
  cudaFree(d_rr_c);
  for (void* q : mirror_allocs)
    cudaFree(q);
  if (ev_a)
    cudaEventDestroy(ev_a);
  if (ev_b)
    cudaEventDestroy(ev_b);
  for (cudaEvent_t e : { ev_ts_first, ev_ts_sfr, ev_ts_tk, ev_state, ev_cf })
    if (e)
      cudaEventDestroy(e);
  for (cudaEvent_t e : ev_slices)
    cudaEventDestroy(e);
  if (copy_stream)
    cudaStreamDestroy(copy_stream);
  if (aux_stream)
    cudaStreamDestroy(aux_stream);
  if (stream)
    cudaStreamDestroy(stream);
}

static int n_fields(const mx_params& p) { return 3 + (p.flag_spin_temp ? 1 : 0) + (p.flag_recombinations ? 1 : 0); }

// The evolve kernel's tensor map of the shells: a 2-D FP32 tensor of N cells
// (inner) by S shells (rows N * 4 bytes apart), box EV_TILE x S.  Encoded
// through the runtime's driver entry point, so the library does not link the
// driver API.  Left out (per-row bulk copies instead) when it does not apply
// or MX_SHELL_MAP=0.
void mx_ctx::make_shell_map()
{
  has_shell_map = false;
  const int S = p.ts_num_filter_steps;
  const char* env = std::getenv("MX_SHELL_MAP");
  if ((env && std::string(env) == "0") || !ev_shell_map_ok(gd.N, S))
    return;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return;
  static_assert(sizeof(CUtensorMap) == sizeof(bulk::TensorMap), "tensor map size");
  CUtensorMap m;
  const cuuint64_t dims[2] = { (cuuint64_t)gd.N, (cuuint64_t)S };
  const cuuint64_t strides[1] = { (cuuint64_t)gd.N * sizeof(float) };
  const cuuint32_t box[2] = { (cuuint32_t)RED_THREADS, (cuuint32_t)S };
  const cuuint32_t estr[2] = { 1, 1 };
  const CUresult r = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn)(
    &m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, d_shells, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return;
  std::memcpy(&shell_map, &m, sizeof(m));
  has_shell_map = true;
}

void mx_ctx::alloc_scratch()
{
  const int G = n_fields(p);
  // unfiltered spectra: rows of fft_pitch(D) on the fused path (its forward
  // transform's layout), of D/2 + 1 (cuFFT's) otherwise; the other users of
  // this scratch index it in slots of C
  unf_C = fused_fft ? (long long)gd.D * gd.D * fft_pitch(gd.D) : gd.C;
  MX_CUDA(cudaMalloc(&d_unf, sizeof(float2) * std::max(gd.C, unf_C) * MAX_FIELDS));
  // Radius batch: as many (radius, field) spectra as the memory plan allows,
  // up to all radii of the snapshot.
  const std::vector<double> radii = filter_radii(p);
  size_t free_b = 0, total_b = 0;
  MX_CUDA(cudaMemGetInfo(&free_b, &total_b));
  work_C = fused_fft ? (long long)gd.D * gd.D * fft_pitch(gd.D) : gd.C;
  const double spectrum = (double)sizeof(float2) * work_C;
  const long long want = (long long)radii.size() * G;
  long long fit = (long long)(0.45 * (double)free_b / spectrum);
  if (work_cap_bytes)
    fit = std::min(fit, (long long)((double)work_cap_bytes / spectrum));
  if (const char* env = std::getenv("MX_MAX_BATCH_SPECTRA"))
    fit = std::min(fit, (long long)std::atoll(env));
  long long cap = std::max<long long>(G, std::min(want, fit));
  cap = std::max<long long>(G, (cap / G) * G);
  if (p.flag_spin_temp)
    cap = std::max<long long>(cap, 1);
  work_fields = cap;
  MX_CUDA(cudaMalloc(&d_work, spectrum * cap));
  MX_CUDA(cudaMalloc(&d_in_ptrs, sizeof(float2*) * MAX_FIELDS));
  MX_CUDA(cudaMalloc(&d_partials, sizeof(double) * RED_BLOCKS * 8));
  MX_CUDA(cudaMalloc(&d_ps_partials, sizeof(double) * RED_BLOCKS * 3 * PS_MAX_BINS));
  MX_CUDA(cudaMalloc(&d_ps_sums, sizeof(double) * (3 * PS_MAX_BINS + 1)));
  MX_CUDA(cudaMallocHost(&h_ps_sums, sizeof(double) * (3 * PS_MAX_BINS + 1)));
  MX_CUDA(cudaMalloc(&d_sums, sizeof(double) * 16));
  MX_CUDA(cudaMallocHost(&h_sums, sizeof(double) * 16));
  MX_CUDA(cudaMallocHost(&h_stage, STAGE_BYTES));
  MX_CUDA(cudaMalloc(&d_rp, sizeof(RadiusParams) * MAX_RADII));
  MX_CUDA(cudaMalloc(&d_err, sizeof(unsigned int)));
  MX_CUDA(cudaMemset(d_err, 0, sizeof(unsigned int)));
  MX_CUDA(cudaMalloc(&d_xe_last, sizeof(float)));
  if (p.flag_spin_temp) {
    MX_CUDA(cudaMalloc(&d_tsc, sizeof(TsDevConst)));
    MX_CUDA(cudaMallocHost(&h_tsc, sizeof(TsDevConst)));
    MX_CUDA(cudaMalloc(&d_shells, sizeof(float) * gd.N * (size_t)p.ts_num_filter_steps));
    make_shell_map();
  }
  // forward transform: padded real input -> half spectrum (out of place)
  int n[3] = { gd.D, gd.D, gd.D };
  int inembed[3] = { gd.D, gd.D, 2 * gd.H };
  int onembed[3] = { gd.D, gd.D, gd.H };
  MX_CUFFT(cufftPlanMany(&r2c_plan, 3, n, inembed, 1, (int)gd.P, onembed, 1, (int)gd.C, CUFFT_R2C, 1));
  MX_CUFFT(cufftSetStream(r2c_plan, stream));
}

cufftHandle mx_ctx::c2r_plan(long long batch)
{
  auto it = c2r_plans.find(batch);
  if (it != c2r_plans.end())
    return it->second;
  cufftHandle h;
  int n[3] = { gd.D, gd.D, gd.D };
  int inembed[3] = { gd.D, gd.D, gd.H };
  int onembed[3] = { gd.D, gd.D, 2 * gd.H };
  MX_CUFFT(cufftPlanMany(&h, 3, n, inembed, 1, (int)gd.C, onembed, 1, (int)gd.P, CUFFT_C2R, (int)batch));
  MX_CUFFT(cufftSetStream(h, stream));
  c2r_plans[batch] = h;
  return h;
}

void mx_ctx::ensure_mirror()
{
  if (mirror.deltax)
    return;
  float** f[] = { &mirror.deltax, &mirror.stars, &mirror.weighted_sfr, &mirror.sfr, &mirror.N_rec, &mirror.x_e_box,
                  &mirror.x_e_box_prev, &mirror.vel };
  for (float** q : f) {
    MX_CUDA(cudaMalloc((void**)q, sizeof(float) * gd.P));
    MX_CUDA(cudaMemset(*q, 0, sizeof(float) * gd.P));
    mirror_allocs.push_back(*q);
  }
  float** r[] = { &mirror.Tk_box, &mirror.TS_box, &mirror.xH, &mirror.z_at_ionization, &mirror.r_bubble,
                  &mirror.J_21, &mirror.J_21_at_ionization, &mirror.Gamma12, &mirror.delta_T };
  for (float** q : r) {
    MX_CUDA(cudaMalloc((void**)q, sizeof(float) * gd.N));
    MX_CUDA(cudaMemset(*q, 0, sizeof(float) * gd.N));
    mirror_allocs.push_back(*q);
  }
  if (p.flag_spin_temp && n_hist > 0) {
    MX_CUDA(cudaMalloc((void**)&mirror.sfr_histories, sizeof(float) * gd.P * n_hist));
    mirror_allocs.push_back(mirror.sfr_histories);
  }
}

// ======================================================================
// find_HII_bubbles (src/core/find_HII_bubbles.c:47-495)
// ======================================================================
// Outputs of find_HII_bubbles that a host-pointer call copies back slab by
// slab: the last radius batch's threshold z-pass runs as `slabs` launches
// over row slabs, and after each one the copy stream (which waits on `ev`)
// copies that slab's rows of xH, z_at_ionization, r_bubble, J_21,
// J_21_at_ionization and Gamma12 into `host`, while the next slab computes.
// `done` is set when that happened (fused transforms only).
// `state_in` (if set): the event after which the state grids the threshold
// reads first (z_at_ionization, J_21_at_ionization, Gamma12) are on the
// device; the first threshold launch waits for it.
struct FhbDownloads
{
  cudaStream_t cs;
  cudaEvent_t ev;
  const mx_grids* host;
  int slabs;
  bool done;
  cudaEvent_t state_in;
};

float* mx_grids::* const SLAB_OUTPUTS[] = { &mx_grids::xH,   &mx_grids::z_at_ionization,    &mx_grids::r_bubble,
                                             &mx_grids::J_21, &mx_grids::J_21_at_ionization, &mx_grids::Gamma12 };

// x- and y-pass of a batch of xa.n radii x xa.G fields into xa.out.
// Algorithmic bytes: the unfiltered spectra read once and the filtered ones
// written (x-pass), the filtered ones read and written (y-pass).
static void run_xy(mx_ctx* c, const XPassArgs& xa, cudaStream_t s)
{
  const double B8C = 8.0 * (double)c->gd.C;
  const double x_bytes = B8C * xa.G * (1 + xa.n), y_bytes = 2.0 * B8C * xa.G * xa.n;
  {
    Prof pr(c, "fft_x_filter", x_bytes, s);
    launch_fft_x_filter(c->gd.D, xa, c->x_threads, s);
  }
  Prof pr(c, "fft_y", y_bytes, s);
  launch_fft_y(c->gd.D, xa.out, xa.C, xa.n * xa.G, c->y_threads, s);
}

static void run_find_HII_bubbles(mx_ctx* c, int snapshot, const mx_grids* g, mx_globals* out, cudaStream_t s,
                                 FhbDownloads* dl = nullptr)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const int uvb = p.uvb_flag, recomb = p.flag_recombinations, spin = p.flag_spin_temp;
  const double redshift = c->zz[snapshot];
  const double prev_z = snapshot == 0 ? c->zz[snapshot] : c->zz[snapshot - 1];
  const float zstep = (float)(prev_z - redshift);
  const float fabs_dtdz = (float)std::fabs(dtdz(p, (float)redshift) / p.hubble_h);
  const double pixel_volume = std::pow(p.box_size / (double)gd.D, 3);
  const int launches0 = kernel_launch_count();

  if (!g->deltax || !g->stars || !g->weighted_sfr || !g->xH || !g->z_at_ionization || !g->r_bubble ||
      (uvb && (!g->J_21 || !g->J_21_at_ionization)) || (recomb && (!g->N_rec || !g->Gamma12)) ||
      (spin && !g->x_e_box))
    throw CudaError{ MX_EINVAL, "find_HII_bubbles: a required grid pointer is NULL" };

  // initial state (find_HII_bubbles.c:102-116)
  const double B4N = 4.0 * (double)gd.N, B8C = 8.0 * (double)gd.C;
  if (uvb) {
    Prof pr(c, "k_fill", B4N, s);
    launch_fill(g->J_21, gd.N, 0.0f, s);
  }
  {
    Prof pr(c, "k_fill", 2 * B4N, s);
    launch_fill(g->xH, gd.N, 1.0f, s);
    launch_fill(g->r_bubble, gd.N, 0.0f, s);
  }

  // forward transforms of the G fields (find_HII_bubbles.c:118-163)
  const float* src[MAX_FIELDS];
  int G = 0, idx_xe = -1, idx_nr = -1;
  src[G++] = g->deltax;
  src[G++] = g->stars;
  src[G++] = g->weighted_sfr;
  if (spin) {
    idx_xe = G;
    src[G++] = g->x_e_box;
  }
  if (recomb) {
    idx_nr = G;
    src[G++] = g->N_rec;
  }
  float2* unf_ptrs[MAX_FIELDS];
  for (int f = 0; f < G; f++)
    unf_ptrs[f] = c->d_unf + (long long)f * c->unf_C;
  if (c->fused_fft) {
    // hand-written forward transform of all G fields (fft3d.cu)
    FwdArgs fa;
    for (int f = 0; f < MAX_FIELDS; f++)
      fa.src[f] = f < G ? src[f] : nullptr;
    fa.G = G;
    fa.out = c->d_unf;
    fa.C = c->unf_C;
    const double BC = 8.0 * (double)c->unf_C;
    Prof pr(c, "fft_forward", G * (B4N * (gd.D + 2) / gd.D + 5.0 * BC), s);
    launch_fft_forward(gd.D, fa, c->y_threads, s);
  } else {
    for (int f = 0; f < G; f++) {
      MX_CUFFT(cufftSetStream(c->r2c_plan, s));
      Prof pr(c, "cufft_r2c", B4N + B8C, s);
      MX_CUFFT(cufftExecR2C(c->r2c_plan, (cufftReal*)src[f], (cufftComplex*)unf_ptrs[f]));
    }
  }
  if (!c->fused_fft)
    upload(c, c->d_in_ptrs, unf_ptrs, sizeof(float2*) * G, s);

  // radius schedule (find_HII_bubbles.c:184-207)
  const std::vector<double> radii = filter_radii(p);
  const int nR = (int)radii.size();
  if (nR > MAX_RADII)
    throw CudaError{ MX_ENOTSUP, "too many filter radii" };
  std::vector<RadiusParams> rps(nR);
  for (int r = 0; r < nR; r++) {
    const double R = radii[r];
    RadiusParams& q = rps[r];
    q.R = R;
    q.last = (r == nR - 1);
    q.M_mean = RtoM(p, c->d, R);
    q.R_cubed = R * R * R;
    q.J21_const = (1.0 + redshift) * (1.0 + redshift) / (4.0 * k::PI) * p.alpha_uv * k::PLANCK * 1e21 * R *
                  p.unit_length_cm * p.nion_phot_per_bary / k::PROTONMASS * p.unit_mass_g /
                  std::pow(p.unit_length_cm, 3) / c->d.unit_time_s;
    q.Gamma_pref = 0;
    if (recomb) {
      q.Gamma_pref = (1.0 + redshift) * (1.0 + redshift) * R * (p.unit_length_cm / p.hubble_h) * k::SIGMA_HI *
                     p.alpha_uv / (p.alpha_uv + 2.75) / 1.0e-12;
      q.Gamma_pref *= (p.unit_mass_g / c->d.unit_time_s) * std::pow(p.unit_length_cm / p.hubble_h, -3.) *
                      p.nion_phot_per_bary / k::PROTONMASS;
    }
    q.kfc = (float)(p.reion_efficiency * (4.0 / 3.0) * k::PI * q.R_cubed / (q.M_mean * pixel_volume));
    q.kj = (float)(q.J21_const / pixel_volume);
    q.kg = (float)(q.Gamma_pref / pixel_volume);
  }
  upload(c, c->d_rp, rps.data(), sizeof(RadiusParams) * nR, s);

  // batched filter -> C2R -> threshold over chunks of radii, largest first.
  // A host call (whose output copies overlap the last batch's threshold
  // pass) puts the remainder first, so that the last batch is a full one;
  // otherwise the remainder goes last, where a remainder of only the
  // unfiltered step needs no transforms.  The grids do not depend on it.
  const int per_batch = (int)std::max<long long>(1, c->work_fields / G);
  const int n_batches = (nR + per_batch - 1) / per_batch;
  const int rem = nR - (n_batches - 1) * per_batch;
  auto batch_size = [&](int i) { return dl ? (i == 0 ? rem : per_batch) : (i == n_batches - 1 ? rem : per_batch); };
  for (int bi = 0, r0 = 0, nb = batch_size(0); r0 < nR; r0 += nb, nb = batch_size(++bi)) {
    // the last, unfiltered step is read from the input grids (identity transform)
    const int nf = (r0 + nb == nR) ? nb - 1 : nb;
    const int nstate = 3 + (uvb ? 2 : 0) + (recomb ? 1 : 0);
    if (c->fused_fft) {
      // fused three-pass inverse transform (fft3d.cu)
      if (nf > 0) {
        XPassArgs xa;
        for (int f = 0; f < MAX_FIELDS; f++)
          xa.in[f] = f < G ? unf_ptrs[f] : nullptr;
        xa.G = G;
        xa.n = nf;
        xa.out = c->d_work;
        xa.C = c->work_C;
        for (int r = 0; r < nf; r++) {
          xa.R[r] = (float)radii[r0 + r];
          xa.apply[r] = 1;
        }
        xa.filter_type = p.filter_type;
        xa.delta_k = (float)(2.0 * k::PI / (float)p.box_size);
        xa.scale = (float)(1.0 / (double)gd.N);
        run_xy(c, xa, s);
      }
      if (dl && dl->state_in && r0 == 0)
        MX_CUDA(cudaStreamWaitEvent(s, dl->state_in, 0));
      ZThresholdArgs za;
      za.spectra = c->d_work;
      za.C = c->work_C;
      za.G = G;
      za.idx_xe = idx_xe;
      za.idx_nr = idx_nr;
      za.n_r = nb;
      za.n_f = nf;
      za.rp = c->d_rp + r0;
      for (int f = 0; f < MAX_FIELDS; f++)
        za.direct[f] = f < G ? src[f] : nullptr;
      za.xH = g->xH;
      za.z_at_ion = g->z_at_ionization;
      za.r_bubble = g->r_bubble;
      za.J21 = g->J_21;
      za.J21_at_ion = g->J_21_at_ionization;
      za.Gamma12 = g->Gamma12;
      za.pixel_volume = pixel_volume;
      za.eff = p.reion_efficiency;
      za.redshift = redshift;
      za.gamma_halo_bias = (float)p.gamma_halo_bias;
      za.uvb = uvb;
      za.recomb = recomb;
      za.spin = spin;
      za.err = c->d_err;
      za.blocks_per_sm = c->z_blocks;
      // spectra read once, unfiltered last step read once, and the per-call
      // state (xH, z_at_ionization read and written; r_bubble, J_21,
      // J_21_at_ionization, Gamma12 written) counted with the first batch
      Prof pr(c, "fft_z_threshold",
              (double)G * nf * B8C + (double)(nb - nf) * G * B4N + (r0 == 0 ? 8.0 * B4N : 0.0), s);
      if (!dl || r0 + nb < nR) {
        if (!launch_fft_z_threshold(gd.D, za, s))
          throw CudaError{ MX_ECUDA, "find_HII_bubbles: field layout does not match the fused z-pass" };
        continue;
      }
      // last batch of a host call: row slabs, each slab's outputs copied
      // back while the next computes
      const int groups = fft_z_row_groups(gd.D);
      const int K = std::max(1, std::min(dl->slabs, groups));
      const long long cells_per_group = (long long)fft_z_rows_per_group(gd.D) * gd.D;
      for (int k = 0; k < K; k++) {
        za.group0 = (int)((long long)groups * k / K);
        za.n_groups = (int)((long long)groups * (k + 1) / K) - za.group0;
        if (!launch_fft_z_threshold(gd.D, za, s))
          throw CudaError{ MX_ECUDA, "find_HII_bubbles: field layout does not match the fused z-pass" };
        MX_CUDA(cudaEventRecord(dl->ev, s));
        MX_CUDA(cudaStreamWaitEvent(dl->cs, dl->ev, 0));
        const long long cell0 = za.group0 * cells_per_group, cells = za.n_groups * cells_per_group;
        for (float* mx_grids::*m : SLAB_OUTPUTS)
          if (dl->host->*m && g->*m)
            MX_CUDA(cudaMemcpyAsync(dl->host->*m + cell0, g->*m + cell0, sizeof(float) * cells,
                                    cudaMemcpyDeviceToHost, dl->cs));
      }
      dl->done = true;
      continue;
    }
    FilterBatch fb;
    fb.n = nf;
    fb.filter_type = p.filter_type;
    fb.scale_mode = 0;
    for (int r = 0; r < nf; r++) {
      fb.R[r] = (float)radii[r0 + r];
      fb.apply[r] = 1;
    }
    if (nf > 0) {
      Prof pr(c, "k_filter", (double)G * B8C * (1 + nf), s);
      launch_filter((const float2* const*)c->d_in_ptrs, G, c->d_work, gd.C, fb, gd, (float)p.box_size, s);
    }
    // one radius (G fields) per cuFFT execution keeps the cuFFT work area at
    // the size of one radius' spectra
    const cufftHandle plan = c->c2r_plan(G);
    MX_CUFFT(cufftSetStream(plan, s));
    for (int r = 0; r < nf; r++) {
      cufftComplex* w = (cufftComplex*)(c->d_work + (long long)r * G * gd.C);
      Prof pr(c, "cufft_c2r", (double)G * (B8C + B4N), s);
      MX_CUFFT(cufftExecC2R(plan, w, (cufftReal*)w));
    }
    if (dl && dl->state_in && r0 == 0)
      MX_CUDA(cudaStreamWaitEvent(s, dl->state_in, 0));
    ThresholdArgs ta;
    ta.fields = (const float*)c->d_work;
    ta.P = gd.P;
    ta.G = G;
    ta.idx_xe = idx_xe;
    ta.idx_nr = idx_nr;
    ta.n_r = nb;
    ta.rp = c->d_rp + r0;
    for (int f = 0; f < MAX_FIELDS; f++)
      ta.direct[f] = f < G ? src[f] : nullptr;
    ta.xH = g->xH;
    ta.z_at_ion = g->z_at_ionization;
    ta.r_bubble = g->r_bubble;
    ta.J21 = g->J_21;
    ta.J21_at_ion = g->J_21_at_ionization;
    ta.Gamma12 = g->Gamma12;
    ta.pixel_volume = pixel_volume;
    ta.eff = p.reion_efficiency;
    ta.redshift = redshift;
    ta.gamma_halo_bias = (float)p.gamma_halo_bias;
    ta.uvb = uvb;
    ta.recomb = recomb;
    ta.spin = spin;
    Prof pr(c, "k_threshold", ((double)nb * G + 2.0 * nstate) * B4N, s);
    launch_threshold(ta, gd, s);
  }

  // global means and N_rec (find_HII_bubbles.c:451-494)
  FhbReduceArgs ra;
  ra.xH = g->xH;
  ra.J21 = g->J_21;
  ra.deltax = g->deltax;
  ra.Gamma12 = g->Gamma12;
  ra.N_rec = g->N_rec;
  ra.rr_xf = c->d_rr_x;
  ra.rr_yf = c->d_rr_y;
  ra.rr_cf = c->d_rr_c;
  ra.rr_scale_inv = (float)(1.0 / c->rr_scale);
  ra.redshift = redshift;
  ra.fabs_dtdz = fabs_dtdz;
  ra.zstep = zstep;
  ra.uvb = uvb;
  ra.recomb = recomb;
  ra.partials = c->d_partials;
  {
    Prof pr(c, "k_fhb_reduce", (2.0 + (uvb ? 1 : 0) + (recomb ? 3 : 0)) * B4N, s);
    launch_fhb_reduce(ra, gd, s);
  }
  launch_finalize(c->d_partials, 4, c->d_sums, s);
  const double* sums = readback(c, (const double*)c->d_sums, 4, s);
  const unsigned int* errw = readback(c, (const unsigned int*)c->d_err, 1, s);
  const double total = std::pow((double)gd.D, 3);
  if (out) {
    out->n_radii = nR;
    out->gpu_launches = kernel_launch_count() - launches0;
  }
  after(c, s, [c, s, sums, errw, out, total, uvb]() {
    if (*errw) {
      MX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), s));
      throw CudaError{ MX_ECUDA, "find_HII_bubbles: a transform pipeline wait timed out" };
    }
    if (out) {
      out->volume_weighted_global_xH = sums[0] / total;
      out->volume_weighted_global_J_21 = uvb ? sums[1] / total : 0.0;
      out->mass_weighted_global_xH = sums[2] / sums[3];
    }
  });
}

// ======================================================================
// ComputeTs (src/core/ComputeTs.c:78-1020)
// ======================================================================
static void fill_kappa(mx_ctx* c, TsDevConst* t)
{
  const NaturalSpline* sp[3] = { &c->ht.kap10, &c->ht.kap_e, &c->ht.kap_p };
  for (int w = 0; w < 3; w++) {
    t->nk[w] = (int)sp[w]->x.size();
    for (int i = 0; i < t->nk[w]; i++) {
      t->kx[w][i] = sp[w]->x[i];
      t->ky[w][i] = sp[w]->y[i];
      t->kc[w][i] = sp[w]->c[i];
    }
  }
}

static void fill_common_ts(mx_ctx* c, TsDevConst* t, double zp)
{
  const mx_params& p = c->p;
  t->zp = (float)zp;
  t->zpd = zp;
  t->n_b0 = c->d.n_b0;
  t->f_h = c->d.f_h;
  t->f_he = c->d.f_he;
  t->no = c->d.no;
  t->hubble_z = hubble(p, (float)zp);
  t->hubble0_h = k::HUBBLE * p.hubble_h;
  t->h = p.hubble_h;
  t->clumping = p.clumping_factor;
  for (int i = 0; i < 14; i++)
    t->xhii[i] = c->ht.xhii[i];
  fill_kappa(c, t);
  // FP32 constants of get_Ts (XRayHeatingFunctions.c:1513-1600, 1847-1882)
  const float zpf = (float)zp;
  const double opz = (double)(1.0f + zpf);
  const double Trad = k::TCMB * opz;
  const double p3 = std::pow(opz, 3.0);
  t->ftrad = (float)Trad;
  t->fxc[0] = (float)(k::T21 / Trad * c->d.no * p3 / k::A10);
  t->fxc[1] = (float)(k::T21 / Trad * c->d.n_b0 * p3 / k::A10);
  t->fxc[2] = t->fxc[0];
  t->ftgp = (float)(1.342881e-7 / t->hubble_z * c->d.no * p3);
  t->fxa = (float)(1.66e11 / opz);
  t->ff_he = (float)c->d.f_he;
  t->ftk_floor = (float)(k::TCMB * (1 + zp));
  for (int w = 0; w < 3; w++)
    for (int i = 0; i < t->nk[w]; i++) {
      t->fkx[w][i] = (float)t->kx[w][i];
      t->fky[w][i] = (float)t->ky[w][i];
      t->fkc[w][i] = (float)t->kc[w][i];
    }
}

// Power of two that brings |v| to [0.5, 1) (1 for v == 0).
static double pow2_scale(double v)
{
  if (!(v > 0.0) || !std::isfinite(v))
    return 1.0;
  int e;
  std::frexp(v, &e);
  return std::ldexp(1.0, -e);
}

// FP32 per-shell coefficients of evolveInt (see TsDevConst).
static void fill_fast_evolve(mx_ctx* c, TsDevConst* t, const ShellPlan& sp, const FreqTables& ft, double zp)
{
  const int S = t->S;
  const float zpf = (float)zp;
  const double opz = (double)(1.0f + zpf);
  const double U = (1.0 / t->pixel_volume) * t->sfr_a * t->sfr_b / k::SOLAR_MASS;
  const double Trad = k::TCMB * opz;
  for (int r = 0; r < S; r++) {
    const double base = U * sp.a_dt_dz[r] * sp.b_pow[r] * ft.const_zp_prefactor;
    double K[3] = { base * ft.dt_dzp * 2.0 / 3.0 / k::BOLTZMANN, base * ft.dt_dzp, base * c->d.n_b0 * t->p3 };
    for (int w = 0; w < 3; w++) {
      double m = 0.0;
      for (int x = 0; x < 14; x++)
        m = std::max(m, std::fabs(ft.tab[((size_t)w * 14 + x) * S + r]));
      const double sc = pow2_scale(m);
      for (int x = 0; x < 14; x++)
        t->ftab[w][x][r] = (float)(ft.tab[((size_t)w * 14 + x) * S + r] * sc);
      K[w] /= sc;
    }
    t->fKH[r] = (float)K[0];
    t->fKI[r] = (float)K[1];
    t->fKL[r] = (float)K[2];
    t->fKS[r] = (float)(U * t->p2 * sp.zpp1[r] * ft.sum_lyn[r] * sp.dt_dzpp[r] * sp.dzpp[r] * t->conv);
  }
  t->fksink = (float)(ft.dt_dzp * c->p.clumping_factor * c->d.f_h * c->d.n_b0 * t->p3);
  t->fadia0 = (float)(3 / (1.0 + zpf));
  t->fdgrowth = (float)ft.dgrowth_dzp;
  t->fgrowth = (float)ft.growth_zp;
  t->fccomp = (float)((-1.51e-4) / (t->hubble_z / (k::HUBBLE * c->p.hubble_h)) / c->p.hubble_h * std::pow(Trad, 4.0) /
                      (1.0 + zpf));
  t->fdzp = (float)t->dzp;
  const float* fl[] = { t->fKH, t->fKI, t->fKL, t->fKS };
  for (const float* q : fl)
    for (int r = 0; r < S; r++)
      if (!std::isfinite(q[r]) || (q[r] != 0.0f && std::fabs(q[r]) < 1e-30f))
        throw CudaError{ MX_ENOTSUP, "ComputeTs: coefficient outside the FP32 range" };
}

// Per-cell constants of the spin-temperature update (ComputeTs.c:666-724,
// XRayHeatingFunctions.c:1241-1435) into *t, which fill_common_ts has set up.
static void fill_ts_constants(mx_ctx* c, TsDevConst* t, const ShellPlan& sp, const FreqTables& ft, double zp,
                              double prev_z, double collapse_fraction, double pixel_volume)
{
  const mx_params& p = c->p;
  const int S = p.ts_num_filter_steps;
  const float zpf = (float)zp;
  t->S = S;
  t->no_light = (collapse_fraction > 0.0) ? 0 : 1;
  t->dzp = zp - prev_z;
  t->dt_dzp = ft.dt_dzp;
  t->growth = ft.growth_zp;
  t->dgrowth = ft.dgrowth_dzp;
  t->prefactor = ft.const_zp_prefactor;
  t->conv = (k::C / (4. * k::PI)) / (k::PROTONMASS / k::SOLAR_MASS);
  t->p2 = std::pow((double)(1.0f + zpf), 2);
  t->p3 = std::pow((double)(1.0f + zpf), 3);
  t->pixel_volume = pixel_volume;
  t->sfr_a = p.unit_mass_g / c->d.unit_time_s;
  t->sfr_b = std::pow(p.unit_length_cm, -3.);
  for (int q = 0; q < S; q++) {
    t->a[q] = sp.a_dt_dz[q];
    t->b[q] = sp.b_pow[q];
    t->zpp1[q] = sp.zpp1[q];
    t->sum_lyn[q] = ft.sum_lyn[q];
    t->dt_dzpp[q] = sp.dt_dzpp[q];
    t->dzpp[q] = sp.dzpp[q];
    for (int x = 0; x < 14; x++)
      for (int w = 0; w < 3; w++)
        t->tab[w][x][q] = ft.tab[((size_t)w * 14 + x) * S + q];
  }
  fill_fast_evolve(c, t, sp, ft, zp);
}

// ComputeTs inputs that a host-pointer call uploads on the copy stream while
// the compute stream works: `first` (stars, deltax, x_e_box_prev: the
// collapse fraction and <x_e>), `sfr`, each history slice (slices[j]), and
// `tk` (Tk_box, read by the per-cell update).  The compute stream waits for
// each right before its first use.  nullptr: every input is already there.
struct TsUploads
{
  cudaEvent_t first, sfr, tk;
  const std::vector<cudaEvent_t>* slices;
};

// Shells of ComputeTs (ComputeTs.c:276-503) into c->d_shells: apply the
// SFR-history operations to `sfr` (in place, like the reference), forward
// transform when the grid changed, then filter + inverse transform in
// batches of shells sharing a spectrum.
static void compute_shells(mx_ctx* c, const ShellPlan& sp, float* sfr, float* sfr_histories, cudaStream_t s,
                           const TsUploads* up = nullptr)
{
  if (up)
    MX_CUDA(cudaStreamWaitEvent(s, up->sfr, 0));
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const int S = p.ts_num_filter_steps;
  float2* sfr_unf = c->d_unf;
  const long long nhalf = gd.C;
  int r = 0;
  while (r < S) {
    for (const SfrOp& op : sp.ops[r]) {
      if (up && op.kind >= SfrOp::LOAD)
        MX_CUDA(cudaStreamWaitEvent(s, (*up->slices)[op.slice], 0));
      Prof pr(c, "k_sfr_history", op.kind <= SfrOp::ZERO_HALF ? 8.0 * (double)nhalf : 12.0 * (double)gd.N, s);
      if (op.kind == SfrOp::SCALE_HALF)
        launch_sfr_scale_half(sfr, nhalf, op.dweight, s);
      else if (op.kind == SfrOp::ZERO_HALF)
        launch_sfr_zero_half(sfr, nhalf, s);
      else
        launch_sfr_load(sfr, sfr_histories + (long long)op.slice * gd.P, op.weight,
                        op.kind == SfrOp::ADD, gd, s);
    }
    // shells r..r_end-1 share this spectrum (no operations in between)
    int r_end = r + 1;
    while (r_end < S && sp.ops[r_end].empty())
      r_end++;
    int q_first = r;
    if (r == 0) {
      // shell 0 is unfiltered: its transform pair is the identity, so the
      // shell is the clamped grid itself
      Prof pr(c, "k_shell_extract", 8.0 * (double)gd.N, s);
      launch_shell_extract(sfr, gd.P, 1, 0, c->d_shells, gd, s);
      q_first = 1;
    }
    if (q_first < r_end && c->fused_fft) {
      FwdArgs fa;
      for (int f = 0; f < MAX_FIELDS; f++)
        fa.src[f] = f == 0 ? sfr : nullptr;
      fa.G = 1;
      fa.out = sfr_unf;
      fa.C = c->unf_C;
      Prof pr(c, "fft_forward", 4.0 * (double)gd.N * (gd.D + 2) / gd.D + 40.0 * (double)c->unf_C, s);
      launch_fft_forward(gd.D, fa, c->y_threads, s);
    } else if (q_first < r_end) {
      MX_CUFFT(cufftSetStream(c->r2c_plan, s));
      Prof pr(c, "cufft_r2c", 4.0 * (double)gd.N + 8.0 * (double)gd.C, s);
      MX_CUFFT(cufftExecR2C(c->r2c_plan, (cufftReal*)sfr, (cufftComplex*)sfr_unf));
    }
    float2* in_ptr[1] = { sfr_unf };
    if (!c->fused_fft)
      upload(c, c->d_in_ptrs, in_ptr, sizeof(float2*), s);
    for (int q0 = q_first; q0 < r_end;) {
      const int nb = (int)std::min<long long>(std::min<long long>(c->work_fields, MAX_RADII), r_end - q0);
      if (c->fused_fft) {
        XPassArgs xa;
        for (int f = 0; f < MAX_FIELDS; f++)
          xa.in[f] = f == 0 ? sfr_unf : nullptr;
        xa.G = 1;
        xa.n = nb;
        xa.out = c->d_work;
        xa.C = c->work_C;
        for (int q = 0; q < nb; q++) {
          xa.R[q] = (float)sp.R[q0 + q];
          xa.apply[q] = 1;
        }
        xa.filter_type = p.ts_heating_filter_type;
        xa.delta_k = (float)(2.0 * k::PI / (float)p.box_size);
        xa.scale = (float)(1.0 / (double)gd.N);
        run_xy(c, xa, s);
        {
          Prof pr(c, "fft_z_store", (8.0 * (double)gd.C + 4.0 * (double)gd.N) * nb, s);
          launch_fft_z_store(gd.D, c->d_work, c->work_C, nb, q0, c->d_shells, gd.N, c->d_err, s);
        }
        q0 += nb;
        continue;
      }
      FilterBatch fb;
      fb.n = nb;
      fb.filter_type = p.ts_heating_filter_type;
      fb.scale_mode = 1;
      for (int q = 0; q < nb; q++) {
        fb.R[q] = (float)sp.R[q0 + q];
        fb.apply[q] = (q0 + q) > 0;
      }
      {
        Prof pr(c, "k_filter_ts", 8.0 * (double)gd.C * (1 + nb), s);
        launch_filter((const float2* const*)c->d_in_ptrs, 1, c->d_work, gd.C, fb, gd, (float)p.box_size, s);
      }
      const cufftHandle plan = c->c2r_plan(1);
      MX_CUFFT(cufftSetStream(plan, s));
      for (int q = 0; q < nb; q++) {
        cufftComplex* w = (cufftComplex*)(c->d_work + (long long)q * gd.C);
        Prof pr(c, "cufft_c2r", 8.0 * (double)gd.C + 4.0 * (double)gd.N, s);
        MX_CUFFT(cufftExecC2R(plan, w, (cufftReal*)w));
      }
      {
        Prof pr(c, "k_shell_extract", 8.0 * (double)gd.N * nb, s);
        launch_shell_extract((const float*)c->d_work, gd.P, nb, q0, c->d_shells, gd, s);
      }
      q0 += nb;
    }
    r = r_end;
  }
}

// ComputeTs's host work inside a captured step: a host node of the graph
// reads the collapse fraction and <x_e> (copied to pinned slots by the node
// before it), builds the frequency-integral tables and fills the evolve
// kernels' constants into the pinned h_tsc, which the next node uploads.
struct TsHostWork
{
  mx_ctx* c = nullptr;
  int snapshot = 0;
  ShellPlan sp;
  double zp = 0, prev_z = 0, pixel_volume = 0, total = 1;
  const double* cf = nullptr;  // pinned: sum of f_coll, sum of x_e
  std::string err;
};

static void CUDART_CB ts_tables_host(void* arg)
{
  TsHostWork* w = static_cast<TsHostWork*>(arg);
  mx_ctx* c = w->c;
  try {
    const double collapse_fraction = w->cf[0] / w->total, x_e_ave = w->cf[1] / w->total;
    c->stored_fcoll[w->snapshot] = collapse_fraction;
    FreqTables ft;
    build_freq_tables(c->p, c->d, c->ht, c->zz, c->stored_fcoll, w->snapshot, w->sp, x_e_ave, w->sp.weight_after,
                      c->nthreads, &ft);
    TsDevConst* t = c->h_tsc;
    std::memset(t, 0, sizeof(TsDevConst));
    fill_common_ts(c, t, w->zp);
    fill_ts_constants(c, t, w->sp, ft, w->zp, w->prev_z, collapse_fraction, w->pixel_volume);
  } catch (const CudaError& e) {
    w->err = e.msg;
  } catch (const std::exception& e) {
    w->err = e.what();
  }
}

static void run_ComputeTs(mx_ctx* c, int snapshot, const mx_grids* g, mx_globals* out, cudaStream_t s,
                          const TsUploads* up = nullptr)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const int launches0 = kernel_launch_count();
  if (!p.flag_spin_temp)
    throw CudaError{ MX_ESTATE, "ComputeTs: flag_spin_temp is off" };
  if (!g->deltax || !g->stars || !g->sfr || !g->x_e_box || !g->x_e_box_prev || !g->Tk_box || !g->TS_box ||
      (c->n_hist > 0 && !g->sfr_histories))
    throw CudaError{ MX_EINVAL, "ComputeTs: a required grid pointer is NULL" };
  const double box = p.box_size / p.hubble_h;
  const double pixel_volume = std::pow(box / (double)gd.D, 3);
  const double total = std::pow((double)gd.D, 3);
  const double zp = c->zz[snapshot];
  const double prev_z = snapshot == 0 ? c->zz[snapshot] : c->zz[snapshot - 1];
  const ShellPlan sp = plan_shells(p, c->zz, snapshot);
  const int S = p.ts_num_filter_steps;
  if (S > MAX_SHELLS)
    throw CudaError{ MX_ENOTSUP, "too many spin-temperature shells" };
  TsDevConst* t = c->h_tsc;
  std::memset(t, 0, sizeof(TsDevConst));
  fill_common_ts(c, t, zp);
  const double R0 = k::L_FACTOR * box / (float)gd.D;
  const double RtoM_h2 = RtoM(p, c->d, R0) * p.hubble_h * p.hubble_h;
  double collapse_fraction = 0.0, x_e_ave = 0.0;
  const double* homog_cf = nullptr;      // read back: sum of f_coll (homogeneous branch)
  const double* evolve_sums = nullptr;   // read back: J_alpha, xalpha, Xheat, Xion sums
  std::shared_ptr<TsHostWork> hw;        // host node of a captured step

  // host-pointer step, inhomogeneous: the shells start as soon as sfr has
  // landed, and the collapse fraction waits for its three grids on the side
  // stream (below)
  const bool early_shells = up && !sp.homogeneous && !c->capturing && c->early_shells;
  if (up && !early_shells) {
    MX_CUDA(cudaStreamWaitEvent(s, up->first, 0));
    if (sp.homogeneous) {
      MX_CUDA(cudaStreamWaitEvent(s, up->sfr, 0));
      MX_CUDA(cudaStreamWaitEvent(s, up->tk, 0));
    }
  }
  if (sp.homogeneous) {
    // ComputeTs.c:189-262
    upload(c, c->d_tsc, t, sizeof(TsDevConst), s);
    HomogArgs ha;
    ha.deltax = g->deltax;
    ha.stars = g->stars;
    ha.x_e_prev = g->x_e_box_prev;
    ha.Tk = g->Tk_box;
    ha.TS = g->TS_box;
    ha.xe0 = (float)(float)c->ht.xion_recfast((float)zp);
    ha.tk0 = (float)(float)c->ht.T_recfast((float)zp);
    ha.cst = c->d_tsc;
    ha.RtoM_h2 = RtoM_h2;
    ha.R3 = std::pow(R0, 3.0);
    ha.pixel_volume = pixel_volume;
    ha.partials = c->d_partials;
    ha.err = c->d_err;
    Prof pr(c, "k_homog", 5.0 * 4.0 * (double)gd.N, s);
    launch_homog(ha, gd, s);
    launch_finalize(c->d_partials, 1, c->d_sums, s);
    homog_cf = readback(c, (const double*)c->d_sums, 1, s);
  } else {
    // collapse fraction and <x_e> of the unsmoothed fields (ComputeTs.c:413-475)
    CfArgs ca;
    ca.stars = g->stars;
    ca.deltax = g->deltax;
    ca.x_e_prev = g->x_e_box_prev;
    ca.RtoM_h2 = RtoM_h2;
    ca.R3 = std::pow(R0, 3.0);
    ca.pixel_volume = pixel_volume;
    ca.partials = c->d_partials;
    if (early_shells) {
      // the shells first on s; the sums on the side stream after the grids
      // they read, copied to the host, where the tables wait for them
      cudaStream_t as = c->aux_stream;
      MX_CUDA(cudaStreamWaitEvent(as, up->first, 0));
      {
        Prof pr(c, "k_cf_xe", 3.0 * 4.0 * (double)gd.N, as);
        launch_cf_xe(ca, gd, as);
      }
      launch_finalize(c->d_partials, 2, c->d_sums, as);
      MX_CUDA(cudaMemcpyAsync(c->h_sums, c->d_sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, as));
      MX_CUDA(cudaEventRecord(c->ev_cf, as));
      compute_shells(c, sp, g->sfr, g->sfr_histories, s, up);
      MX_CUDA(cudaEventSynchronize(c->ev_cf));
      collapse_fraction = c->h_sums[0] / total;
      x_e_ave = c->h_sums[1] / total;
      c->stored_fcoll[snapshot] = collapse_fraction;
      FreqTables ft;
      build_freq_tables(p, c->d, c->ht, c->zz, c->stored_fcoll, snapshot, sp, x_e_ave, sp.weight_after, c->nthreads,
                        &ft);
      fill_ts_constants(c, t, sp, ft, zp, prev_z, collapse_fraction, pixel_volume);
      // the evolve kernel rewrites x_e_box_prev, which the side stream read
      MX_CUDA(cudaStreamWaitEvent(s, c->ev_cf, 0));
      MX_CUDA(cudaMemcpyAsync(c->d_tsc, t, sizeof(TsDevConst), cudaMemcpyHostToDevice, s));
    } else {
    {
      Prof pr(c, "k_cf_xe", 3.0 * 4.0 * (double)gd.N, s);
      launch_cf_xe(ca, gd, s);
    }
    launch_finalize(c->d_partials, 2, c->d_sums, s);
    if (c->capturing) {
      // a captured step: the tables are built by a host node on a side
      // branch of the graph while the shells are smoothed on s
      hw = std::make_shared<TsHostWork>();
      hw->c = c;
      hw->snapshot = snapshot;
      hw->sp = sp;
      hw->zp = zp;
      hw->prev_z = prev_z;
      hw->pixel_volume = pixel_volume;
      hw->total = total;
      cudaStream_t hs = c->copy_stream;
      MX_CUDA(cudaEventRecord(c->ev_a, s));
      MX_CUDA(cudaStreamWaitEvent(hs, c->ev_a, 0));
      hw->cf = readback(c, (const double*)c->d_sums, 2, hs);
      MX_CUDA(cudaLaunchHostFunc(hs, ts_tables_host, hw.get()));
      MX_CUDA(cudaMemcpyAsync(c->d_tsc, c->h_tsc, sizeof(TsDevConst), cudaMemcpyHostToDevice, hs));
      MX_CUDA(cudaEventRecord(c->ev_b, hs));
      c->graph_keep.push_back(hw);
      compute_shells(c, sp, g->sfr, g->sfr_histories, s, up);
      MX_CUDA(cudaStreamWaitEvent(s, c->ev_b, 0));
    } else {
      MX_CUDA(cudaMemcpyAsync(c->h_sums, c->d_sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
      MX_CUDA(cudaStreamSynchronize(s));
      collapse_fraction = c->h_sums[0] / total;
      x_e_ave = c->h_sums[1] / total;
      c->stored_fcoll[snapshot] = collapse_fraction;

      // X-ray frequency tables on host threads while the shells are smoothed
      FreqTables ft;
      std::vector<double> zz = c->zz;
      std::future<void> tables = std::async(std::launch::async, [&]() {
        build_freq_tables(p, c->d, c->ht, zz, c->stored_fcoll, snapshot, sp, x_e_ave, sp.weight_after, c->nthreads,
                          &ft);
      });

      // shells (ComputeTs.c:276-503): apply the SFR-history operations, forward
      // transform when the grid changed, then filter + inverse transform in
      // batches of shells sharing a spectrum.
      try {
        compute_shells(c, sp, g->sfr, g->sfr_histories, s, up);
      } catch (...) {
        tables.wait();
        throw;
      }
      tables.get();

      fill_ts_constants(c, t, sp, ft, zp, prev_z, collapse_fraction, pixel_volume);
      MX_CUDA(cudaMemcpyAsync(c->d_tsc, t, sizeof(TsDevConst), cudaMemcpyHostToDevice, s));
    }
    }
    EvolveArgs ea;
    ea.shells = c->d_shells;
    ea.deltax = g->deltax;
    ea.x_e_prev = g->x_e_box_prev;
    ea.Tk = g->Tk_box;
    ea.TS = g->TS_box;
    ea.cst = c->d_tsc;
    ea.partials = c->d_partials;
    ea.err = c->d_err;
    ea.n_shells = S;
    if (up)
      MX_CUDA(cudaStreamWaitEvent(s, up->tk, 0));
    int ev_blocks = RED_BLOCKS;
    {
      Prof pr(c, "k_evolve", ((double)S + 6.0) * 4.0 * (double)gd.N, s);
      ev_blocks = launch_evolve(ea, gd, c->has_shell_map ? &c->shell_map : nullptr, s);
    }
    launch_finalize(c->d_partials, 4, c->d_sums + 8, s, ev_blocks);
    evolve_sums = readback(c, (const double*)(c->d_sums + 8), 4, s);
  }

  // x_e_box <- x_e_box_prev (ComputeTs.c:940) and the means (:942-974)
  {
    Prof pr(c, "copy_x_e_box", 8.0 * (double)gd.P, s);
    MX_CUDA(cudaMemcpyAsync(g->x_e_box, g->x_e_box_prev, sizeof(float) * gd.P, cudaMemcpyDeviceToDevice, s));
  }
  {
    Prof pr(c, "k_ts_means", 8.0 * (double)gd.N, s);
    launch_ts_means(g->TS_box, g->Tk_box, c->d_partials, gd, s);
  }
  launch_finalize(c->d_partials, 2, c->d_sums, s);
  const double* means = readback(c, (const double*)c->d_sums, 2, s);
  // the reference's <x_e> reads the last cell's x_e_box_prev (ComputeTs.c:957)
  const long long last_pad = (long long)(gd.D - 1) + 2LL * gd.H * ((long long)(gd.D - 1) + (long long)gd.D * (gd.D - 1));
  const float* xe_last = readback(c, (const float*)(g->x_e_box_prev + last_pad), 1, s);
  const unsigned int* errw = readback(c, (const unsigned int*)c->d_err, 1, s);
  if (out)
    out->gpu_launches = kernel_launch_count() - launches0;
  const bool homog = sp.homogeneous;
  after(c, s, [=]() {
    if (*errw) {
      MX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), s));
      throw CudaError{ MX_ECUDA, (*errw & 2u) ? "ComputeTs: a pipeline wait (transform or shell copies) timed out"
                                              : "ComputeTs: spin-temperature iteration did not converge" };
    }
    if (hw && !hw->err.empty())
      throw CudaError{ MX_ETABLE, "ComputeTs tables: " + hw->err };
    double cf = collapse_fraction, xe = x_e_ave;
    if (homog_cf)
      cf = homog_cf[0] / total;
    if (hw) {
      cf = hw->cf[0] / total;
      xe = hw->cf[1] / total;
    }
    if (out) {
      if (!homog) {
        out->volume_ave_J_alpha = evolve_sums[0] / total;
        out->volume_ave_xalpha = evolve_sums[1] / total;
        out->volume_ave_Xheat = evolve_sums[2] / total;
        out->volume_ave_Xion = evolve_sums[3] / total;
      }
      out->volume_ave_TS = means[0] / total;
      out->volume_ave_TK = means[1] / total;
      out->volume_ave_xe = (double)xe_last[0];
      out->x_e_ave = xe;
      out->collapse_fraction = cf;
    }
  });
}

// ======================================================================
// ComputeBrightnessTemperatureBox (src/core/BrightnessTemperature.c:24-549)
// ======================================================================
// Peculiar-velocity corrections (BrightnessTemperature.c:158-509), after
// the base delta_T; vel is converted in place like the reference does.
static void run_pecvel(mx_ctx* c, const mx_grids* g, float redshift, cudaStream_t s)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const float H_z = (float)(float)hubble(p, redshift);
  {
    Prof pr(c, "k_vel_convert", 8.0 * (double)gd.N, s);
    launch_vel_convert(g->vel, p.trees_id, redshift, gd, s);
  }
  float2* spec = c->d_unf;  // slot 0: spectrum, then dv/dx in place
  {
    MX_CUFFT(cufftSetStream(c->r2c_plan, s));
    Prof pr(c, "cufft_r2c", 4.0 * (double)gd.N + 8.0 * (double)gd.C, s);
    MX_CUFFT(cufftExecR2C(c->r2c_plan, (cufftReal*)g->vel, (cufftComplex*)spec));
  }
  {
    // velocity_gradient (reionization.c:2172-2187): k from BoxSize in Mpc/h
    const float box_f = (float)p.box_size;
    const float dk = (float)(2.0 * k::PI / box_f);
    Prof pr(c, "k_vel_grad_k", 16.0 * (double)gd.C, s);
    launch_vel_grad_k(spec, gd, p.hubble_h, dk, s);
  }
  {
    const cufftHandle plan = c->c2r_plan(1);
    MX_CUFFT(cufftSetStream(plan, s));
    Prof pr(c, "cufft_c2r", 8.0 * (double)gd.C + 4.0 * (double)gd.N, s);
    MX_CUFFT(cufftExecC2R(plan, (cufftComplex*)spec, (cufftReal*)spec));
  }
  PecvelArgs pa;
  pa.grad = reinterpret_cast<const float*>(spec);
  pa.delta_T = g->delta_T;
  pa.TS = g->TS_box;
  pa.mode = p.flag_pecvel;
  pa.H_z = H_z;
  pa.redshift = redshift;
  pa.max_v_deriv = std::fabs((double)(0.2f * H_z));  // fabs(MAX_DVDR * H_z), MAX_DVDR = (float)0.2
  pa.T_rad = k::TCMB * (1. + redshift);
  {
    Prof pr(c, "k_pecvel_cells", (p.flag_pecvel > 1 ? 16.0 : 12.0) * (double)gd.N, s);
    launch_pecvel_cells(pa, gd, s);
  }
  if (p.flag_pecvel == 3) {
    RsdArgs ra;
    ra.vel = g->vel;
    ra.delta_T = g->delta_T;
    ra.xH = g->xH;
    ra.los = reinterpret_cast<float*>(c->d_unf + gd.C);  // slot 1 as REAL scratch
    ra.delta_T_out = g->delta_T;
    ra.box = p.box_size / p.hubble_h;
    ra.subcell_width = (ra.box / ((double)gd.D)) / (double)RSD_STEPS;
    for (int i = 0; i < RSD_STEPS; i++) {
      ra.x_pos_offset[i] = (float)(ra.subcell_width * (float)i + ra.subcell_width / 2.);
      ra.x_pos[i] = (float)(ra.x_pos_offset[i] / (ra.box / (float)gd.D));
    }
    ra.H_z = H_z;
    Prof pr(c, "k_rsd_columns", 20.0 * (double)gd.N, s);
    launch_rsd(ra, gd, s);
  }
}

static void run_delta_T(mx_ctx* c, int snapshot, const mx_grids* g, mx_globals* out, cudaStream_t s)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const int launches0 = kernel_launch_count();
  const bool pecvel = p.flag_spin_temp && p.flag_pecvel > 0;
  if (p.flag_pecvel < 0 || p.flag_pecvel > 3)
    throw CudaError{ MX_EINVAL, "Flag_IncludePecVelsFor21cm must be 0-3" };
  if (!g->deltax || !g->xH || !g->delta_T || (p.flag_spin_temp && !g->TS_box) || (pecvel && !g->vel))
    throw CudaError{ MX_EINVAL, "ComputeBrightnessTemperatureBox: a required grid pointer is NULL" };
  const float redshift = (float)(float)c->zz[snapshot];
  const float Hubble_h = (float)(float)p.hubble_h;
  const float OmegaM = (float)(float)p.omega_m;
  const float OmegaB = (float)(OmegaM * p.baryon_frac);
  DeltaTArgs a;
  a.const_factor = (float)(27.0 * (OmegaB * Hubble_h * Hubble_h / 0.023) *
                           std::sqrt((0.15 / OmegaM / Hubble_h / Hubble_h) * (1.0 + redshift) / 10.0));
  a.T_rad_f = (float)(k::TCMB * (1. + redshift));
  a.redshift = redshift;
  a.deltax = g->deltax;
  a.xH = g->xH;
  a.TS = g->TS_box;
  a.delta_T = g->delta_T;
  a.spin = p.flag_spin_temp;
  a.pecvel = p.flag_pecvel;
  a.partials = c->d_partials;
  {
    Prof pr(c, "k_delta_T", (p.flag_spin_temp ? 4.0 : 3.0) * 4.0 * (double)gd.N, s);
    launch_delta_T(a, gd, s);
  }
  if (pecvel) {
    run_pecvel(c, g, redshift, s);
    Prof pr(c, "k_ps_mean", 4.0 * (double)gd.N, s);
    launch_ps_mean(g->delta_T, gd.N, c->d_ps_partials, c->d_sums, s);
  } else {
    launch_finalize(c->d_partials, 1, c->d_sums, s);
  }
  const double* sum = readback(c, (const double*)c->d_sums, 1, s);
  if (out)
    out->gpu_launches = kernel_launch_count() - launches0;
  const double total = std::pow((double)gd.D, 3);
  after(c, s, [sum, out, total]() {
    if (out)
      out->volume_ave_Tb = sum[0] / total;
  });
}

// ======================================================================
// 21 cm power spectrum (src/core/ComputePowerSpectrum.c:18-255)
// ======================================================================
// Bin ceilings of Initialise_PowerSpectrum / Compute_PS (:22-40, :133-141):
// edges[0] = 0, edges[b + 1] = delta_k * 1.35^b by the reference's float
// recurrence while below delta_k * D.  Returns the number of bins.
static int ps_edges(const mx_params& p, float* edges, int cap, float* delta_k_out, float* volume_out)
{
  const double box_size = p.box_size / p.hubble_h;  // Mpc
  const float k_factor = 1.35f;
  const float delta_k = (float)(2. * k::PI / box_size);
  const float k_max = delta_k * p.grid_dim;
  float k_ceil = delta_k;
  int n = 0;
  edges[0] = 0.0f;
  while (k_ceil < k_max) {
    if (n + 1 > cap)
      throw CudaError{ MX_ENOTSUP, "too many power-spectrum bins" };
    edges[n + 1] = k_ceil;
    n++;
    k_ceil *= k_factor;
  }
  *delta_k_out = delta_k;
  *volume_out = std::pow((float)box_size, 3.0f);
  return n;
}

static int run_power_spectrum(mx_ctx* c, const float* dT, float* ps_k, float* ps_data, float* ps_error, int cap,
                              cudaStream_t s)
{
  const GridDims& gd = c->gd;
  PsArgs a;
  a.nb = ps_edges(c->p, a.edges, PS_MAX_BINS, &a.delta_k, &a.volume);
  if (a.nb > cap)
    throw CudaError{ MX_EINVAL, "output arrays shorter than the number of power-spectrum bins" };
  float* field = reinterpret_cast<float*>(c->d_work);  // padded real scratch (one spectrum's bytes)
  double* mean_sum = c->d_ps_sums + 3 * PS_MAX_BINS;
  {
    Prof pr(c, "k_ps_mean", 4.0 * (double)gd.N, s);
    launch_ps_mean(dT, gd.N, c->d_ps_partials, mean_sum, s);
  }
  {
    Prof pr(c, "k_ps_field", 8.0 * (double)gd.N, s);
    launch_ps_field(dT, mean_sum, a.volume, gd, field, s);
  }
  {
    MX_CUFFT(cufftSetStream(c->r2c_plan, s));
    Prof pr(c, "cufft_r2c", 4.0 * (double)gd.N + 8.0 * (double)gd.C, s);
    MX_CUFFT(cufftExecR2C(c->r2c_plan, (cufftReal*)field, (cufftComplex*)c->d_unf));
  }
  a.spec = c->d_unf;
  a.D = gd.D;
  a.partials = c->d_ps_partials;
  {
    Prof pr(c, "k_ps_bin", 8.0 * (double)gd.C, s);
    launch_ps_bin(a, c->d_ps_sums, s);
  }
  MX_CUDA(cudaMemcpyAsync(c->h_ps_sums, c->d_ps_sums, sizeof(double) * 3 * a.nb, cudaMemcpyDeviceToHost, s));
  MX_CUDA(cudaStreamSynchronize(s));
  // :228-240
  for (int i = 0; i < a.nb; i++) {
    const double p_box = c->h_ps_sums[i], k_ave = c->h_ps_sums[a.nb + i], ct = c->h_ps_sums[2 * a.nb + i];
    ps_k[i] = (float)(k_ave / ct);
    ps_data[i] = (float)(p_box / ct);
    ps_error[i] = (float)((p_box / ct) / std::sqrt(ct));
  }
  return a.nb;
}

// ======================================================================
// Power-spectrum loss and the adjoint of ComputeTs + the 21cm box
// ======================================================================
// L = sum_b (P_b - T_b)^2 over nbins bins [edges[b], edges[b+1]) of the
// power spectrum of f = delta_T V / N, P_b = sum k^3 |X_k|^2 / (2 pi^2 V) / n_b
// over the half-spectrum modes of the bin (each counted once, k and V in Mpc
// units, the binning of Compute_PS).  With grad: dL/d(delta_T) (REAL).
static double run_ps_loss(mx_ctx* c, const float* dT, int nbins, const float* edges, const float* target, float* P,
                          float* grad, cudaStream_t s)
{
  const GridDims& gd = c->gd;
  if (nbins < 1 || nbins + 1 > PS_MAX_BINS)
    throw CudaError{ MX_EINVAL, "power-spectrum loss: 1 to 47 bins" };
  PsArgs a;
  float e0[PS_MAX_BINS + 1];
  float dk = 0, vol = 0;
  ps_edges(c->p, e0, PS_MAX_BINS, &dk, &vol);
  a.delta_k = dk;
  a.volume = vol;
  // bin 0 collects the modes below edges[0] and is not part of the loss
  a.nb = nbins + 1;
  a.edges[0] = 0.0f;
  for (int b = 0; b <= nbins; b++) {
    if (!(edges[b] > (b ? edges[b - 1] : 0.0f)))
      throw CudaError{ MX_EINVAL, "power-spectrum loss: edges must be positive and increasing" };
    a.edges[b + 1] = edges[b];
  }
  a.D = gd.D;
  a.partials = c->d_ps_partials;
  float* field = reinterpret_cast<float*>(c->d_work);
  const float scale = (float)((double)vol / (double)gd.N);
  {
    Prof pr(c, "k_ps_scale", 8.0 * (double)gd.N, s);
    launch_ps_scale(dT, scale, gd, field, s);
  }
  MX_CUFFT(cufftSetStream(c->r2c_plan, s));
  MX_CUFFT(cufftExecR2C(c->r2c_plan, (cufftReal*)field, (cufftComplex*)c->d_unf));
  a.spec = c->d_unf;
  {
    Prof pr(c, "k_ps_bin", 8.0 * (double)gd.C, s);
    launch_ps_bin(a, c->d_ps_sums, s);
  }
  MX_CUDA(cudaMemcpyAsync(c->h_ps_sums, c->d_ps_sums, sizeof(double) * 3 * a.nb, cudaMemcpyDeviceToHost, s));
  MX_CUDA(cudaStreamSynchronize(s));
  const double pdiv = 2.0 * k::PI * k::PI * (double)vol;
  double loss = 0.0;
  double coef[PS_MAX_BINS] = { 0 };
  for (int b = 0; b < nbins; b++) {
    const double sum = c->h_ps_sums[b + 1], ct = c->h_ps_sums[2 * a.nb + b + 1];
    const double pb = ct > 0 ? sum / ct : 0.0;
    if (P)
      P[b] = (float)pb;
    const double d = pb - (double)target[b];
    loss += d * d;
    // dL/dRe X_k = 2 c_k Re X_k (and Im) with c_k = 2 (P_b - T_b) k^3 / (pdiv n_b);
    // k_ps_loss_grad multiplies by k^3
    coef[b + 1] = ct > 0 ? 2.0 * d / (pdiv * ct) : 0.0;
  }
  if (grad) {
    // dL/df = C2R(Y) with Y = coef' k^3 X (see k_ps_loss_grad); dL/d(delta_T) = scale dL/df
    MX_CUDA(cudaMemcpyAsync(c->d_adj_coef, coef, sizeof(double) * a.nb, cudaMemcpyHostToDevice, s));
    float2* spec = reinterpret_cast<float2*>(c->d_work);
    MX_CUDA(cudaMemcpyAsync(spec, c->d_unf, sizeof(float2) * gd.C, cudaMemcpyDeviceToDevice, s));
    {
      Prof pr(c, "k_ps_loss_grad", 16.0 * (double)gd.C, s);
      launch_ps_loss_grad(a, c->d_adj_coef, spec, s);
    }
    const cufftHandle plan = c->c2r_plan(1);
    MX_CUFFT(cufftSetStream(plan, s));
    MX_CUFFT(cufftExecC2R(plan, (cufftComplex*)spec, (cufftReal*)spec));
    launch_padded_to_real(reinterpret_cast<const float*>(spec), scale, gd, grad, s);
  }
  return loss;
}

static void ensure_adjoint_scratch(mx_ctx* c)
{
  if (c->d_adj_sfr)
    return;
  const GridDims& gd = c->gd;
  MX_CUDA(cudaMalloc(&c->d_adj_sfr, sizeof(float) * gd.P));
  MX_CUDA(cudaMalloc(&c->d_adj_dp, sizeof(float4) * 14 * MAX_SHELLS));
  MX_CUDA(cudaMalloc(&c->d_adj_coef, sizeof(double) * PS_MAX_BINS));
  int n[3] = { gd.D, gd.D, gd.D };
  int inembed[3] = { gd.D, gd.D, gd.D };
  int onembed[3] = { gd.D, gd.D, gd.H };
  MX_CUFFT(cufftPlanMany(&c->r2c_real_plan, 3, n, inembed, 1, (int)gd.N, onembed, 1, (int)gd.C, CUFFT_R2C, 1));
}

// (K_H tab_H, K_I tab_I, K_L tab_L) of every (x_HII node, shell) in double:
// the per-cell sums of the FP32 evolve without the power-of-two rescaling.
static std::vector<double> shell_products(mx_ctx* c, const TsDevConst* t, const ShellPlan& sp, const FreqTables& ft)
{
  const int S = t->S;
  const double U = (1.0 / t->pixel_volume) * t->sfr_a * t->sfr_b / k::SOLAR_MASS;
  std::vector<double> out((size_t)3 * 14 * S);
  for (int r = 0; r < S; r++) {
    const double base = U * sp.a_dt_dz[r] * sp.b_pow[r] * ft.const_zp_prefactor;
    const double K[3] = { base * ft.dt_dzp * 2.0 / 3.0 / k::BOLTZMANN, base * ft.dt_dzp, base * c->d.n_b0 * t->p3 };
    for (int w = 0; w < 3; w++)
      for (int x = 0; x < 14; x++)
        out[((size_t)w * 14 + x) * S + r] = K[w] * ft.tab[((size_t)w * 14 + x) * S + r];
  }
  return out;
}

// Adjoint of ComputeTs (one snapshot, not homogeneous) and of the 21cm box
// without peculiar velocities, with the ionisation flags of find_HII_bubbles
// held fixed.  `g` holds the forward's inputs and outputs: deltax, stars (as
// find_HII_bubbles read them), sfr (before ComputeTs reweighted it),
// sfr_histories, x_e_box_prev and Tk_box (the state before the step), x_e_box,
// xH and TS_box (after it).  The shells are recomputed.  Out: dL/d(sfr)
// (PADDED), dL/d(stars) (PADDED), grad_params = {dL/dL_X, dL/dE0}.
static void run_adjoint(mx_ctx* c, int snapshot, const mx_grids* g, const float* grad_dT, float* grad_sfr,
                        float* grad_stars, double* grad_params, cudaStream_t s)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  if (!p.flag_spin_temp)
    throw CudaError{ MX_ENOTSUP, "adjoint: needs the spin temperature" };
  if (p.flag_pecvel != 0)
    throw CudaError{ MX_ENOTSUP, "adjoint: peculiar-velocity modes are not differentiated" };
  if (!g || !g->deltax || !g->stars || !g->sfr || !g->x_e_box_prev || !g->Tk_box || !g->x_e_box || !g->xH ||
      !g->TS_box || (c->n_hist > 0 && !g->sfr_histories) || !grad_dT || !grad_sfr || !grad_stars || !grad_params)
    throw CudaError{ MX_EINVAL, "adjoint: a required pointer is NULL" };
  ensure_adjoint_scratch(c);
  const double box = p.box_size / p.hubble_h;
  const double pixel_volume = std::pow(box / (double)gd.D, 3);
  const double total = std::pow((double)gd.D, 3);
  const double zp = c->zz[snapshot];
  const double prev_z = snapshot == 0 ? c->zz[snapshot] : c->zz[snapshot - 1];
  const ShellPlan sp = plan_shells(p, c->zz, snapshot);
  const int S = p.ts_num_filter_steps;
  if (S > MAX_SHELLS)
    throw CudaError{ MX_ENOTSUP, "too many spin-temperature shells" };
  if (sp.homogeneous)
    throw CudaError{ MX_ENOTSUP, "adjoint: the homogeneous branch has no SFR dependence" };
  TsDevConst* t = c->h_tsc;
  std::memset(t, 0, sizeof(TsDevConst));
  fill_common_ts(c, t, zp);
  const double R0 = k::L_FACTOR * box / (float)gd.D;
  const double RtoM_h2 = RtoM(p, c->d, R0) * p.hubble_h * p.hubble_h;
  // collapse fraction and <x_e> of the state before the step (as the forward)
  CfArgs ca;
  ca.stars = g->stars;
  ca.deltax = g->deltax;
  ca.x_e_prev = g->x_e_box_prev;
  ca.RtoM_h2 = RtoM_h2;
  ca.R3 = std::pow(R0, 3.0);
  ca.pixel_volume = pixel_volume;
  ca.partials = c->d_partials;
  launch_cf_xe(ca, gd, s);
  launch_finalize(c->d_partials, 2, c->d_sums, s);
  MX_CUDA(cudaMemcpyAsync(c->h_sums, c->d_sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
  MX_CUDA(cudaStreamSynchronize(s));
  const double collapse_fraction = c->h_sums[0] / total;
  const double x_e_ave = c->h_sums[1] / total;
  c->stored_fcoll[snapshot] = collapse_fraction;
  // frequency tables at E0 and E0 (1 +- h) for d/dE0, on host threads while
  // the shells are recomputed
  const double h = 1e-3;
  FreqTables ft, ftp, ftm;
  mx_params pp = p, pm = p;
  pp.nu_xray_gal_threshold = p.nu_xray_gal_threshold * (1 + h);
  pm.nu_xray_gal_threshold = p.nu_xray_gal_threshold * (1 - h);
  const int nt = std::max(1, c->nthreads / 3);
  auto build = [&](const mx_params& q, FreqTables* out) {
    return std::async(std::launch::async, [&, out]() {
      build_freq_tables(q, c->d, c->ht, c->zz, c->stored_fcoll, snapshot, sp, x_e_ave, sp.weight_after, nt, out);
    });
  };
  std::future<void> tables[3] = { build(p, &ft), build(pp, &ftp), build(pm, &ftm) };
  try {
    // shells of the forward, from a copy of the SFR grid
    MX_CUDA(cudaMemcpyAsync(c->d_adj_sfr, g->sfr, sizeof(float) * gd.P, cudaMemcpyDeviceToDevice, s));
    compute_shells(c, sp, c->d_adj_sfr, g->sfr_histories, s);
  } catch (...) {
    for (auto& f : tables)
      f.wait();
    throw;
  }
  for (auto& f : tables)
    f.get();
  fill_ts_constants(c, t, sp, ft, zp, prev_z, collapse_fraction, pixel_volume);
  MX_CUDA(cudaMemcpyAsync(c->d_tsc, t, sizeof(TsDevConst), cudaMemcpyHostToDevice, s));
  {
    const std::vector<double> P1 = shell_products(c, t, sp, ftp), P0 = shell_products(c, t, sp, ftm);
    std::vector<float4> dp((size_t)14 * S);
    const double dE = 2 * h * p.nu_xray_gal_threshold;
    for (int x = 0; x < 14; x++)
      for (int r = 0; r < S; r++) {
        float v[3];
        for (int w = 0; w < 3; w++) {
          const size_t i = ((size_t)w * 14 + x) * S + r;
          v[w] = (float)((P1[i] - P0[i]) / dE);
        }
        dp[(size_t)x * S + r] = make_float4(v[0], v[1], v[2], 0.0f);
      }
    MX_CUDA(cudaMemcpyAsync(c->d_adj_dp, dp.data(), sizeof(float4) * dp.size(), cudaMemcpyHostToDevice, s));
    MX_CUDA(cudaStreamSynchronize(s));  // dp leaves scope
  }
  // the 21cm box constants (run_delta_T)
  const float redshift = (float)(float)zp;
  const float Hubble_h = (float)(float)p.hubble_h;
  const float OmegaM = (float)(float)p.omega_m;
  const float OmegaB = (float)(OmegaM * p.baryon_frac);
  const std::vector<double> radii = filter_radii(p);
  const double R_last = radii.back();
  const double pv_fhb = std::pow(p.box_size / (double)gd.D, 3);
  AdjointArgs a;
  a.shells = c->d_shells;
  a.deltax = g->deltax;
  a.x_e_prev = g->x_e_box_prev;
  a.Tk = g->Tk_box;
  a.x_e_new = g->x_e_box;
  a.stars = g->stars;
  a.xH = g->xH;
  a.TS = g->TS_box;
  a.grad_dT = grad_dT;
  a.grad_stars = grad_stars;
  a.cst = c->d_tsc;
  a.dP_dE0 = c->d_adj_dp;
  a.dT_factor = (float)(27.0 * (OmegaB * Hubble_h * Hubble_h / 0.023) *
                        std::sqrt((0.15 / OmegaM / Hubble_h / Hubble_h) * (1.0 + redshift) / 10.0));
  a.dT_trad = (float)(k::TCMB * (1. + redshift));
  a.kfc_last = (float)(p.reion_efficiency * (4.0 / 3.0) * k::PI * R_last * R_last * R_last /
                       (RtoM(p, c->d, R_last) * pv_fhb));
  a.partials = c->d_partials;
  a.err = c->d_err;
  a.n_shells = S;
  MX_CUDA(cudaMemsetAsync(grad_stars, 0, sizeof(float) * gd.P, s));
  {
    Prof pr(c, "k_evolve_adjoint", ((double)S * 2 + 10.0) * 4.0 * (double)gd.N, s);
    launch_evolve_adjoint(a, gd, c->has_shell_map ? &c->shell_map : nullptr, s);
  }
  launch_finalize(c->d_partials, 2, c->d_sums, s);
  // dL/d(shell) -> dL/d(sfr): each group of shells sharing a spectrum is a sum
  // of symmetric filter convolutions of the group's SFR field, which is
  // alpha * sfr (+ history terms) with one alpha per half of the padded array
  MX_CUDA(cudaMemsetAsync(grad_sfr, 0, sizeof(float) * gd.P, s));
  float2* acc = c->d_work;
  float2* U = c->d_work + c->work_C;
  double alpha[2] = { 1.0, 1.0 };
  const float delta_k = (float)(2.0 * k::PI / (float)p.box_size);
  const float scale = (float)(1.0 / (double)gd.N);
  int r = 0;
  while (r < S) {
    for (const SfrOp& op : sp.ops[r]) {
      if (op.kind == SfrOp::SCALE_HALF)
        alpha[0] *= op.dweight;
      else if (op.kind == SfrOp::ZERO_HALF)
        alpha[0] = 0.0;
      else if (op.kind == SfrOp::LOAD)
        alpha[0] = alpha[1] = 0.0;
    }
    int r_end = r + 1;
    while (r_end < S && sp.ops[r_end].empty())
      r_end++;
    const bool has0 = r == 0;
    bool first = true;
    for (int q = has0 ? 1 : r; q < r_end; q++) {
      MX_CUFFT(cufftSetStream(c->r2c_real_plan, s));
      MX_CUFFT(cufftExecR2C(c->r2c_real_plan, (cufftReal*)(c->d_shells + (long long)q * gd.N), (cufftComplex*)U));
      launch_filter_accumulate(gd.D, acc, U, (float)sp.R[q], p.ts_heating_filter_type, delta_k, scale, first, s);
      first = false;
    }
    if (!first) {
      const cufftHandle plan = c->c2r_plan(1);
      MX_CUFFT(cufftSetStream(plan, s));
      MX_CUFFT(cufftExecC2R(plan, (cufftComplex*)acc, (cufftReal*)acc));
    }
    if (alpha[0] != 0.0 || alpha[1] != 0.0)
      launch_adjoint_axpy(grad_sfr, first ? nullptr : reinterpret_cast<const float*>(acc),
                          has0 ? c->d_shells : nullptr, (float)alpha[0], (float)alpha[1], gd, s);
    r = r_end;
  }
  double sums[2];
  MX_CUDA(cudaMemcpyAsync(sums, c->d_sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
  unsigned int errw = 0;
  MX_CUDA(cudaMemcpyAsync(&errw, c->d_err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
  MX_CUDA(cudaStreamSynchronize(s));
  if (errw) {
    MX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), s));
    throw CudaError{ MX_ECUDA, "adjoint: a pipeline wait timed out" };
  }
  grad_params[0] = sums[0] / p.lx_gal;
  grad_params[1] = sums[1];
}

// ======================================================================
// Light cone (src/core/ConstructLightcone.c:12-166)
// ======================================================================
// Redshifts of the slices ConstructLightcone fills at `snapshot` (the
// reference's walk from the light cone's low-redshift end in steps of one
// comoving cell, dR / drdz, keeping those in [ZZ[snapshot], ZZ[snapshot-1])).
static std::vector<double> lc_slices(const mx_ctx* c, int snapshot)
{
  const mx_params& p = c->p;
  const double box_size = p.box_size / p.hubble_h;
  const double dR = (box_size / (double)p.grid_dim) * k::MPC;
  const double z2 = c->zz[snapshot - 1];
  double z_LC = c->zz[c->lc_end_snapshot];
  std::vector<double> zs;
  while (z_LC < z2) {
    if (z_LC >= c->zz[snapshot] && z_LC < c->zz[snapshot - 1])
      zs.push_back(z_LC);
    z_LC -= dR / drdz(p, (float)z_LC);
  }
  return zs;
}

// Initialise_ConstructLightcone (:12-67)
static long long lightcone_init(mx_ctx* c, double end_redshift, int last_output_snap)
{
  const mx_params& p = c->p;
  if (c->zz.empty())
    throw CudaError{ MX_ESTATE, "mx_set_redshifts has not been called" };
  if (last_output_snap < 0 || last_output_snap >= (int)c->zz.size())
    throw CudaError{ MX_EINVAL, "last output snapshot out of range" };
  const double box_size = p.box_size / p.hubble_h;
  const double dR = (box_size / (double)p.grid_dim) * k::MPC;
  const double start_redshift = c->zz[0];
  int i = 0;
  while (i < (int)c->zz.size() - 1 && c->zz[i] > end_redshift)
    i++;
  int closest = std::min(i, last_output_snap);
  double z1 = c->zz[closest], z_LC = z1;
  long long total = 0;
  i = 0;
  while (z1 < start_redshift) {
    const double z2 = c->zz[closest - 1 - i];
    while (z_LC < z2) {
      total++;
      z_LC -= dR / drdz(p, (float)z_LC);
    }
    z1 = z2;
    i += 1;
  }
  c->lc_length = total;
  c->lc_end_snapshot = closest;
  c->lc_pos = total;
  long long mx = 0;
  for (int s = 1; s <= closest; s++)
    mx = std::max<long long>(mx, (long long)lc_slices(c, s).size());
  cudaFree(c->d_lc_times);
  cudaFree(c->d_lc_scratch);
  c->d_lc_times = nullptr;
  c->d_lc_scratch = nullptr;
  c->lc_max_slices = mx;
  if (mx > 0) {
    MX_CUDA(cudaMalloc(&c->d_lc_times, sizeof(double) * mx));
    MX_CUDA(cudaMalloc(&c->d_lc_scratch, sizeof(float) * (size_t)c->gd.D * c->gd.D * (size_t)mx));
  }
  return total;
}

// ConstructLightcone (:69-166).  Device pointers; `out` is either the
// caller's device light cone (pitch = length, written at the slice offset)
// or the scratch (pitch = slices of this snapshot) when host_lc is given.
static void construct_lightcone(mx_ctx* c, int snapshot, const float* dT, const float* dT_prev, float* dev_lc,
                                float* host_lc, float* lc_z, cudaStream_t s)
{
  const GridDims& gd = c->gd;
  if (c->lc_length < 0)
    throw CudaError{ MX_ESTATE, "mx_lightcone_init has not been called" };
  if (snapshot == 0) {
    c->lc_pos = c->lc_length;
    return;
  }
  const std::vector<double> zs = lc_slices(c, snapshot);
  const long long n = (long long)zs.size();
  c->lc_pos -= n;
  if (n == 0)
    return;
  if (c->lc_pos < 0 || n > c->lc_max_slices)
    throw CudaError{ MX_ESTATE, "light-cone snapshots called out of order" };
  const long long slice0 = c->lc_pos;
  std::vector<double> t(n);
  for (long long i = 0; i < n; i++) {
    t[i] = gettime(c->p, zs[i]);
    lc_z[slice0 + i] = (float)zs[i];
  }
  MX_CUDA(cudaMemcpyAsync(c->d_lc_times, t.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  LightconeArgs a;
  a.delta_T = dT;
  a.delta_T_prev = dT_prev;
  a.t_slice = c->d_lc_times;
  a.n = (int)n;
  a.iz0 = (int)(slice0 % gd.D);
  a.t1 = gettime(c->p, c->zz[snapshot]);
  a.t2 = gettime(c->p, c->zz[snapshot - 1]);
  if (host_lc) {
    a.out = c->d_lc_scratch;
    a.pitch = n;
  } else {
    a.out = dev_lc + slice0;
    a.pitch = c->lc_length;
  }
  {
    Prof pr(c, "k_lightcone", 12.0 * (double)gd.D * gd.D * n, s);
    launch_lightcone(a, gd, s);
  }
  if (host_lc)
    MX_CUDA(cudaMemcpy2DAsync(host_lc + slice0, sizeof(float) * c->lc_length, c->d_lc_scratch, sizeof(float) * n,
                              sizeof(float) * n, (size_t)gd.D * gd.D, cudaMemcpyDeviceToHost, s));
}

// ======================================================================
// construct_baryon_grids (reionization.c:1353-1615) and calculate_Mvir_crit
// (physics/reionization.c:10-59)
// ======================================================================
// hubble_time (virial_properties.c:79-93), internal time units
static double hubble_time(const mx_ctx* c, int snapshot)
{
  const double zp1 = c->zz[snapshot] + 1;
  return 1.0 / (c->d.hubble_int * std::sqrt(c->p.omega_m * zp1 * zp1 * zp1 + c->p.omega_k * zp1 * zp1 +
                                            c->p.omega_lambda));
}

struct GalaxyScratch
{
  unsigned *keys_in, *keys;
  int *idx_in, *idx;
  void* sort_tmp;
  size_t sort_bytes;
  // device copies of host galaxy arrays
  float* pos;
  int* type;
  double *fesc, *gross, *bhm, *ebhm;
};

// Galaxy scratch in one allocation that grows with the galaxy count.
static GalaxyScratch galaxy_scratch(mx_ctx* c, int n, bool host_copy, cudaStream_t s)
{
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t nn = (size_t)std::max(n, 1);
  GalaxyScratch g{};
  g.sort_bytes = deposit_sort_bytes(n);
  size_t bytes = 4 * up(4 * nn) + up(g.sort_bytes);
  if (host_copy)
    bytes += up(12 * nn) + up(4 * nn) + 4 * up(8 * nn);
  if (bytes > c->gal_bytes) {
    MX_CUDA(cudaStreamSynchronize(s));
    MX_CUDA(cudaFree(c->d_gal));
    c->d_gal = nullptr;
    c->gal_bytes = 0;
    MX_CUDA(cudaMalloc(&c->d_gal, bytes));
    c->gal_bytes = bytes;
  }
  char* q = static_cast<char*>(c->d_gal);
  auto take = [&](size_t b) {
    char* r = q;
    q += up(b);
    return r;
  };
  g.keys_in = reinterpret_cast<unsigned*>(take(4 * nn));
  g.keys = reinterpret_cast<unsigned*>(take(4 * nn));
  g.idx_in = reinterpret_cast<int*>(take(4 * nn));
  g.idx = reinterpret_cast<int*>(take(4 * nn));
  g.sort_tmp = take(g.sort_bytes);
  if (host_copy) {
    g.pos = reinterpret_cast<float*>(take(12 * nn));
    g.type = reinterpret_cast<int*>(take(4 * nn));
    g.fesc = reinterpret_cast<double*>(take(8 * nn));
    g.gross = reinterpret_cast<double*>(take(8 * nn));
    g.bhm = reinterpret_cast<double*>(take(8 * nn));
    g.ebhm = reinterpret_cast<double*>(take(8 * nn));
  }
  return g;
}

static void check_galaxies(const mx_params& p, const mx_galaxies* gals, int flag_bh)
{
  if (!gals || gals->n < 0 || gals->n > INT32_MAX / 3)
    throw CudaError{ MX_EINVAL, "construct_baryon_grids: invalid galaxy list" };
  if (gals->n > 0 && (!gals->pos || !gals->type || !gals->fesc_weighted_gsm ||
                      (p.flag_spin_temp && !gals->gross_stellar_mass) ||
                      (flag_bh && (!gals->black_hole_mass || !gals->effective_bhm))))
    throw CudaError{ MX_EINVAL, "construct_baryon_grids: a galaxy array the configuration reads is NULL" };
}

// Deposit of device galaxy arrays into device grids.  `sfr_hist` holds the
// n_hist slices; the reference shifts them one snapshot back first
// (reionization.c:1384-1389), slice by slice from the oldest.
static void run_deposit(mx_ctx* c, int snapshot, const mx_galaxies& gal, const GalaxyScratch& gs, int flag_bh,
                        double bh_limit, double alpha_uv_bh, float* stars, float* wsfr, float* sfr, float* sfr_hist,
                        bool shift_history, cudaStream_t s)
{
  const mx_params& p = c->p;
  const GridDims& gd = c->gd;
  const bool spin = p.flag_spin_temp != 0;
  if (gd.N >= 0xffffffffLL)
    throw CudaError{ MX_ENOTSUP, "construct_baryon_grids: 32-bit cell keys hold grids below 2^32 - 1 cells" };
  if (spin && shift_history && sfr_hist)
    for (int k = c->n_hist - 2; k >= 0; k--)
      MX_CUDA(cudaMemcpyAsync(sfr_hist + (size_t)(k + 1) * gd.P, sfr_hist + (size_t)k * gd.P, sizeof(float) * gd.P,
                              cudaMemcpyDeviceToDevice, s));
  DepositArgs a{};
  a.n = (int)gal.n;
  a.pos = gal.pos;
  a.type = gal.type;
  a.fesc_gsm = gal.fesc_weighted_gsm;
  a.gross_sm = gal.gross_stellar_mass;
  a.bhm = gal.black_hole_mass;
  a.ebhm = gal.effective_bhm;
  a.flag_bh = flag_bh;
  a.bh_limit = bh_limit;
  a.alpha_uv_bh = alpha_uv_bh;
  a.alpha_uv = p.alpha_uv;
  a.box_size = p.box_size;
  a.spin = spin;
  a.sfr_timescale = p.reion_sfr_timescale * hubble_time(c, snapshot);
  a.keys_in = gs.keys_in;
  a.keys = gs.keys;
  a.idx_in = gs.idx_in;
  a.idx = gs.idx;
  // REAL sums in unfiltered-spectrum scratch slots 0-2
  a.buf_stars = reinterpret_cast<float*>(c->d_unf);
  a.buf_wsfr = reinterpret_cast<float*>(c->d_unf + gd.C);
  a.buf_sfr = reinterpret_cast<float*>(c->d_unf + 2 * gd.C);
  a.err = c->d_err;
  a.stars = stars;
  a.weighted_sfr = wsfr;
  a.sfr = sfr;
  a.sfr_hist0 = sfr_hist;
  {
    Prof pr(c, "deposit", (double)gal.n * 44.0 + 4.0 * gd.P * (spin ? 5 : 2), s);
    MX_CUDA(launch_deposit(a, gs.sort_tmp, gs.sort_bytes, gd, s));
  }
  unsigned int errw = 0;
  MX_CUDA(cudaMemcpyAsync(&errw, c->d_err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
  MX_CUDA(cudaStreamSynchronize(s));
  if (errw) {
    MX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), s));
    throw CudaError{ MX_EINVAL, "construct_baryon_grids: a galaxy lies below the box (negative grid index)" };
  }
}

// ======================================================================
// C ABI
// ======================================================================
template <class F>
static int guarded(mx_ctx* c, F&& f)
{
  if (!c)
    return MX_EINVAL;
  try {
    if (cudaSetDevice(c->device) != cudaSuccess)
      throw CudaError{ MX_ECUDA, "cudaSetDevice failed" };
    f();
    // a launch that never ran (resources, configuration) leaves no trace but
    // this error
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess)
      throw CudaError{ MX_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(le) };
    c->err.clear();
    return MX_OK;
  } catch (const CudaError& e) {
    c->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    c->err = "host allocation failed";
    return MX_ENOMEM;
  } catch (const std::exception& e) {
    c->err = e.what();
    return MX_EINVAL;
  }
}

// Device grids must be 8-byte aligned: cuFFT reads its real inputs in pairs,
// as do the fused transforms (any CUDA allocator gives 256-byte alignment; a
// float pointer alone guarantees 4).
static void check_device_grids(const mx_grids* dev)
{
  if (!dev)
    throw CudaError{ MX_EINVAL, "NULL grids" };
  const float* const ptrs[] = { dev->deltax,  dev->stars,  dev->weighted_sfr, dev->sfr,        dev->sfr_histories,
                                dev->N_rec,   dev->x_e_box, dev->x_e_box_prev, dev->Tk_box,    dev->TS_box,
                                dev->xH,      dev->z_at_ionization, dev->r_bubble, dev->J_21,  dev->J_21_at_ionization,
                                dev->Gamma12, dev->delta_T, dev->vel };
  for (const float* q : ptrs)
    if ((uintptr_t)q % 8 != 0)
      throw CudaError{ MX_EINVAL, "device grids must be 8-byte aligned" };
}

static void check_snapshot(mx_ctx* c, int snapshot)
{
  if (c->zz.empty())
    throw CudaError{ MX_ESTATE, "mx_set_redshifts has not been called" };
  if (snapshot < 0 || snapshot >= (int)c->zz.size() || snapshot >= 1000)
    throw CudaError{ MX_EINVAL, "snapshot out of range" };
}

static cudaStream_t pick(mx_ctx* c, void* stream) { return stream ? (cudaStream_t)stream : c->stream; }

// The device step (ComputeTs -> find_HII_bubbles -> 21cm box) as one CUDA
// graph: captured on the context stream (thread-local capture mode), then
// instantiated and launched on `s`; the reads back of the step run after the
// graph has completed.  Every call captures the step anew: its kernel
// arguments, radius parameters and history operations depend on the
// snapshot.
static void step_graph(mx_ctx* c, int snapshot, const mx_grids* dev, mx_globals* out, cudaStream_t s)
{
  cudaStream_t cs = c->stream;
  mx_globals scratch{};
  mx_globals* o = out ? out : &scratch;
  c->stage_used = 0;
  c->finishers.clear();
  c->graph_keep.clear();
  cudaGraph_t graph = nullptr;
  int launches = 0;
  // cuFFT plans allocate their work areas when created, which a capture
  // does not allow: create the ones the step uses first
  if (!c->fused_fft) {
    c->c2r_plan(n_fields(c->p));
    if (c->p.flag_spin_temp)
      c->c2r_plan(1);
  }
  if (c->p.flag_spin_temp && c->p.flag_pecvel > 0)
    c->c2r_plan(1);
  MX_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  try {
    if (c->p.flag_spin_temp) {
      run_ComputeTs(c, snapshot, dev, o, cs);
      launches += o->gpu_launches;
    }
    run_find_HII_bubbles(c, snapshot, dev, o, cs);
    launches += o->gpu_launches;
    if (c->p.flag_21cm) {
      run_delta_T(c, snapshot, dev, o, cs);
      launches += o->gpu_launches;
    }
  } catch (...) {
    c->capturing = false;
    if (cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph)
      cudaGraphDestroy(graph);
    c->finishers.clear();
    c->graph_keep.clear();
    throw;
  }
  c->capturing = false;
  MX_CUDA(cudaStreamEndCapture(cs, &graph));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess)
    throw CudaError{ MX_ECUDA, std::string("step graph: ") + cudaGetErrorString(ei) };
  const cudaError_t el = cudaGraphLaunch(exec, s);
  const cudaError_t es = el == cudaSuccess ? cudaStreamSynchronize(s) : el;
  cudaGraphExecDestroy(exec);
  if (es != cudaSuccess)
    throw CudaError{ MX_ECUDA, std::string("step graph: ") + cudaGetErrorString(es) };
  std::vector<std::function<void()>> fin;
  fin.swap(c->finishers);
  c->graph_keep.clear();
  for (auto& f : fin)
    f();
  c->stage_used = 0;
  if (out)
    out->gpu_launches = launches;
}

extern "C" {

const char* mx_build_info(void) { return "meraxes_gb300 reion step, sm_103a, abi 1"; }

int64_t mx_lightcone_init(mx_ctx* ctx, double end_redshift, int32_t last_output_snap, int32_t* end_snapshot)
{
  long long n = 0;
  const int rc = guarded(ctx, [&]() {
    n = lightcone_init(ctx, end_redshift, last_output_snap);
    if (end_snapshot)
      *end_snapshot = ctx->lc_end_snapshot;
  });
  return rc == MX_OK ? (int64_t)n : (int64_t)rc;
}

int mx_ConstructLightcone(mx_ctx* ctx, int32_t snapshot, const float* delta_T, float* delta_T_prev, float* lightcone,
                          float* lightcone_redshifts)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!delta_T || !delta_T_prev || !lightcone || !lightcone_redshifts)
      throw CudaError{ MX_EINVAL, "ConstructLightcone: NULL pointer" };
    cudaStream_t s = ctx->stream;
    const size_t bytes = sizeof(float) * ctx->gd.N;
    if (snapshot > 0) {
      // the two co-eval boxes go to unfiltered-spectrum scratch (slots 0, 1)
      float* d0 = reinterpret_cast<float*>(ctx->d_unf);
      float* d1 = reinterpret_cast<float*>(ctx->d_unf + ctx->gd.C);
      MX_CUDA(cudaMemcpyAsync(d0, delta_T, bytes, cudaMemcpyHostToDevice, s));
      MX_CUDA(cudaMemcpyAsync(d1, delta_T_prev, bytes, cudaMemcpyHostToDevice, s));
      construct_lightcone(ctx, snapshot, d0, d1, nullptr, lightcone, lightcone_redshifts, s);
      MX_CUDA(cudaStreamSynchronize(s));
    } else {
      construct_lightcone(ctx, snapshot, nullptr, nullptr, nullptr, lightcone, lightcone_redshifts, s);
    }
    std::memcpy(delta_T_prev, delta_T, bytes);
  });
}

int mx_ConstructLightcone_device(mx_ctx* ctx, int32_t snapshot, const float* delta_T, float* delta_T_prev,
                                 float* lightcone, float* lightcone_redshifts, void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!delta_T || !delta_T_prev || !lightcone || !lightcone_redshifts)
      throw CudaError{ MX_EINVAL, "ConstructLightcone: NULL pointer" };
    cudaStream_t s = pick(ctx, stream);
    construct_lightcone(ctx, snapshot, delta_T, delta_T_prev, lightcone, nullptr, lightcone_redshifts, s);
    MX_CUDA(cudaMemcpyAsync(delta_T_prev, delta_T, sizeof(float) * ctx->gd.N, cudaMemcpyDeviceToDevice, s));
  });
}

int32_t mx_ps_length(const mx_ctx* ctx)
{
  if (!ctx)
    return MX_EINVAL;
  float edges[PS_MAX_BINS + 1], dk, vol;
  try {
    return ps_edges(ctx->p, edges, PS_MAX_BINS, &dk, &vol);
  } catch (const CudaError& e) {
    return e.code;
  }
}

int mx_Compute_PS(mx_ctx* ctx, const float* delta_T, float* ps_k, float* ps_data, float* ps_error, int32_t cap)
{
  int nb = 0;
  const int rc = guarded(ctx, [&]() {
    if (!delta_T || !ps_k || !ps_data || !ps_error)
      throw CudaError{ MX_EINVAL, "Compute_PS: NULL pointer" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    MX_CUDA(cudaMemcpyAsync(ctx->mirror.delta_T, delta_T, sizeof(float) * ctx->gd.N, cudaMemcpyHostToDevice, s));
    nb = run_power_spectrum(ctx, ctx->mirror.delta_T, ps_k, ps_data, ps_error, cap, s);
  });
  return rc == MX_OK ? nb : rc;
}

int mx_Compute_PS_device(mx_ctx* ctx, const float* delta_T, float* ps_k, float* ps_data, float* ps_error, int32_t cap,
                         void* stream)
{
  int nb = 0;
  const int rc = guarded(ctx, [&]() {
    if (!delta_T || !ps_k || !ps_data || !ps_error)
      throw CudaError{ MX_EINVAL, "Compute_PS: NULL pointer" };
    nb = run_power_spectrum(ctx, delta_T, ps_k, ps_data, ps_error, cap, pick(ctx, stream));
  });
  return rc == MX_OK ? nb : rc;
}

int mx_set_xray_params(mx_ctx* ctx, double lx_gal, double nu_xray_gal_threshold)
{
  return guarded(ctx, [&]() {
    if (!(lx_gal > 0) || !(nu_xray_gal_threshold > 0) || !(nu_xray_gal_threshold < ctx->p.nu_xray_max))
      throw CudaError{ MX_EINVAL, "X-ray parameters out of range" };
    ctx->p.lx_gal = lx_gal;
    ctx->p.nu_xray_gal_threshold = nu_xray_gal_threshold;
  });
}

int mx_ps_loss_device(mx_ctx* ctx, const float* delta_T, int32_t nbins, const float* edges, const float* target,
                      double* loss, float* P, float* grad_delta_T, void* stream)
{
  return guarded(ctx, [&]() {
    if (!delta_T || !edges || !target || !loss)
      throw CudaError{ MX_EINVAL, "ps_loss: NULL pointer" };
    ensure_adjoint_scratch(ctx);
    *loss = run_ps_loss(ctx, delta_T, nbins, edges, target, P, grad_delta_T, pick(ctx, stream));
    if (grad_delta_T)
      MX_CUDA(cudaStreamSynchronize(pick(ctx, stream)));
  });
}

int mx_adjoint_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* saved, const float* grad_delta_T,
                      float* grad_sfr, float* grad_stars, double* grad_params, void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    run_adjoint(ctx, snapshot, saved, grad_delta_T, grad_sfr, grad_stars, grad_params, pick(ctx, stream));
  });
}

int mx_construct_baryon_grids(mx_ctx* ctx, int32_t snapshot, const mx_galaxies* galaxies, int32_t flag_bh_feedback,
                              double bh_limit, double alpha_uv_bh, mx_grids* grids)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    const mx_params& p = ctx->p;
    const GridDims& gd = ctx->gd;
    check_galaxies(p, galaxies, flag_bh_feedback);
    const bool spin = p.flag_spin_temp != 0;
    const bool hist = spin && ctx->n_hist > 0;
    if (!grids || !grids->stars || !grids->weighted_sfr || (spin && !grids->sfr) || (hist && !grids->sfr_histories))
      throw CudaError{ MX_EINVAL, "construct_baryon_grids: an output grid is NULL" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    const int n = (int)galaxies->n;
    const GalaxyScratch gs = galaxy_scratch(ctx, n, true, s);
    mx_galaxies dg{};
    dg.n = n;
    dg.pos = gs.pos;
    dg.type = gs.type;
    dg.fesc_weighted_gsm = gs.fesc;
    dg.gross_stellar_mass = spin ? gs.gross : nullptr;
    dg.black_hole_mass = flag_bh_feedback ? gs.bhm : nullptr;
    dg.effective_bhm = flag_bh_feedback ? gs.ebhm : nullptr;
    if (n > 0) {
      MX_CUDA(cudaMemcpyAsync(gs.pos, galaxies->pos, 12 * (size_t)n, cudaMemcpyHostToDevice, s));
      MX_CUDA(cudaMemcpyAsync(gs.type, galaxies->type, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
      MX_CUDA(cudaMemcpyAsync(gs.fesc, galaxies->fesc_weighted_gsm, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
      if (spin)
        MX_CUDA(cudaMemcpyAsync(gs.gross, galaxies->gross_stellar_mass, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
      if (flag_bh_feedback) {
        MX_CUDA(cudaMemcpyAsync(gs.bhm, galaxies->black_hole_mass, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
        MX_CUDA(cudaMemcpyAsync(gs.ebhm, galaxies->effective_bhm, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
      }
    }
    // older history slices move on the host; the newest goes through the
    // device, which writes its cells and keeps its padding
    const size_t slice = sizeof(float) * gd.P;
    if (hist) {
      std::memmove(grids->sfr_histories + gd.P, grids->sfr_histories, slice * (size_t)(ctx->n_hist - 1));
      MX_CUDA(cudaMemcpyAsync(ctx->mirror.sfr_histories, grids->sfr_histories, slice, cudaMemcpyHostToDevice, s));
    }
    run_deposit(ctx, snapshot, dg, gs, flag_bh_feedback, bh_limit, alpha_uv_bh, ctx->mirror.stars,
                ctx->mirror.weighted_sfr, ctx->mirror.sfr, hist ? ctx->mirror.sfr_histories : nullptr, false, s);
    MX_CUDA(cudaMemcpyAsync(grids->stars, ctx->mirror.stars, slice, cudaMemcpyDeviceToHost, s));
    MX_CUDA(cudaMemcpyAsync(grids->weighted_sfr, ctx->mirror.weighted_sfr, slice, cudaMemcpyDeviceToHost, s));
    if (spin)
      MX_CUDA(cudaMemcpyAsync(grids->sfr, ctx->mirror.sfr, slice, cudaMemcpyDeviceToHost, s));
    if (hist)
      MX_CUDA(cudaMemcpyAsync(grids->sfr_histories, ctx->mirror.sfr_histories, slice, cudaMemcpyDeviceToHost, s));
    MX_CUDA(cudaStreamSynchronize(s));
  });
}

int mx_construct_baryon_grids_device(mx_ctx* ctx, int32_t snapshot, const mx_galaxies* galaxies,
                                     int32_t flag_bh_feedback, double bh_limit, double alpha_uv_bh, mx_grids* grids,
                                     void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    const mx_params& p = ctx->p;
    check_galaxies(p, galaxies, flag_bh_feedback);
    const bool spin = p.flag_spin_temp != 0;
    const bool hist = spin && ctx->n_hist > 0;
    if (!grids || !grids->stars || !grids->weighted_sfr || (spin && !grids->sfr) || (hist && !grids->sfr_histories))
      throw CudaError{ MX_EINVAL, "construct_baryon_grids: an output grid is NULL" };
    const void* dbl[] = { galaxies->fesc_weighted_gsm, galaxies->gross_stellar_mass, galaxies->black_hole_mass,
                          galaxies->effective_bhm };
    for (const void* q : dbl)
      if ((uintptr_t)q % 8 != 0)
        throw CudaError{ MX_EINVAL, "construct_baryon_grids: device galaxy arrays must be 8-byte aligned" };
    cudaStream_t s = pick(ctx, stream);
    const GalaxyScratch gs = galaxy_scratch(ctx, (int)galaxies->n, false, s);
    run_deposit(ctx, snapshot, *galaxies, gs, flag_bh_feedback, bh_limit, alpha_uv_bh, grids->stars,
                grids->weighted_sfr, grids->sfr, hist ? grids->sfr_histories : nullptr, true, s);
  });
}

int mx_calculate_Mvir_crit(mx_ctx* ctx, double redshift, const double sm_params[5], const float* J_21_at_ionization,
                           const float* z_at_ionization, float* Mvir_crit)
{
  return guarded(ctx, [&]() {
    if (!sm_params || !J_21_at_ionization || !z_at_ionization || !Mvir_crit)
      throw CudaError{ MX_EINVAL, "calculate_Mvir_crit: NULL pointer" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    const size_t bytes = sizeof(float) * ctx->gd.N;
    float* d_out = reinterpret_cast<float*>(ctx->d_unf);
    MX_CUDA(cudaMemcpyAsync(ctx->mirror.J_21_at_ionization, J_21_at_ionization, bytes, cudaMemcpyHostToDevice, s));
    MX_CUDA(cudaMemcpyAsync(ctx->mirror.z_at_ionization, z_at_ionization, bytes, cudaMemcpyHostToDevice, s));
    {
      Prof pr(ctx, "k_Mvir_crit", 12.0 * ctx->gd.N, s);
      launch_Mvir_crit(redshift, sm_params, ctx->p.hubble_h, ctx->mirror.J_21_at_ionization,
                       ctx->mirror.z_at_ionization, d_out, ctx->gd, s);
    }
    MX_CUDA(cudaGetLastError());
    MX_CUDA(cudaMemcpyAsync(Mvir_crit, d_out, bytes, cudaMemcpyDeviceToHost, s));
    MX_CUDA(cudaStreamSynchronize(s));
  });
}

int mx_calculate_Mvir_crit_device(mx_ctx* ctx, double redshift, const double sm_params[5],
                                  const float* J_21_at_ionization, const float* z_at_ionization, float* Mvir_crit,
                                  void* stream)
{
  return guarded(ctx, [&]() {
    if (!sm_params || !J_21_at_ionization || !z_at_ionization || !Mvir_crit)
      throw CudaError{ MX_EINVAL, "calculate_Mvir_crit: NULL pointer" };
    cudaStream_t s = pick(ctx, stream);
    {
      Prof pr(ctx, "k_Mvir_crit", 12.0 * ctx->gd.N, s);
      launch_Mvir_crit(redshift, sm_params, ctx->p.hubble_h, J_21_at_ionization, z_at_ionization, Mvir_crit, ctx->gd,
                       s);
    }
    MX_CUDA(cudaGetLastError());
  });
}

static int create_ctx(const mx_params* params, const char* tables_dir, size_t work_cap_bytes, mx_ctx** out);

int mx_create(const mx_params* params, const char* tables_dir, mx_ctx** out)
{
  return create_ctx(params, tables_dir, 0, out);
}

int mx_create_limited(const mx_params* params, const char* tables_dir, size_t max_work_bytes, mx_ctx** out)
{
  return create_ctx(params, tables_dir, max_work_bytes, out);
}

// Block-size autotuner of the fused x- and y-pass.  Both passes are
// available with 256 and 512 threads per block and give identical results
// (the thread count changes only which thread runs which column transform,
// not the arithmetic).  Which one is faster depends on the grid size: at
// small grids the larger block hides more latency, at 512^3 the smaller one
// keeps more blocks resident.  The context times both on its own scratch at
// creation (a zero spectrum, up to four radii, best of three launches) and
// keeps the faster.  MX_XPASS_THREADS / MX_YPASS_THREADS (256 or 512) fix a
// choice; MX_AUTOTUNE=0 keeps the defaults (x 512, y 256).
// Register budget of the threshold z-pass (power-of-two grids): 2 resident
// blocks per SM (128 registers) or 3 (80, with a few spills).  Timed at
// context creation on scratch: up to 4 radii of zero spectra of the
// context's fields and six zero state grids in the transform work buffer,
// best of three launches after one warm-up; MX_ZPASS_BLOCKS fixes it.
static void tune_zpass(mx_ctx* c)
{
  if (const char* env = std::getenv("MX_ZPASS_BLOCKS")) {
    c->z_blocks = std::atoi(env) == 3 ? 3 : 2;
    return;
  }
  const char* at = std::getenv("MX_AUTOTUNE");
  if ((at && std::string(at) == "0") || !c->fused_fft || (c->gd.D & (c->gd.D - 1)) != 0)
    return;
  const GridDims& gd = c->gd;
  const int G = n_fields(c->p);
  const long long spectrum_bytes = (long long)sizeof(float2) * c->work_C;
  const long long state_bytes = 6LL * gd.N * (long long)sizeof(float);
  const long long state_spectra = (state_bytes + spectrum_bytes - 1) / spectrum_bytes;
  const int nr = (int)std::min<long long>(4, (c->work_fields - state_spectra) / G);
  if (nr < 1)
    return;
  cudaStream_t s = c->stream;
  float* state = reinterpret_cast<float*>(c->d_work + (long long)nr * G * c->work_C);
  MX_CUDA(cudaMemsetAsync(c->d_work, 0, (size_t)(spectrum_bytes * nr * G + state_bytes), s));
  std::vector<RadiusParams> rps(nr);
  for (RadiusParams& q : rps) {
    q = RadiusParams{};
    q.R = q.M_mean = q.R_cubed = 1.0;
  }
  MX_CUDA(cudaMemcpyAsync(c->d_rp, rps.data(), sizeof(RadiusParams) * nr, cudaMemcpyHostToDevice, s));
  const bool spin = c->p.flag_spin_temp != 0, recomb = c->p.flag_recombinations != 0;
  ZThresholdArgs za;
  za.spectra = c->d_work;
  za.C = c->work_C;
  za.G = G;
  za.idx_xe = spin ? 3 : -1;
  za.idx_nr = recomb ? (spin ? 4 : 3) : -1;
  za.n_r = nr;
  za.n_f = nr;
  za.rp = c->d_rp;
  for (int f = 0; f < MAX_FIELDS; f++)
    za.direct[f] = nullptr;
  za.xH = state;
  za.z_at_ion = state + gd.N;
  za.r_bubble = state + 2 * gd.N;
  za.J21 = state + 3 * gd.N;
  za.J21_at_ion = state + 4 * gd.N;
  za.Gamma12 = state + 5 * gd.N;
  za.pixel_volume = 1.0;
  za.eff = 1.0;
  za.redshift = 10.0;
  za.gamma_halo_bias = 1.0f;
  za.uvb = c->p.uvb_flag;
  za.recomb = recomb;
  za.spin = spin;
  za.err = c->d_err;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MX_CUDA(cudaEventCreate(&e0));
  MX_CUDA(cudaEventCreate(&e1));
  float best[2] = { 1e30f, 1e30f };
  for (int v = 0; v < 2; v++) {
    za.blocks_per_sm = v + 2;
    launch_fft_z_threshold(gd.D, za, s);  // warm-up
    for (int i = 0; i < 3; i++) {
      cudaEventRecord(e0, s);
      launch_fft_z_threshold(gd.D, za, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      best[v] = std::min(best[v], ms);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MX_CUDA(cudaGetLastError());
  MX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), s));
  MX_CUDA(cudaStreamSynchronize(s));
  c->z_blocks = best[1] < best[0] ? 3 : 2;
}

static void tune_fft(mx_ctx* c)
{
  auto env_threads = [](const char* name) {
    const char* v = std::getenv(name);
    const int t = v ? std::atoi(v) : 0;
    return (t == 256 || t == 512) ? t : 0;
  };
  if (c->fused_fft && (c->gd.D & (c->gd.D - 1)) != 0) {
    // grids with a factor 3 run one block size (384 threads: 24 slots of 16
    // columns, a multiple of the radix-3 and radix-2/4/8 steps)
    c->x_threads = c->y_threads = 384;
    return;
  }
  const int fx = env_threads("MX_XPASS_THREADS"), fy = env_threads("MX_YPASS_THREADS");
  if (fx)
    c->x_threads = fx;
  if (fy)
    c->y_threads = fy;
  const char* at = std::getenv("MX_AUTOTUNE");
  if ((fx && fy) || (at && std::string(at) == "0") || !c->fused_fft)
    return;
  const GridDims& gd = c->gd;
  cudaStream_t s = c->stream;
  MX_CUDA(cudaMemsetAsync(c->d_unf, 0, sizeof(float2) * c->unf_C, s));
  const int n = (int)std::min<long long>(std::min<long long>(c->work_fields, 4), MAX_RADII);
  XPassArgs xa;
  for (int f = 0; f < MAX_FIELDS; f++)
    xa.in[f] = f == 0 ? c->d_unf : nullptr;
  xa.G = 1;
  xa.n = n;
  xa.out = c->d_work;
  xa.C = c->work_C;
  for (int r = 0; r < n; r++) {
    xa.R[r] = (float)(c->p.box_size / 8.0);
    xa.apply[r] = 1;
  }
  xa.filter_type = c->p.filter_type;
  xa.delta_k = (float)(2.0 * k::PI / c->p.box_size);
  xa.scale = (float)(1.0 / (double)gd.N);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MX_CUDA(cudaEventCreate(&e0));
  MX_CUDA(cudaEventCreate(&e1));
  auto best_ms = [&](auto&& launch) {
    launch();  // warm-up
    float best = 1e30f;
    for (int i = 0; i < 3; i++) {
      cudaEventRecord(e0, s);
      launch();
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, ms);
    }
    return best;
  };
  const int cand[2] = { 256, 512 };
  float tx[2] = { 0, 0 }, ty[2] = { 0, 0 };
  for (int i = 0; i < 2; i++) {
    if (!fx)
      tx[i] = best_ms([&] { launch_fft_x_filter(gd.D, xa, cand[i], s); });
    if (!fy)
      ty[i] = best_ms([&] { launch_fft_y(gd.D, c->d_work, c->work_C, n, cand[i], s); });
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MX_CUDA(cudaGetLastError());
  MX_CUDA(cudaStreamSynchronize(s));
  if (!fx)
    c->x_threads = tx[0] < tx[1] ? 256 : 512;
  if (!fy)
    c->y_threads = ty[0] < ty[1] ? 256 : 512;
}

static int create_ctx(const mx_params* params, const char* tables_dir, size_t work_cap_bytes, mx_ctx** out)
{
  g_create_error.clear();
  if (!params || !out) {
    g_create_error = "mx_create: NULL argument";
    return MX_EINVAL;
  }
  *out = nullptr;
  const mx_params& p = *params;
  if (p.abi_version != MX_ABI_VERSION) {
    g_create_error = "mx_create: abi_version mismatch";
    return MX_EINVAL;
  }
  if (p.grid_dim < 2 || p.grid_dim % 2 != 0 || p.grid_dim > 2048 || !(p.box_size > 0) || !(p.delta_r_factor > 1.0) ||
      p.filter_type < 0 || p.filter_type > 2 || p.rtom_filter_type < 0 || p.rtom_filter_type > 1 ||
      (p.flag_spin_temp && (p.ts_num_filter_steps < 1 || p.ts_num_filter_steps > MAX_SHELLS ||
                            p.ts_heating_filter_type < 0 || p.ts_heating_filter_type > 2))) {
    g_create_error = "mx_create: invalid parameter";
    return MX_EINVAL;
  }
  std::unique_ptr<mx_ctx> c(new (std::nothrow) mx_ctx());
  if (!c) {
    g_create_error = "mx_create: host allocation failed";
    return MX_ENOMEM;
  }
  c->p = p;
  c->d.init(p);
  c->gd.D = p.grid_dim;
  c->gd.H = p.grid_dim / 2 + 1;
  c->gd.C = (long long)p.grid_dim * p.grid_dim * c->gd.H;
  c->gd.N = (long long)p.grid_dim * p.grid_dim * p.grid_dim;
  c->gd.P = 2 * c->gd.C;
  c->tables_dir = tables_dir ? tables_dir : "";
  std::memset(c->stored_fcoll, 0, sizeof(c->stored_fcoll));
  c->nthreads = std::max(1, std::min(64, hw_threads()));
  if (const char* env = std::getenv("MX_HOST_THREADS"))
    c->nthreads = std::max(1, std::atoi(env));
  if (const char* env = std::getenv("MX_TS_EARLY_SHELLS"))
    c->early_shells = std::atoi(env) != 0;

  c->fused_fft = fft3d_supported(p.grid_dim);
  if (const char* env = std::getenv("MX_TRANSFORM"))
    if (std::string(env) == "cufft")
      c->fused_fft = false;
  try {
    if (cudaGetDevice(&c->device) != cudaSuccess)
      throw CudaError{ MX_ECUDA, "no CUDA device" };
    // poll limit of the pipeline waits (process-wide on this device): the
    // default, or a lower one that a test of the give-up path asks for
    {
      long long polls = bulk::WAIT_LIMIT_ITERS;
      if (const char* env = std::getenv("MX_WAIT_POLL_LIMIT"))
        polls = std::max(1LL, std::min(polls, std::atoll(env)));
      MX_CUDA(fft_set_wait_polls(polls));
      MX_CUDA(ts_set_wait_polls(polls));
    }
    MX_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    MX_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    MX_CUDA(cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_cf, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_b, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_ts_first, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_ts_sfr, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_ts_tk, cudaEventDisableTiming));
    MX_CUDA(cudaEventCreateWithFlags(&c->ev_state, cudaEventDisableTiming));
    if (p.filter_type != 0 && p.filter_type != 1 && p.filter_type != 2)
      throw CudaError{ MX_EINVAL, "invalid filter type" };
    if (p.flag_spin_temp) {
      std::string e;
      int rc = c->ht.load(p, c->tables_dir, &e);
      if (rc)
        throw CudaError{ rc, e };
    }
    if (p.flag_recombinations) {
      c->rr.build(p, c->d, c->nthreads);
      const size_t n = c->rr.y.size();
      // FP32 copy of the table, rescaled by a power of two to O(1) values
      double m = 0.0;
      for (size_t i = 0; i < n; i++)
        if (std::isfinite(c->rr.y[i]))
          m = std::max(m, std::fabs(c->rr.y[i]));
      int e = 0;
      std::frexp(m > 0 ? m : 1.0, &e);
      c->rr_scale = std::ldexp(1.0, -e);
      std::vector<float> xf(c->rr.lng.begin(), c->rr.lng.end()), yf(n), cf(n);
      for (size_t i = 0; i < n; i++) {
        yf[i] = (float)(c->rr.y[i] * c->rr_scale);
        cf[i] = (float)(c->rr.c[i] * c->rr_scale);
      }
      MX_CUDA(cudaMalloc(&c->d_rr_x, sizeof(float) * xf.size()));
      MX_CUDA(cudaMalloc(&c->d_rr_y, sizeof(float) * n));
      MX_CUDA(cudaMalloc(&c->d_rr_c, sizeof(float) * n));
      MX_CUDA(cudaMemcpy(c->d_rr_x, xf.data(), sizeof(float) * xf.size(), cudaMemcpyHostToDevice));
      MX_CUDA(cudaMemcpy(c->d_rr_y, yf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
      MX_CUDA(cudaMemcpy(c->d_rr_c, cf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    }
    c->work_cap_bytes = work_cap_bytes;
    c->alloc_scratch();
    tune_fft(c.get());
    tune_zpass(c.get());
  } catch (const CudaError& e) {
    g_create_error = e.msg;
    return e.code == MX_ECUDA && e.msg.find("memory") != std::string::npos ? MX_ENOMEM : e.code;
  }
  *out = c.release();
  return MX_OK;
}

void mx_destroy(mx_ctx* ctx)
{
  if (!ctx)
    return;
  cudaSetDevice(ctx->device);
  delete ctx;
}

const char* mx_last_error(const mx_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int mx_set_redshifts(mx_ctx* ctx, const double* zz, int32_t n_snaps)
{
  return guarded(ctx, [&]() {
    if (!zz || n_snaps < 1 || n_snaps > 1000)
      throw CudaError{ MX_EINVAL, "mx_set_redshifts: bad list" };
    ctx->zz.assign(zz, zz + n_snaps);
    ctx->n_hist = ctx->p.flag_spin_temp ? n_sfr_histories(ctx->p, ctx->zz) : 0;
  });
}

int32_t mx_n_sfr_histories(const mx_ctx* ctx) { return ctx ? ctx->n_hist : -1; }

int32_t mx_zpass_blocks_per_sm(const mx_ctx* ctx)
{
  if (!ctx)
    return MX_EINVAL;
  return ctx->fused_fft && (ctx->gd.D & (ctx->gd.D - 1)) == 0 ? ctx->z_blocks : 0;
}

int mx_fft_block_sizes(const mx_ctx* ctx, int32_t* x_threads, int32_t* y_threads)
{
  if (!ctx || !x_threads || !y_threads)
    return MX_EINVAL;
  *x_threads = ctx->fused_fft ? ctx->x_threads : 0;
  *y_threads = ctx->fused_fft ? ctx->y_threads : 0;
  return MX_OK;
}

int mx_profile_enable(mx_ctx* ctx, int32_t on)
{
  return guarded(ctx, [&]() {
    MX_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->prof.clear();
    ctx->prof_on = on != 0;
  });
}

int32_t mx_profile_read(mx_ctx* ctx, mx_kernel_stat* out, int32_t cap)
{
  if (!ctx)
    return MX_EINVAL;
  std::vector<mx_kernel_stat> stats;
  const int rc = guarded(ctx, [&]() {
    MX_CUDA(cudaDeviceSynchronize());
    for (const auto& r : ctx->prof) {
      float ms = 0.f;
      MX_CUDA(cudaEventElapsedTime(&ms, ctx->prof_events[r.ev], ctx->prof_events[r.ev + 1]));
      auto it = std::find_if(stats.begin(), stats.end(),
                             [&](const mx_kernel_stat& k) { return std::strcmp(k.name, r.name) == 0; });
      if (it == stats.end()) {
        mx_kernel_stat k{};
        std::snprintf(k.name, sizeof k.name, "%s", r.name);
        stats.push_back(k);
        it = stats.end() - 1;
      }
      it->launches++;
      it->ms += ms;
      it->bytes += r.bytes;
    }
  });
  if (rc != MX_OK)
    return rc;
  for (int i = 0; i < (int)stats.size() && i < cap; i++)
    out[i] = stats[i];
  return (int32_t)stats.size();
}

int32_t mx_filter_radii(const mx_ctx* ctx, double* radii, int32_t cap)
{
  if (!ctx)
    return MX_EINVAL;
  const std::vector<double> r = filter_radii(ctx->p);
  for (int i = 0; i < (int)r.size() && i < cap; i++)
    radii[i] = r[i];
  return (int32_t)r.size();
}

int mx_find_HII_bubbles_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    check_device_grids(dev);
    run_find_HII_bubbles(ctx, snapshot, dev, out, pick(ctx, stream));
  });
}

int mx_ComputeTs_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    check_device_grids(dev);
    run_ComputeTs(ctx, snapshot, dev, out, pick(ctx, stream));
  });
}

int mx_ComputeBrightnessTemperatureBox_device(mx_ctx* ctx,
                                              int32_t snapshot,
                                              const mx_grids* dev,
                                              mx_globals* out,
                                              void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    check_device_grids(dev);
    run_delta_T(ctx, snapshot, dev, out, pick(ctx, stream));
  });
}

int mx_set_step_graph(mx_ctx* ctx, int32_t on)
{
  return guarded(ctx, [&]() { ctx->graph_on = on != 0; });
}

int mx_step_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    check_device_grids(dev);
    cudaStream_t s = pick(ctx, stream);
    if (ctx->graph_on) {
      step_graph(ctx, snapshot, dev, out, s);
      return;
    }
    int launches = 0;
    if (ctx->p.flag_spin_temp) {
      run_ComputeTs(ctx, snapshot, dev, out, s);
      launches += out ? out->gpu_launches : 0;
    }
    run_find_HII_bubbles(ctx, snapshot, dev, out, s);
    launches += out ? out->gpu_launches : 0;
    if (ctx->p.flag_21cm) {
      run_delta_T(ctx, snapshot, dev, out, s);
      launches += out ? out->gpu_launches : 0;
    }
    if (out)
      out->gpu_launches = launches;
  });
}

// ------------------------------------------------------------ host family
namespace {
enum Dir { IN = 1, OUT = 2 };
struct FieldIO
{
  float* mx_grids::*member;
  bool padded;
  int dir;
};

void copy_fields(mx_ctx* c, const mx_grids* host, const std::vector<FieldIO>& fields, int dir, cudaStream_t s)
{
  for (const FieldIO& f : fields) {
    if (!(f.dir & dir))
      continue;
    float* h = host->*(f.member);
    float* d = c->mirror.*(f.member);
    if (!h)
      continue;
    // vel is read (and converted in place) only by the peculiar-velocity modes
    if (f.member == &mx_grids::vel && !(c->p.flag_spin_temp && c->p.flag_pecvel > 0))
      continue;
    const size_t n = f.padded ? (size_t)c->gd.P : (size_t)c->gd.N;
    if (dir == IN)
      MX_CUDA(cudaMemcpyAsync(d, h, n * sizeof(float), cudaMemcpyHostToDevice, s));
    else
      MX_CUDA(cudaMemcpyAsync(h, d, n * sizeof(float), cudaMemcpyDeviceToHost, s));
  }
}

// Device grids for a host call: the mirror, with NULL where the caller passed NULL.
mx_grids mirror_for(mx_ctx* c, const mx_grids* host)
{
  mx_grids m = c->mirror;
  float* mx_grids::*all[] = { &mx_grids::deltax,   &mx_grids::stars,        &mx_grids::weighted_sfr,
                              &mx_grids::sfr,      &mx_grids::sfr_histories, &mx_grids::N_rec,
                              &mx_grids::x_e_box,  &mx_grids::x_e_box_prev, &mx_grids::Tk_box,
                              &mx_grids::TS_box,   &mx_grids::xH,           &mx_grids::z_at_ionization,
                              &mx_grids::r_bubble, &mx_grids::J_21,         &mx_grids::J_21_at_ionization,
                              &mx_grids::Gamma12,  &mx_grids::delta_T,      &mx_grids::vel };
  for (auto mem : all)
    if (!(host->*mem))
      m.*mem = nullptr;
  return m;
}

const std::vector<FieldIO>& fhb_fields()
{
  static const std::vector<FieldIO> f = {
    { &mx_grids::deltax, true, IN },           { &mx_grids::stars, true, IN },
    { &mx_grids::weighted_sfr, true, IN },     { &mx_grids::x_e_box, true, IN },
    { &mx_grids::N_rec, true, IN | OUT },      { &mx_grids::xH, false, OUT },
    { &mx_grids::z_at_ionization, false, IN | OUT }, { &mx_grids::r_bubble, false, OUT },
    { &mx_grids::J_21, false, OUT },           { &mx_grids::J_21_at_ionization, false, IN | OUT },
    { &mx_grids::Gamma12, false, IN | OUT },
  };
  return f;
}
const std::vector<FieldIO>& ts_fields()
{
  static const std::vector<FieldIO> f = {
    { &mx_grids::deltax, true, IN },        { &mx_grids::stars, true, IN },
    { &mx_grids::sfr, true, IN | OUT },     { &mx_grids::x_e_box, true, OUT },
    { &mx_grids::x_e_box_prev, true, IN | OUT }, { &mx_grids::Tk_box, false, IN | OUT },
    { &mx_grids::TS_box, false, OUT },
  };
  return f;
}
const std::vector<FieldIO>& dt_fields()
{
  static const std::vector<FieldIO> f = {
    { &mx_grids::deltax, true, IN },
    { &mx_grids::xH, false, IN },
    { &mx_grids::TS_box, false, IN },
    { &mx_grids::delta_T, false, OUT },
    { &mx_grids::vel, true, IN | OUT },  // only with peculiar velocities (see copy_fields)
  };
  return f;
}

void copy_histories(mx_ctx* c, const mx_grids* host, cudaStream_t s)
{
  if (c->n_hist > 0 && host->sfr_histories)
    MX_CUDA(cudaMemcpyAsync(c->mirror.sfr_histories, host->sfr_histories, sizeof(float) * c->gd.P * c->n_hist,
                            cudaMemcpyHostToDevice, s));
}
}  // namespace

int mx_find_HII_bubbles(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!host)
      throw CudaError{ MX_EINVAL, "NULL grids" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    copy_fields(ctx, host, fhb_fields(), IN, s);
    mx_grids m = mirror_for(ctx, host);
    run_find_HII_bubbles(ctx, snapshot, &m, out, s);
    copy_fields(ctx, host, fhb_fields(), OUT, s);
    MX_CUDA(cudaStreamSynchronize(s));
  });
}

int mx_ComputeTs(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!host)
      throw CudaError{ MX_EINVAL, "NULL grids" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    copy_fields(ctx, host, ts_fields(), IN, s);
    copy_histories(ctx, host, s);
    mx_grids m = mirror_for(ctx, host);
    run_ComputeTs(ctx, snapshot, &m, out, s);
    copy_fields(ctx, host, ts_fields(), OUT, s);
    MX_CUDA(cudaStreamSynchronize(s));
  });
}

int mx_ComputeBrightnessTemperatureBox(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!host)
      throw CudaError{ MX_EINVAL, "NULL grids" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream;
    copy_fields(ctx, host, dt_fields(), IN, s);
    mx_grids m = mirror_for(ctx, host);
    run_delta_T(ctx, snapshot, &m, out, s);
    copy_fields(ctx, host, dt_fields(), OUT, s);
    MX_CUDA(cudaStreamSynchronize(s));
  });
}

// mx_step on host grids.  The grids cross in three groups so that the copies
// overlap the compute of the other stages:
//   1. ComputeTs inputs (and the SFR histories), on the compute stream;
//   2. find_HII_bubbles inputs that ComputeTs does not touch, on the copy
//      stream while ComputeTs runs; find_HII_bubbles waits for them;
//   3. ComputeTs outputs (final once it ends: find_HII_bubbles and the 21cm
//      box only read them), back on the copy stream while find_HII_bubbles
//      runs; the find_HII_bubbles outputs and delta_T at the end.
// x_e_box is not uploaded when ComputeTs runs: it writes x_e_box before
// find_HII_bubbles reads it.  Each grid crosses at most once per direction.
int mx_step(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out)
{
  return guarded(ctx, [&]() {
    check_snapshot(ctx, snapshot);
    if (!host)
      throw CudaError{ MX_EINVAL, "NULL grids" };
    ctx->ensure_mirror();
    cudaStream_t s = ctx->stream, cs = ctx->copy_stream;
    const bool spin = ctx->p.flag_spin_temp != 0, b21 = ctx->p.flag_21cm != 0;
    auto has = [](const std::vector<FieldIO>& v, float* mx_grids::*m) {
      for (const FieldIO& f : v)
        if (f.member == m)
          return true;
      return false;
    };
    std::vector<FieldIO> ts_in, fhb_in, ts_out, late_out;
    if (spin) {
      for (const FieldIO& f : ts_fields()) {
        if (f.dir & IN)
          ts_in.push_back({ f.member, f.padded, IN });
        if (f.dir & OUT)
          ts_out.push_back({ f.member, f.padded, OUT });
      }
    }
    for (const FieldIO& f : fhb_fields()) {
      if ((f.dir & IN) && !has(ts_in, f.member) && !(spin && has(ts_out, f.member)))
        fhb_in.push_back({ f.member, f.padded, IN });
      if ((f.dir & OUT) && !has(ts_out, f.member))
        late_out.push_back({ f.member, f.padded, OUT });
    }
    if (b21) {
      fhb_in.push_back({ &mx_grids::vel, true, IN });  // peculiar-velocity modes only
      late_out.push_back({ &mx_grids::vel, true, OUT });
      late_out.push_back({ &mx_grids::delta_T, false, OUT });
    }
    // The copy stream starts after the compute stream's earlier work and
    // carries every input: first sfr (the shells of the current SFR start on
    // it), then what ComputeTs's collapse fraction reads (stars, deltax,
    // x_e_box_prev), the SFR-history slices in the order the shell
    // operations first read them (slices no operation reads are not needed),
    // Tk_box, and the find_HII_bubbles inputs.  The compute stream waits for
    // each right before its first use (TsUploads), so most of the upload runs
    // under the shell transforms.
    MX_CUDA(cudaEventRecord(ctx->ev_a, s));
    MX_CUDA(cudaStreamWaitEvent(cs, ctx->ev_a, 0));
    TsUploads up{};
    if (spin) {
      auto upload = [&](float* mx_grids::*member, bool padded) {
        copy_fields(ctx, host, { { member, padded, IN } }, IN, cs);
      };
      if (ctx->early_shells) {
        upload(&mx_grids::sfr, true);
        MX_CUDA(cudaEventRecord(ctx->ev_ts_sfr, cs));
      }
      upload(&mx_grids::stars, true);
      upload(&mx_grids::deltax, true);
      upload(&mx_grids::x_e_box_prev, true);
      MX_CUDA(cudaEventRecord(ctx->ev_ts_first, cs));
      if (!ctx->early_shells) {
        upload(&mx_grids::sfr, true);
        MX_CUDA(cudaEventRecord(ctx->ev_ts_sfr, cs));
      }
      while ((int)ctx->ev_slices.size() < ctx->n_hist) {
        cudaEvent_t e = nullptr;
        MX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->ev_slices.push_back(e);
      }
      const ShellPlan sp = plan_shells(ctx->p, ctx->zz, snapshot);
      std::vector<char> sent(ctx->n_hist, 0);
      if (!sp.homogeneous && host->sfr_histories)
        for (const std::vector<SfrOp>& ops : sp.ops)
          for (const SfrOp& op : ops)
            if (op.kind >= SfrOp::LOAD && op.slice >= 0 && op.slice < ctx->n_hist && !sent[op.slice]) {
              const size_t P = (size_t)ctx->gd.P;
              MX_CUDA(cudaMemcpyAsync(ctx->mirror.sfr_histories + P * op.slice, host->sfr_histories + P * op.slice,
                                      sizeof(float) * P, cudaMemcpyHostToDevice, cs));
              MX_CUDA(cudaEventRecord(ctx->ev_slices[op.slice], cs));
              sent[op.slice] = 1;
            }
      upload(&mx_grids::Tk_box, false);
      MX_CUDA(cudaEventRecord(ctx->ev_ts_tk, cs));
      up = { ctx->ev_ts_first, ctx->ev_ts_sfr, ctx->ev_ts_tk, &ctx->ev_slices };
    }
    // find_HII_bubbles: the grids its forward transforms read (ev_b), then
    // the state grids its first threshold pass reads (ev_state)
    std::vector<FieldIO> fhb_early, fhb_state;
    for (const FieldIO& f : fhb_in)
      (f.member == &mx_grids::z_at_ionization || f.member == &mx_grids::J_21_at_ionization ||
           f.member == &mx_grids::Gamma12
         ? fhb_state
         : fhb_early)
        .push_back(f);
    copy_fields(ctx, host, fhb_early, IN, cs);
    MX_CUDA(cudaEventRecord(ctx->ev_b, cs));
    copy_fields(ctx, host, fhb_state, IN, cs);
    MX_CUDA(cudaEventRecord(ctx->ev_state, cs));
    mx_grids m = mirror_for(ctx, host);
    int launches = 0;
    if (spin) {
      run_ComputeTs(ctx, snapshot, &m, out, s, &up);
      launches += out ? out->gpu_launches : 0;
      MX_CUDA(cudaEventRecord(ctx->ev_a, s));
      MX_CUDA(cudaStreamWaitEvent(cs, ctx->ev_a, 0));
      copy_fields(ctx, host, ts_out, OUT, cs);
    }
    MX_CUDA(cudaStreamWaitEvent(s, ctx->ev_b, 0));
    // eight row slabs: the outputs of all but the last eighth go back while the
    // threshold pass computes (at 512^3, two paired runs put eight 1.7 and 16 ms
    // ahead of four, within the run-to-run spread of e2e on one host, and
    // sixteen behind both)
    FhbDownloads dl{ cs, ctx->ev_a, host, 8, false, ctx->ev_state };
    run_find_HII_bubbles(ctx, snapshot, &m, out, s, &dl);
    launches += out ? out->gpu_launches : 0;
    if (b21) {
      run_delta_T(ctx, snapshot, &m, out, s);
      launches += out ? out->gpu_launches : 0;
    }
    if (dl.done) {
      std::vector<FieldIO> rest;
      for (const FieldIO& f : late_out)
        if (std::find(std::begin(SLAB_OUTPUTS), std::end(SLAB_OUTPUTS), f.member) == std::end(SLAB_OUTPUTS))
          rest.push_back(f);
      late_out.swap(rest);
    }
    copy_fields(ctx, host, late_out, OUT, s);
    MX_CUDA(cudaStreamSynchronize(cs));
    MX_CUDA(cudaStreamSynchronize(s));
    if (out)
      out->gpu_launches = launches;
  });
}

}  // extern "C"

// =================================================================== batch
// mx_batch_*: independent boxes on a pool of host threads, each with its own
// contexts and streams (include/mx_reion.h).
namespace {
// The configuration a context is built for: the item's parameters with
// those a context takes per item (the X-ray parameters) cleared.
mx_params batch_key(const mx_params& p)
{
  mx_params k;
  std::memcpy(&k, &p, sizeof(k));
  k.lx_gal = 0.0;
  k.nu_xray_gal_threshold = 0.0;
  return k;
}

struct BatchWorker
{
  mx_ctx* ctx = nullptr;
  mx_params key{};
};
}  // namespace

struct mx_batch
{
  std::string tables_dir;
  size_t max_work_bytes = 0;
  int device = 0;
  std::vector<BatchWorker> workers;
  // mx_batch_run_graph: one context per item position, and the stream the
  // batch graph is captured and launched on
  std::vector<BatchWorker> gctx;
  cudaStream_t gstream = nullptr;
  cudaEvent_t gfork = nullptr;
  std::mutex mu;
  std::string err;
  int err_item = -1;

  void fail(int item, const std::string& msg)
  {
    std::lock_guard<std::mutex> lk(mu);
    if (err_item < 0 || item < err_item) {
      err_item = item;
      err = "item " + std::to_string(item) + ": " + msg;
    }
  }

  // The worker's context for the item's configuration: kept (with the
  // previous box's history cleared and the item's X-ray parameters) or
  // created.  False (status and error set) if creation failed.
  bool prepare(BatchWorker& w, mx_batch_item& it, int index)
  {
    const mx_params key = batch_key(*it.params);
    if (w.ctx && std::memcmp(&key, &w.key, sizeof(key)) == 0) {
      // same configuration: clear the previous box's history
      std::memset(w.ctx->stored_fcoll, 0, sizeof(w.ctx->stored_fcoll));
      w.ctx->lc_length = -1;
      w.ctx->lc_pos = 0;
      w.ctx->lc_end_snapshot = 0;
      w.ctx->p.lx_gal = it.params->lx_gal;
      w.ctx->p.nu_xray_gal_threshold = it.params->nu_xray_gal_threshold;
    } else {
      if (w.ctx) {
        mx_destroy(w.ctx);
        w.ctx = nullptr;
      }
      const double D = it.params->grid_dim;
      const size_t cap = max_work_bytes ? max_work_bytes : (size_t)(200.0 * D * D * (D / 2 + 16));
      const int rc = create_ctx(it.params, tables_dir.c_str(), cap, &w.ctx);
      if (rc != MX_OK) {
        it.status = rc;
        fail(index, g_create_error);
        w.ctx = nullptr;
        return false;
      }
      w.key = key;
    }
    return true;
  }

  void run_item(BatchWorker& w, mx_batch_item& it, int index)
  {
    if (!prepare(w, it, index))
      return;
    int rc = mx_set_redshifts(w.ctx, it.redshifts, it.n_snaps);
    mx_globals scratch{};
    if (rc == MX_OK)
      rc = mx_step(w.ctx, it.snapshot, it.grids, it.out ? it.out : &scratch);
    it.status = rc;
    if (rc != MX_OK)
      fail(index, w.ctx->err);
  }
};

extern "C" {

int mx_batch_create(const char* tables_dir, int32_t max_workers, size_t max_work_bytes, mx_batch** out)
{
  if (!out || max_workers < 0)
    return MX_EINVAL;
  *out = nullptr;
  std::unique_ptr<mx_batch> b(new (std::nothrow) mx_batch());
  if (!b)
    return MX_ENOMEM;
  if (cudaGetDevice(&b->device) != cudaSuccess)
    return MX_ECUDA;
  b->tables_dir = tables_dir ? tables_dir : "";
  b->max_work_bytes = max_work_bytes;
  b->workers.resize(max_workers > 0 ? max_workers : 8);
  *out = b.release();
  return MX_OK;
}

void mx_batch_destroy(mx_batch* b)
{
  if (!b)
    return;
  cudaSetDevice(b->device);
  for (BatchWorker& w : b->workers)
    if (w.ctx)
      mx_destroy(w.ctx);
  for (BatchWorker& w : b->gctx)
    if (w.ctx)
      mx_destroy(w.ctx);
  if (b->gfork)
    cudaEventDestroy(b->gfork);
  if (b->gstream)
    cudaStreamDestroy(b->gstream);
  delete b;
}

const char* mx_batch_last_error(const mx_batch* b) { return b ? b->err.c_str() : "mx_batch: NULL batch"; }

int mx_batch_run(mx_batch* b, mx_batch_item* items, int32_t n_items)
{
  if (!b)
    return MX_EINVAL;
  b->err.clear();
  b->err_item = -1;
  if (n_items < 0 || (n_items > 0 && !items)) {
    b->err = "mx_batch_run: bad item list";
    return MX_EINVAL;
  }
  for (int i = 0; i < n_items; i++)
    if (!items[i].params || !items[i].redshifts || !items[i].grids) {
      b->err = "item " + std::to_string(i) + ": NULL params, redshifts or grids";
      items[i].status = MX_EINVAL;
      return MX_EINVAL;
    }
  if (n_items == 0)
    return MX_OK;
  // groups of equal configurations, in order of their first item
  std::vector<mx_params> gkeys;
  std::vector<std::vector<int>> groups;
  for (int i = 0; i < n_items; i++) {
    const mx_params k = batch_key(*items[i].params);
    size_t g = 0;
    while (g < gkeys.size() && std::memcmp(&gkeys[g], &k, sizeof(k)) != 0)
      g++;
    if (g == gkeys.size()) {
      gkeys.push_back(k);
      groups.emplace_back();
    }
    groups[g].push_back(i);
  }
  // workers per group in proportion to its items (at least one each, at
  // most its items); a worker already holding a group's configuration stays
  // with that group
  const int W = (int)b->workers.size();
  const int G = (int)groups.size();
  std::vector<int> want(G);
  for (int g = 0; g < G; g++)
    want[g] = std::max(1, std::min((int)groups[g].size(), (int)((double)W * groups[g].size() / n_items)));
  std::vector<std::vector<int>> gw(G);  // worker slots of each group
  std::vector<bool> used(W, false);
  for (int g = 0; g < G; g++)
    for (int w = 0; w < W && (int)gw[g].size() < want[g]; w++)
      if (!used[w] && b->workers[w].ctx && std::memcmp(&b->workers[w].key, &gkeys[g], sizeof(mx_params)) == 0) {
        gw[g].push_back(w);
        used[w] = true;
      }
  for (int g = 0; g < G; g++)
    for (int w = 0; w < W && (int)gw[g].size() < want[g]; w++)
      if (!used[w]) {
        gw[g].push_back(w);
        used[w] = true;
      }
  // workers left over go, one at a time, to the group with the most items
  // per worker
  for (int w = 0; w < W; w++) {
    if (used[w])
      continue;
    int best = -1;
    double most = 1.0;
    for (int g = 0; g < G; g++) {
      const double per = gw[g].empty() ? 1e30 : (double)groups[g].size() / gw[g].size();
      if (per > most) {
        most = per;
        best = g;
      }
    }
    if (best < 0)
      break;
    gw[best].push_back(w);
    used[w] = true;
  }
  // more groups than workers: the groups without a worker go to the workers
  // in turn (run after that worker's own group)
  std::vector<std::vector<int>> queue(W);
  std::vector<std::atomic<int>> next(G);
  for (int g = 0; g < G; g++)
    next[g] = 0;
  std::vector<std::vector<int>> wgroups(W);  // groups a worker serves, in order
  int spill = 0;
  for (int g = 0; g < G; g++) {
    if (gw[g].empty())
      gw[g].push_back(spill++ % W);
    for (int w : gw[g])
      wgroups[w].push_back(g);
  }
  auto work = [&](int w) {
    cudaSetDevice(b->device);
    for (int g : wgroups[w])
      for (int j = next[g]++; j < (int)groups[g].size(); j = next[g]++)
        b->run_item(b->workers[w], items[groups[g][j]], groups[g][j]);
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < W; w++)
    if (!wgroups[w].empty())
      pool.emplace_back(work, w);
  for (std::thread& th : pool)
    th.join();
  for (int i = 0; i < n_items; i++)
    if (items[i].status != MX_OK)
      return items[i].status;
  return MX_OK;
}

namespace {
bool host_pinned(const void* p)
{
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// The grids a step reads from the host (inputs not written by an earlier
// stage of the step) and writes back, in the order ComputeTs,
// find_HII_bubbles, brightness temperature (as mx_step).
void step_copy_lists(const mx_params& p, std::vector<FieldIO>* in, std::vector<FieldIO>* out)
{
  std::vector<const std::vector<FieldIO>*> lists;
  if (p.flag_spin_temp)
    lists.push_back(&ts_fields());
  lists.push_back(&fhb_fields());
  if (p.flag_21cm)
    lists.push_back(&dt_fields());
  auto has = [](const std::vector<FieldIO>& v, float* mx_grids::*m) {
    for (const FieldIO& f : v)
      if (f.member == m)
        return true;
    return false;
  };
  for (const std::vector<FieldIO>* l : lists)
    for (const FieldIO& f : *l) {
      if ((f.dir & IN) && !has(*out, f.member) && !has(*in, f.member))
        in->push_back({ f.member, f.padded, IN });
      if ((f.dir & OUT) && !has(*out, f.member))
        out->push_back({ f.member, f.padded, OUT });
    }
}
}  // namespace

int mx_batch_run_graph(mx_batch* b, mx_batch_item* items, int32_t n_items)
{
  if (!b)
    return MX_EINVAL;
  b->err.clear();
  b->err_item = -1;
  if (n_items < 0 || (n_items > 0 && !items)) {
    b->err = "mx_batch_run_graph: bad item list";
    return MX_EINVAL;
  }
  for (int i = 0; i < n_items; i++) {
    if (!items[i].params || !items[i].redshifts || !items[i].grids) {
      b->err = "item " + std::to_string(i) + ": NULL params, redshifts or grids";
      items[i].status = MX_EINVAL;
      return MX_EINVAL;
    }
    items[i].status = MX_OK;
  }
  if (n_items == 0)
    return MX_OK;
  if (cudaSetDevice(b->device) != cudaSuccess) {
    b->err = "mx_batch_run_graph: cudaSetDevice failed";
    return MX_ECUDA;
  }
  if (!b->gstream) {
    if (cudaStreamCreateWithFlags(&b->gstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->gfork, cudaEventDisableTiming) != cudaSuccess) {
      b->err = "mx_batch_run_graph: stream creation failed";
      return MX_ECUDA;
    }
  }
  // contexts, redshifts, device mirrors and cuFFT plans: everything that
  // allocates, before the capture
  if ((int)b->gctx.size() < n_items)
    b->gctx.resize(n_items);
  std::vector<std::vector<FieldIO>> ins(n_items), outs(n_items);
  for (int i = 0; i < n_items; i++) {
    mx_batch_item& it = items[i];
    BatchWorker& w = b->gctx[i];
    if (!b->prepare(w, it, i))
      return it.status;
    mx_ctx* c = w.ctx;
    const int rc = guarded(c, [&]() {
      if (mx_set_redshifts(c, it.redshifts, it.n_snaps) != MX_OK)
        throw CudaError{ MX_EINVAL, c->err };
      check_snapshot(c, it.snapshot);
      c->ensure_mirror();
      if (!c->fused_fft) {
        c->c2r_plan(n_fields(c->p));
        if (c->p.flag_spin_temp)
          c->c2r_plan(1);
      }
      if (c->p.flag_spin_temp && c->p.flag_pecvel > 0)
        c->c2r_plan(1);
      step_copy_lists(c->p, &ins[i], &outs[i]);
      const mx_grids* h = it.grids;
      float* mx_grids::*all[] = { &mx_grids::deltax,   &mx_grids::stars,        &mx_grids::weighted_sfr,
                                  &mx_grids::sfr,      &mx_grids::sfr_histories, &mx_grids::N_rec,
                                  &mx_grids::x_e_box,  &mx_grids::x_e_box_prev, &mx_grids::Tk_box,
                                  &mx_grids::TS_box,   &mx_grids::xH,           &mx_grids::z_at_ionization,
                                  &mx_grids::r_bubble, &mx_grids::J_21,         &mx_grids::J_21_at_ionization,
                                  &mx_grids::Gamma12,  &mx_grids::delta_T,      &mx_grids::vel };
      for (auto m : all)
        if (h->*m && !host_pinned(h->*m))
          throw CudaError{ MX_EINVAL, "a host grid is not page-locked (the graph's copies need pinned memory)" };
    });
    if (rc != MX_OK) {
      it.status = rc;
      b->fail(i, c->err);
      return rc;
    }
  }
  // one capture: each item's copies in, step and copies out on its own
  // context stream, forked from and joined to the batch stream
  cudaGraph_t graph = nullptr;
  std::vector<mx_globals> scratch(n_items);
  std::vector<int> launches(n_items, 0);
  int failed = -1;
  std::string msg;
  if (cudaStreamBeginCapture(b->gstream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    b->err = "mx_batch_run_graph: capture could not begin";
    return MX_ECUDA;
  }
  try {
    MX_CUDA(cudaEventRecord(b->gfork, b->gstream));
    for (int i = 0; i < n_items; i++) {
      failed = i;
      mx_batch_item& it = items[i];
      mx_ctx* c = b->gctx[i].ctx;
      mx_globals* o = it.out ? it.out : &scratch[i];
      cudaStream_t s = c->stream;
      MX_CUDA(cudaStreamWaitEvent(s, b->gfork, 0));
      c->capturing = true;
      c->stage_used = 0;
      c->finishers.clear();
      c->graph_keep.clear();
      copy_fields(c, it.grids, ins[i], IN, s);
      if (c->p.flag_spin_temp)
        copy_histories(c, it.grids, s);
      mx_grids m = mirror_for(c, it.grids);
      if (c->p.flag_spin_temp) {
        run_ComputeTs(c, it.snapshot, &m, o, s);
        launches[i] += o->gpu_launches;
      }
      run_find_HII_bubbles(c, it.snapshot, &m, o, s);
      launches[i] += o->gpu_launches;
      if (c->p.flag_21cm) {
        run_delta_T(c, it.snapshot, &m, o, s);
        launches[i] += o->gpu_launches;
      }
      copy_fields(c, it.grids, outs[i], OUT, s);
      MX_CUDA(cudaEventRecord(c->ev_state, s));
      MX_CUDA(cudaStreamWaitEvent(b->gstream, c->ev_state, 0));
      c->capturing = false;
    }
    failed = -1;
  } catch (const CudaError& e) {
    msg = e.msg;
  } catch (const std::exception& e) {
    msg = e.what();
  }
  for (int i = 0; i < n_items; i++)
    if (b->gctx[i].ctx)
      b->gctx[i].ctx->capturing = false;
  const cudaError_t ec = cudaStreamEndCapture(b->gstream, &graph);
  if (failed >= 0 || ec != cudaSuccess) {
    if (graph)
      cudaGraphDestroy(graph);
    if (failed < 0) {
      failed = 0;
      msg = std::string("batch graph capture: ") + cudaGetErrorString(ec);
    }
    for (int i = 0; i < n_items; i++) {
      items[i].status = MX_ECUDA;
      if (b->gctx[i].ctx) {
        b->gctx[i].ctx->finishers.clear();
        b->gctx[i].ctx->graph_keep.clear();
      }
    }
    b->fail(failed, msg);
    return MX_ECUDA;
  }
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e == cudaSuccess)
    e = cudaGraphLaunch(exec, b->gstream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(b->gstream);
  if (exec)
    cudaGraphExecDestroy(exec);
  // each item's reads back, error checks and globals
  for (int i = 0; i < n_items; i++) {
    mx_ctx* c = b->gctx[i].ctx;
    std::vector<std::function<void()>> fin;
    fin.swap(c->finishers);
    c->graph_keep.clear();
    if (e != cudaSuccess) {
      items[i].status = MX_ECUDA;
      b->fail(i, std::string("batch graph: ") + cudaGetErrorString(e));
      continue;
    }
    const int rc = guarded(c, [&]() {
      for (auto& f : fin)
        f();
    });
    c->stage_used = 0;
    items[i].status = rc;
    if (rc != MX_OK)
      b->fail(i, c->err);
    else if (items[i].out)
      items[i].out->gpu_launches = launches[i];
  }
  for (int i = 0; i < n_items; i++)
    if (items[i].status != MX_OK)
      return items[i].status;
  return MX_OK;
}

}  // extern "C"
