/*
 * Implementations behind the shim headers in oracle/shims/ — TEST
 * INFRASTRUCTURE ONLY.  They let the reference's own C sources
 * (src/core/{find_HII_bubbles,ComputeTs,XRayHeatingFunctions,recombinations,
 * BrightnessTemperature,reionization,misc_tools,utils}.c) be compiled
 * unmodified into oracle/_ref/, with:
 *   FFTW  -> mx_numerics.c FFT (double internally, float in/out)
 *   GSL   -> mx_numerics.c natural cubic spline / QAG-GK61 / Brent
 *   MPI   -> a single rank
 */
#include <stdlib.h>
#include <string.h>

#include "fftw3-mpi.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_roots.h"
#include "gsl/gsl_spline.h"
#include "mpi.h"
#include "mx_numerics.h"

/* ---------------------------------------------------------------- FFTW */
struct mxs_fftwf_plan_s
{
  int D;
  int dir; /* -1 r2c, +1 c2r */
  void* in;
  void* out;
};

float* fftwf_alloc_real(size_t n) { return (float*)calloc(n ? n : 1, sizeof(float)); }
fftwf_complex* fftwf_alloc_complex(size_t n) { return (fftwf_complex*)calloc(n ? n : 1, sizeof(fftwf_complex)); }
void fftwf_free(void* p) { free(p); }
void fftwf_mpi_init(void) {}
void fftwf_mpi_cleanup(void) {}
void fftwf_mpi_broadcast_wisdom(MPI_Comm c) { (void)c; }
void fftwf_mpi_gather_wisdom(MPI_Comm c) { (void)c; }
int fftwf_import_wisdom_from_filename(const char* f) { (void)f; return 0; }
int fftwf_export_wisdom_to_filename(const char* f) { (void)f; return 0; }

ptrdiff_t fftwf_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm comm, ptrdiff_t* local_n0,
                                  ptrdiff_t* local_0_start)
{
  (void)comm;
  *local_n0 = n0;
  *local_0_start = 0;
  return n0 * n1 * n2;
}

static fftwf_plan mk_plan(ptrdiff_t n0, int dir, void* in, void* out)
{
  fftwf_plan p = (fftwf_plan)malloc(sizeof(*p));
  p->D = (int)n0;
  p->dir = dir;
  p->in = in;
  p->out = out;
  return p;
}
fftwf_plan fftwf_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, float* in, fftwf_complex* out,
                                     MPI_Comm comm, unsigned flags)
{
  (void)n1; (void)n2; (void)comm; (void)flags;
  return mk_plan(n0, -1, in, out);
}
fftwf_plan fftwf_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftwf_complex* in, float* out,
                                     MPI_Comm comm, unsigned flags)
{
  (void)n1; (void)n2; (void)comm; (void)flags;
  return mk_plan(n0, +1, in, out);
}
void fftwf_execute(const fftwf_plan p)
{
  if (p->dir < 0)
    mxo_r2c_3d(p->D, (const float*)p->in, 1, (float*)p->out); /* MPI r2c input is padded */
  else
    mxo_c2r_3d(p->D, (const float*)p->in, (float*)p->out);
}
void fftwf_destroy_plan(fftwf_plan p) { free(p); }

/* ----------------------------------------------------------------- MPI */
static size_t dt_size(MPI_Datatype dt) { return (size_t)(dt & 0xff); }
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm)
{
  (void)op; (void)comm;
  if (sendbuf != MPI_IN_PLACE)
    memcpy(recvbuf, sendbuf, (size_t)count * dt_size(dt));
  return 0;
}
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, int root, MPI_Comm comm)
{
  (void)root;
  return MPI_Allreduce(sendbuf, recvbuf, count, dt, op, comm);
}
int MPI_Bcast(void* buf, int count, MPI_Datatype dt, int root, MPI_Comm comm)
{
  (void)buf; (void)count; (void)dt; (void)root; (void)comm;
  return 0;
}
int MPI_Allgather(const void* sendbuf, int scount, MPI_Datatype sdt, void* recvbuf, int rcount, MPI_Datatype rdt,
                  MPI_Comm comm)
{
  (void)rcount; (void)rdt; (void)comm;
  memcpy(recvbuf, sendbuf, (size_t)scount * dt_size(sdt));
  return 0;
}
int MPI_Send(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm)
{
  (void)buf; (void)count; (void)dt; (void)dest; (void)tag; (void)comm;
  return 0;
}
int MPI_Recv(void* buf, int count, MPI_Datatype dt, int src, int tag, MPI_Comm comm, MPI_Status* st)
{
  (void)buf; (void)count; (void)dt; (void)src; (void)tag; (void)comm; (void)st;
  return 0;
}
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype sdt, int dest, int stag, void* rbuf, int rcount,
                 MPI_Datatype rdt, int src, int rtag, MPI_Comm comm, MPI_Status* st)
{
  (void)dest; (void)stag; (void)rcount; (void)rdt; (void)src; (void)rtag; (void)comm; (void)st;
  memcpy(rbuf, sbuf, (size_t)scount * dt_size(sdt));
  return 0;
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm comm, int* rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int* size) { (void)comm; *size = 1; return 0; }

/* ----------------------------------------------------------------- GSL */
gsl_error_handler_t* gsl_set_error_handler_off(void) { return NULL; }

gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n)
{
  gsl_integration_workspace* w = (gsl_integration_workspace*)malloc(sizeof(*w));
  w->limit = n;
  return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace* w) { free(w); }
int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs, double epsrel, size_t limit,
                        int key, gsl_integration_workspace* w, double* result, double* abserr)
{
  (void)key; /* every call site in the path uses GSL_INTEG_GAUSS61 */
  if (limit > w->limit)
    limit = w->limit;
  return mxo_qag61(f->function, f->params, a, b, epsabs, epsrel, limit, result, abserr);
}

static const gsl_interp_type cspline_type = { "cspline" };
const gsl_interp_type* gsl_interp_cspline = &cspline_type;
gsl_interp_accel* gsl_interp_accel_alloc(void) { return (gsl_interp_accel*)calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel* a) { free(a); }

struct mxs_gsl_spline
{
  mxo_spline s;
  size_t size;
};
gsl_spline* gsl_spline_alloc(const gsl_interp_type* T, size_t size)
{
  (void)T;
  gsl_spline* s = (gsl_spline*)calloc(1, sizeof(*s));
  s->size = size;
  return s;
}
int gsl_spline_init(gsl_spline* s, const double xa[], const double ya[], size_t size)
{
  if (s->s.x)
    mxo_spline_free(&s->s);
  return mxo_spline_init(&s->s, xa, ya, (int)size);
}
double gsl_spline_eval(const gsl_spline* s, double x, gsl_interp_accel* a)
{
  (void)a;
  return mxo_spline_eval(&s->s, x);
}
void gsl_spline_free(gsl_spline* s)
{
  if (!s)
    return;
  if (s->s.x)
    mxo_spline_free(&s->s);
  free(s);
}

static const gsl_root_fsolver_type brent_type = { "brent" };
const gsl_root_fsolver_type* gsl_root_fsolver_brent = &brent_type;
struct mxs_gsl_root_fsolver
{
  mxo_brent b;
};
gsl_root_fsolver* gsl_root_fsolver_alloc(const gsl_root_fsolver_type* T)
{
  (void)T;
  return (gsl_root_fsolver*)calloc(1, sizeof(gsl_root_fsolver));
}
int gsl_root_fsolver_set(gsl_root_fsolver* s, gsl_function* f, double x_lower, double x_upper)
{
  return mxo_brent_set(&s->b, f->function, f->params, x_lower, x_upper);
}
int gsl_root_fsolver_iterate(gsl_root_fsolver* s) { return mxo_brent_iterate(&s->b); }
double gsl_root_fsolver_root(const gsl_root_fsolver* s) { return s->b.root; }
double gsl_root_fsolver_x_lower(const gsl_root_fsolver* s) { return s->b.x_lower; }
double gsl_root_fsolver_x_upper(const gsl_root_fsolver* s) { return s->b.x_upper; }
void gsl_root_fsolver_free(gsl_root_fsolver* s) { free(s); }
int gsl_root_test_interval(double x_lower, double x_upper, double epsabs, double epsrel)
{
  return mxo_root_test_interval(x_lower, x_upper, epsabs, epsrel) == 0 ? GSL_SUCCESS : GSL_CONTINUE;
}

/* ------------------------------------------------------------------------
 * Functions referenced by the compiled reference files but outside the grid
 * step (galaxy I/O, debugging, exit quotes).  They are never reached by the
 * calls this oracle makes; reaching one is a driver bug, so they abort.
 * ---------------------------------------------------------------------- */
#include <stdio.h>
static void mxs_unreachable(const char* what)
{
  fprintf(stderr, "oracle/_ref: %s is outside the reionization grid step\n", what);
  abort();
}
void cleanup(void) { mxs_unreachable("cleanup"); }
void cn_quote(void) {}
void mpi_debug_here(void) { mxs_unreachable("mpi_debug_here"); }
void read_grid(int property, int snapshot, float* slab) { (void)property; (void)snapshot; (void)slab; mxs_unreachable("read_grid"); }
