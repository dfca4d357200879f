/*
 * mx_reion.h — C ABI of the GB300 reionization grid step.
 *
 * This library replaces, for one process owning the whole box on one GPU, the
 * three per-snapshot entry points of the Meraxes reionization step:
 *
 *   void find_HII_bubbles(int snapshot, timer_info* timer_total);
 *        reference: src/core/find_HII_bubbles.h:12, body find_HII_bubbles.c:47-532
 *   void ComputeTs(int snapshot, timer_info* timer_total);
 *        reference: src/core/ComputeTs.h:13, body ComputeTs.c:78-1045
 *   void ComputeBrightnessTemperatureBox(int snapshot);
 *        reference: src/core/BrightnessTemperature.h:9, body BrightnessTemperature.c:24-549
 *
 * The reference reads everything from the global `run_globals`; this ABI takes
 * the same data explicitly: the run parameters (mx_params, the subset of
 * run_params_t / physics_params_t / run_units_t the step reads), the snapshot
 * redshift list (run_globals.ZZ), and the grids (mx_grids, the
 * run_globals.reion_grids fields) in the reference's own memory layouts:
 *
 *   PADDED  float[D][D][2(D/2+1)]  (FFTW in-place r2c layout; misc_tools.c:205)
 *   REAL    float[D][D][D]                                     (misc_tools.c:208)
 *
 * Every entry point returns 0 on success or a negative MX_E* code; the text of
 * the last error on a context is returned by mx_last_error().  No C++
 * exception crosses this boundary and nothing calls exit().
 *
 * Two families of calls:
 *   mx_<step>(...)          grids are HOST pointers; inputs are copied to the
 *                           device, outputs copied back (what the reference's
 *                           C driver needs as a drop-in).
 *   mx_<step>_device(...)   grids are DEVICE pointers owned by the caller; no
 *                           host copies; work is ordered on `stream`
 *                           (a cudaStream_t, or NULL for the context stream).
 */
#ifndef MX_REION_H
#define MX_REION_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MX_ABI_VERSION 1

/* Status codes. */
#define MX_OK 0
#define MX_EINVAL (-1)   /* invalid parameter / argument */
#define MX_ENOMEM (-2)   /* device or host allocation failed */
#define MX_ECUDA (-3)    /* CUDA runtime or cuFFT error */
#define MX_ETABLE (-4)   /* physics table missing or unreadable */
#define MX_ESTATE (-5)   /* call order / snapshot list error */
#define MX_ENOTSUP (-6)  /* configuration not supported */

/* Run parameters read by the step.  Field names follow the reference's
 * parameter names (src/meraxes.h run_params_t / physics_params_t / run_units_t;
 * defaults in input/params/defaults.par). */
typedef struct mx_params
{
  int32_t grid_dim; /* ReionGridDim */
  int32_t abi_version; /* must be MX_ABI_VERSION */
  double box_size;  /* BoxSize [Mpc/h] */

  /* cosmology */
  double hubble_h;     /* Hubble_h */
  double omega_m;      /* OmegaM */
  double omega_lambda; /* OmegaLambda */
  double omega_r;      /* OmegaR */
  double omega_k;      /* OmegaK */
  double baryon_frac;  /* BaryonFrac */
  double w_lambda;     /* wLambda */

  /* units */
  double unit_length_cm;     /* UnitLength_in_cm */
  double unit_mass_g;        /* UnitMass_in_g */
  double unit_velocity_cm_s; /* UnitVelocity_in_cm_per_s */

  /* switches */
  int32_t flag_recombinations;    /* Flag_IncludeRecombinations */
  int32_t flag_spin_temp;         /* Flag_IncludeSpinTemp */
  int32_t flag_21cm;              /* Flag_Compute21cmBrightTemp */
  int32_t flag_pecvel;            /* Flag_IncludePecVelsFor21cm (0..3) */
  int32_t uvb_flag;               /* ReionUVBFlag */
  int32_t filter_type;            /* ReionFilterType: 0 tophat, 1 sharp-k, 2 Gaussian */
  int32_t rtom_filter_type;       /* ReionRtoMFilterType: 0 tophat, 1 Gaussian */
  int32_t ts_heating_filter_type; /* TsHeatingFilterType */
  int32_t ts_num_filter_steps;    /* TsNumFilterSteps */
  int32_t trees_id;               /* TreesID: velocity unit convention */

  /* excursion set */
  double delta_r_factor;      /* ReionDeltaRFactor */
  double r_bubble_min;        /* ReionRBubbleMin [Mpc/h] */
  double r_bubble_max;        /* ReionRBubbleMax [Mpc/h] */
  double r_bubble_max_recomb; /* ReionRBubbleMaxRecomb [Mpc/h] */
  double reion_efficiency;    /* physics.ReionEfficiency (as set by set_ReionEfficiency) */
  double nion_phot_per_bary;  /* ReionNionPhotPerBary */
  double gamma_halo_bias;     /* ReionGammaHaloBias */
  double alpha_uv;            /* ReionAlphaUV */
  double y_he;                /* Y_He */

  /* X-ray heating / spin temperature */
  double max_heating_redshift;  /* ReionMaxHeatingRedshift */
  double lx_gal;                /* LXrayGal [erg/s per Msun/yr] */
  double nu_xray_gal_threshold; /* NuXrayGalThreshold [eV] */
  double spec_index_xray_gal;   /* SpecIndexXrayGal */
  double nu_xray_soft_cut;      /* NuXraySoftCut [eV] */
  double nu_xray_max;           /* NuXrayMax [eV] */
  double reion_sfr_timescale;   /* ReionSfrTimescale (construct_baryon_grids) */
  double clumping_factor;       /* x_e sink clumping; the reference hard-codes
                                   CLUMPING_FACTOR = 2 (XRayHeatingFunctions.h:30-32) */
} mx_params;

/* Grid pointers (all HOST or all DEVICE, depending on the call family).
 * Fields the configuration does not use may be NULL. */
typedef struct mx_grids
{
  float* deltax;       /* PADDED, in */
  float* stars;        /* PADDED, in */
  float* weighted_sfr; /* PADDED, in */
  float* sfr;          /* PADDED, in; reweighted in place by ComputeTs like the reference */
  float* sfr_histories; /* n_sfr_histories slices of 2*D*D*(D/2+1) floats, in */
  float* N_rec;        /* PADDED, in/out (recombinations) */
  float* x_e_box;      /* PADDED, in (find_HII_bubbles) / out (ComputeTs) */
  float* x_e_box_prev; /* PADDED, in/out (ComputeTs) */
  float* Tk_box;       /* REAL, in/out (ComputeTs) */
  float* TS_box;       /* REAL, out (ComputeTs) */
  float* xH;           /* REAL, out */
  float* z_at_ionization;    /* REAL, in/out (init to -1) */
  float* r_bubble;           /* REAL, out */
  float* J_21;               /* REAL, out (UVB) */
  float* J_21_at_ionization; /* REAL, in/out (UVB) */
  float* Gamma12;            /* REAL, in/out (recombinations) */
  float* delta_T;            /* REAL, out (21cm) */
  float* vel;                /* PADDED, in; converted in place like the reference */
} mx_grids;

/* Global scalars written by the step (run_globals.reion_grids.* and the
 * file-scope globals of XRayHeatingFunctions.c). */
typedef struct mx_globals
{
  double volume_weighted_global_xH;   /* find_HII_bubbles.c:492 */
  double volume_weighted_global_J_21; /* find_HII_bubbles.c:493 */
  double mass_weighted_global_xH;     /* find_HII_bubbles.c:494 */
  double volume_ave_J_alpha;          /* ComputeTs.c:926 */
  double volume_ave_xalpha;
  double volume_ave_Xheat;
  double volume_ave_Xion;
  double volume_ave_TS;   /* ComputeTs.c:972 */
  double volume_ave_TK;
  double volume_ave_xe;   /* as the reference computes it (ComputeTs.c:957) */
  double volume_ave_Tb;   /* BrightnessTemperature.c:545 */
  double x_e_ave;         /* cell mean of x_e_box_prev (ComputeTs.c:475) */
  double collapse_fraction; /* stored_fcoll[snapshot] (ComputeTs.c:468) */
  int32_t n_radii;        /* filter radii used by find_HII_bubbles */
  int32_t gpu_launches;   /* kernels launched by the last call */
} mx_globals;

typedef struct mx_ctx mx_ctx;

/* Context lifetime.  `tables_dir` is the directory holding the 21cmFAST
 * tables (recfast_LCDM.dat, stellar_spectra.dat, kappa_*_table.dat,
 * x_int_tables/); it is only read when flag_spin_temp is set.  The context
 * owns all device scratch, cuFFT plans and physics tables. */
int mx_create(const mx_params* params, const char* tables_dir, mx_ctx** out);
/* mx_create with the transform work buffer capped at max_work_bytes (it
 * holds at least the fields of one filter radius), for several contexts on
 * one GPU, e.g. a batch of independent boxes.  mx_create takes up to 45% of
 * the free device memory for it.  No reference counterpart. */
int mx_create_limited(const mx_params* params, const char* tables_dir, size_t max_work_bytes, mx_ctx** out);
void mx_destroy(mx_ctx* ctx);

/* ---------------------------------------------------------------------------
 * Batch of independent boxes (no reference counterpart: the reference runs one
 * box per process).  Each item is one box's mx_step: its own configuration
 * (grid size, physics, X-ray parameters), redshift list, snapshot and host
 * grids (updated in place as by mx_step).
 *
 * A batch object owns up to max_workers workers (0: 8), each with its own
 * contexts (mx_create_limited with max_work_bytes; 0: 200 D^2 (D/2 + 16)
 * bytes, about 25 spectra) and CUDA stream.  mx_batch_run steps every item on
 * concurrent host threads, so the boxes' kernels overlap on the GPU.  Items
 * of one configuration (the parameters apart from lx_gal and
 * nu_xray_gal_threshold) form a group; the workers are split over the groups
 * in proportion to their items, and a group's items go to its workers in
 * turn.  A worker keeps its context between items and between runs while the
 * configuration stays the same, clearing the per-box history (collapse
 * fractions of earlier snapshots, light cone) and setting the item's
 * redshifts and X-ray parameters before each item.  An item's result does not
 * depend on the packing.  mx_batch_run returns MX_OK when every item
 * succeeded, else the code of the first failed item (in item order);
 * items[i].status holds each item's code and mx_batch_last_error the first
 * failure's message.  One mx_batch_run at a time per batch object.
 * ------------------------------------------------------------------------- */
typedef struct mx_batch_item
{
  const mx_params* params;
  const double* redshifts; /* run_globals.ZZ of the box */
  int32_t n_snaps;
  int32_t snapshot;
  const mx_grids* grids;   /* host pointers */
  mx_globals* out;         /* may be NULL */
  int32_t status;          /* written by mx_batch_run */
} mx_batch_item;

typedef struct mx_batch mx_batch;
int mx_batch_create(const char* tables_dir, int32_t max_workers, size_t max_work_bytes, mx_batch** out);
int mx_batch_run(mx_batch* batch, mx_batch_item* items, int32_t n_items);
/* The same items as ONE CUDA graph, launched once: every item has its own
 * context (kept between runs while its position's configuration stays the
 * same, with the per-box history cleared); one capture puts each item's
 * host->device copies, its step (ComputeTs -> find_HII_bubbles -> 21cm box,
 * with the frequency tables built by a host node) and its device->host copies
 * on a branch of the graph, and a single cudaGraphLaunch runs every box.  The
 * host grids must be page-locked (cudaHostAlloc / cudaHostRegister), as the
 * graph's copy nodes need pinned memory; other grids return MX_EINVAL.
 * Results equal those of mx_step per box.  No reference counterpart (the
 * reference runs one box per MPI job). */
int mx_batch_run_graph(mx_batch* batch, mx_batch_item* items, int32_t n_items);
void mx_batch_destroy(mx_batch* batch);
const char* mx_batch_last_error(const mx_batch* batch);
const char* mx_last_error(const mx_ctx* ctx); /* ctx may be NULL: last mx_create error */

/* run_globals.ZZ: redshift of every snapshot (descending).  Also computes the
 * number of stored SFR-history slices (set_sfr_history, ComputeTs.c:32-76). */
int mx_set_redshifts(mx_ctx* ctx, const double* zz, int32_t n_snaps);
int32_t mx_n_sfr_histories(const mx_ctx* ctx);
/* Threads per block that the context's autotuner chose for the x- and
 * y-pass of its fused inverse transforms (256 or 512; 0 and 0 when the grid
 * uses cuFFT).  No reference counterpart. */
int mx_fft_block_sizes(const mx_ctx* ctx, int32_t* x_threads, int32_t* y_threads);
/* Resident blocks per SM that the context's autotuner budgeted the threshold
 * z-pass's registers for (2 or 3; 0 when the grid does not run that kernel).
 * No reference counterpart. */
int32_t mx_zpass_blocks_per_sm(const mx_ctx* ctx);
/* Filter radii of find_HII_bubbles for this configuration (largest first). */
int32_t mx_filter_radii(const mx_ctx* ctx, double* radii, int32_t cap);

/* Host-pointer entry points (drop-in for the reference functions). */
int mx_find_HII_bubbles(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out);
int mx_ComputeTs(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out);
int mx_ComputeBrightnessTemperatureBox(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out);
/* ComputeTs (if spin temperature) -> find_HII_bubbles -> brightness
 * temperature (if flag_21cm), the order of dracarys.c:352-390. */
int mx_step(mx_ctx* ctx, int32_t snapshot, const mx_grids* host, mx_globals* out);

/* Device-pointer entry points.  Every non-NULL grid pointer must be 8-byte
 * aligned (cuFFT's requirement for its real inputs; cudaMalloc and
 * fftwf_malloc give 256 and 16 bytes); other pointers return MX_EINVAL. */
int mx_find_HII_bubbles_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream);
int mx_ComputeTs_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream);
int mx_ComputeBrightnessTemperatureBox_device(mx_ctx* ctx,
                                              int32_t snapshot,
                                              const mx_grids* dev,
                                              mx_globals* out,
                                              void* stream);
int mx_step_device(mx_ctx* ctx, int32_t snapshot, const mx_grids* dev, mx_globals* out, void* stream);
/* With on != 0, each later mx_step_device call captures the whole step
 * (ComputeTs, find_HII_bubbles, the 21cm box) into one CUDA graph on the
 * context's stream and launches it on `stream`; ComputeTs's frequency tables
 * are built by a host node of the graph while the shells are smoothed.  The
 * grids and globals equal those of the uncaptured step bit for bit.  Each
 * call captures anew (kernel arguments depend on the snapshot); per-kernel
 * profiling records its events as event nodes of the graph.  No reference
 * counterpart (the reference runs the three calls from the dracarys loop). */
int mx_set_step_graph(mx_ctx* ctx, int32_t on);

/* Per-kernel timing with CUDA events recorded on the launching stream around
 * every kernel and cuFFT execution of the context.  No reference counterpart
 * (the reference times whole calls with gettimeofday, utils.c:9-24).
 * mx_profile_enable(ctx, 1) clears and starts collection; mx_profile_read
 * synchronises the context stream, then fills up to `cap` entries (one per
 * kernel name) and returns the number of distinct names. */
typedef struct mx_kernel_stat
{
  char name[40];
  int32_t launches;
  double ms;    /* summed event time */
  double bytes; /* summed algorithmic HBM bytes (reads + writes) */
} mx_kernel_stat;
int mx_profile_enable(mx_ctx* ctx, int32_t on);
int32_t mx_profile_read(mx_ctx* ctx, mx_kernel_stat* out, int32_t cap);

/* Light cone: Initialise_ConstructLightcone and ConstructLightcone
 * (src/core/ConstructLightcone.c:12-166, header ConstructLightcone.h).  The
 * reference keeps LightconeLength, EndSnapshotLightcone and CurrentLCPos in
 * run_globals.params and the boxes in run_globals.reion_grids; here the
 * context keeps the first three and the caller passes the arrays.
 * mx_lightcone_init(ctx, EndRedshiftLightcone, LastOutputSnap, &end) returns
 * LightconeLength (or a negative MX_E* code) and sets *end to
 * EndSnapshotLightcone; call it after mx_set_redshifts.
 * mx_ConstructLightcone is called for every snapshot in order, like the
 * reference: it fills the slices between ZZ[snapshot] and ZZ[snapshot-1] of
 * lightcone (float[D][D][LightconeLength], slice fastest: grid_index_LC,
 * misc_tools.c:222-229) by time interpolation between delta_T_prev and
 * delta_T (REAL grids), writes their redshifts into lightcone_redshifts
 * (float[LightconeLength], a HOST array in both variants), then copies
 * delta_T into delta_T_prev.  The _device variant takes device grids and a
 * device light cone. */
int64_t mx_lightcone_init(mx_ctx* ctx, double end_redshift, int32_t last_output_snap, int32_t* end_snapshot);
int mx_ConstructLightcone(mx_ctx* ctx,
                          int32_t snapshot,
                          const float* delta_T,
                          float* delta_T_prev,
                          float* lightcone,
                          float* lightcone_redshifts);
int mx_ConstructLightcone_device(mx_ctx* ctx,
                                 int32_t snapshot,
                                 const float* delta_T,
                                 float* delta_T_prev,
                                 float* lightcone,
                                 float* lightcone_redshifts,
                                 void* stream);

/* 21 cm power spectrum of a delta_T grid (REAL layout): Initialise_PowerSpectrum
 * and Compute_PS (src/core/ComputePowerSpectrum.c:18-255, header
 * ComputePowerSpectrum.h:9-10).  The reference writes
 * run_globals.reion_grids.PS_k / PS_data / PS_error; here the caller passes
 * three host arrays of at least mx_ps_length(ctx) floats.  Bins: ratio 1.35
 * from 2 pi / (BoxSize / h) up to D times that; every half-spectrum mode is
 * counted once.  Returns the number of bins, or a negative MX_E* code.
 * mx_Compute_PS takes a host grid; _device a device grid on `stream`. */
int32_t mx_ps_length(const mx_ctx* ctx);
int mx_Compute_PS(mx_ctx* ctx, const float* delta_T, float* ps_k, float* ps_data, float* ps_error, int32_t cap);
int mx_Compute_PS_device(mx_ctx* ctx,
                         const float* delta_T,
                         float* ps_k,
                         float* ps_data,
                         float* ps_error,
                         int32_t cap,
                         void* stream);

/* Galaxy properties read by construct_baryon_grids, one entry per galaxy of
 * the snapshot in the reference's galaxy-list order (map_galaxies_to_slabs,
 * reionization.c:1109-1161, sorts the gal_to_slab_t map stably; one rank).
 * Field names follow galaxy_t (src/meraxes.h).  gross_stellar_mass is read
 * only with the spin temperature, black_hole_mass and effective_bhm only with
 * BH feedback; the others may be NULL then. */
typedef struct mx_galaxies
{
  int64_t n;
  const float* pos;                  /* Pos, float[n][3], Mpc/h */
  const int32_t* type;               /* Type; galaxies of Type > 2 are skipped */
  const double* fesc_weighted_gsm;   /* FescWeightedGSM */
  const double* gross_stellar_mass;  /* GrossStellarMass */
  const double* black_hole_mass;     /* BlackHoleMass */
  const double* effective_bhm;       /* EffectiveBHM */
} mx_galaxies;

/* Galaxy -> grid deposit: construct_baryon_grids(snapshot, local_ngals)
 * (src/core/reionization.c:1353-1615, declared reionization.h:66; one rank,
 * no mini-haloes).  Writes grids->stars and grids->weighted_sfr (PADDED) and,
 * with the spin temperature, grids->sfr and the newest slice of
 * grids->sfr_histories after shifting the older slices back by one, like the
 * reference.  Each galaxy goes to its nearest grid point (pos_to_ngp,
 * misc_tools.c:163-173); the cell sums are the reference's float sums in
 * galaxy order.  flag_bh_feedback, bh_limit and alpha_uv_bh are
 * physics.Flag_BHFeedback, BlackHoleMassLimitReion and ReionAlphaUVBH; the
 * SFR timescale is ReionSfrTimescale * hubble_time(snapshot).  A galaxy below
 * the box (a negative grid index, where the reference asserts) gives
 * MX_EINVAL; grids with 2^32 - 1 cells or more give MX_ENOTSUP.
 * mx_construct_baryon_grids takes HOST galaxy arrays and grids;
 * the _device variant takes DEVICE arrays (the double arrays 8-byte aligned)
 * and grids, orders the work on `stream` and waits for it before returning
 * (to report the error above).  The galaxy scratch (sort keys and CUB
 * storage) grows with the largest galaxy count seen. */
int mx_construct_baryon_grids(mx_ctx* ctx,
                              int32_t snapshot,
                              const mx_galaxies* galaxies,
                              int32_t flag_bh_feedback,
                              double bh_limit,
                              double alpha_uv_bh,
                              mx_grids* grids);
int mx_construct_baryon_grids_device(mx_ctx* ctx,
                                     int32_t snapshot,
                                     const mx_galaxies* galaxies,
                                     int32_t flag_bh_feedback,
                                     double bh_limit,
                                     double alpha_uv_bh,
                                     mx_grids* grids,
                                     void* stream);

/* Critical virial mass of UVB feedback per cell: calculate_Mvir_crit(redshift)
 * (src/physics/reionization.c:10-59, declared physics/reionization.h:11;
 * Sobacchi & Mesinger 2013b).  sm_params = {ReionSMParam_m0, _a, _b, _c, _d};
 * J_21_at_ionization, z_at_ionization and Mvir_crit are REAL grids; cells not
 * yet ionised at `redshift` get 0.  Computed in double per cell, like the
 * reference; pow is CUDA's, so a cell may differ from the reference's by one
 * float ulp.  Host grids for mx_calculate_Mvir_crit, device grids on `stream`
 * for the _device variant (which does not wait). */
int mx_calculate_Mvir_crit(mx_ctx* ctx,
                           double redshift,
                           const double sm_params[5],
                           const float* J_21_at_ionization,
                           const float* z_at_ionization,
                           float* Mvir_crit);
int mx_calculate_Mvir_crit_device(mx_ctx* ctx,
                                  double redshift,
                                  const double sm_params[5],
                                  const float* J_21_at_ionization,
                                  const float* z_at_ionization,
                                  float* Mvir_crit,
                                  void* stream);

/* ---------------------------------------------------------------------------
 * Differentiation (no counterpart in the reference's C code: the gradients of
 * a 21 cm power-spectrum loss through ComputeTs and the 21cm box, with the
 * ionisation flags of find_HII_bubbles held fixed).
 *
 * mx_set_xray_params sets LXrayGal and NuXrayGalThreshold (E0, eV) for the
 * following calls (the parameters a gradient is taken for).
 *
 * mx_ps_loss_device: L = sum_b (P_b - target_b)^2 over nbins bins
 * [edges[b], edges[b+1]) (1/Mpc, host arrays, increasing, edges[0] > 0) of
 * the power spectrum of f = delta_T * V / N (V = (BoxSize/h)^3), where
 * P_b = sum k^3 |F_k|^2 / (2 pi^2 V) / n_b over the half-spectrum modes of the
 * bin, each counted once (the binning of Compute_PS,
 * ComputePowerSpectrum.c:160-215).  Writes *loss, P[nbins] (host, may be
 * NULL) and, if grad_delta_T is not NULL, dL/d(delta_T) (device, REAL).
 *
 * mx_adjoint_device: the adjoint of ComputeTs (ComputeTs.c:78-1045, one
 * snapshot, not the homogeneous branch) and of the 21cm box without peculiar
 * velocities (BrightnessTemperature.c:495-545), given dL/d(delta_T).  `saved`
 * holds device grids of the forward step: deltax, stars (as find_HII_bubbles
 * read them), sfr (before ComputeTs reweighted it), sfr_histories,
 * x_e_box_prev and Tk_box (the state before the step), x_e_box, xH and TS_box
 * (after the step).  The 40 shells are recomputed, not stored.  xH enters
 * through the partial ionisation of the last, unfiltered step
 * (find_HII_bubbles.c:416-428) where 0 < xH < 1; the flags are fixed.
 * Outputs (device): grad_sfr (PADDED), grad_stars (PADDED), and grad_params
 * (host, 2 doubles) = {dL/dLXrayGal, dL/dNuXrayGalThreshold}.  The E0
 * derivative of the frequency tables is a central difference (relative step
 * 1e-3) of the host-built tables.
 * ------------------------------------------------------------------------- */
int mx_set_xray_params(mx_ctx* ctx, double lx_gal, double nu_xray_gal_threshold);
int mx_ps_loss_device(mx_ctx* ctx,
                      const float* delta_T,
                      int32_t nbins,
                      const float* edges,
                      const float* target,
                      double* loss,
                      float* P,
                      float* grad_delta_T,
                      void* stream);
int mx_adjoint_device(mx_ctx* ctx,
                      int32_t snapshot,
                      const mx_grids* saved,
                      const float* grad_delta_T,
                      float* grad_sfr,
                      float* grad_stars,
                      double* grad_params,
                      void* stream);

/* Build information: returns a static string. */
const char* mx_build_info(void);

/* Brightness-temperature box without any device allocation.  No counterpart
 * in the reference: it is the computation of
 * ComputeBrightnessTemperatureBox without peculiar velocities (constants
 * BrightnessTemperature.c:48-53, cell formula :82-124, volume average
 * :530-545) for callers that cannot allocate device memory.  The cell formula
 * runs in float (the reference rounds const_factor * xH * (1 + deltax) from
 * double once): a few ulp, inside the 1e-4 relative tolerance of delta_T.
 * Spin temperature together with flag_pecvel > 0 returns MX_ENOTSUP (the
 * peculiar-velocity modes need the context's transforms).  A host that keeps all its
 * grids resident has often given the rest of the GPU to its own pool.  A
 * thread that must not stall cannot call cudaMalloc/cudaFree, which may
 * synchronise the device.  No context is needed.  All pointers are device
 * pointers in the run_globals.reion_grids layouts (deltax PADDED, the others
 * REAL).  delta_T is written; *volume_ave_Tb (one device double) receives the
 * volume average.  The work is queued on `stream` and the call does not wait.
 *
 * Scratch: a fixed MX_NOALLOC_SCRATCH_BYTES __device__ array inside the
 * library, shared by every call on a device.  It holds one partial sum per
 * 16384 cells and a completion ticket that must be zero when a launch starts.
 * Each call zeroes the ticket on `stream` before its kernel.  Grids above
 * MX_NOALLOC_MAX_CELLS cells (512^3) are rejected with MX_EINVAL.  Calls that
 * overlap in time on one device (different streams or threads, not ordered
 * by the caller) race on that scratch and give wrong means: serialise them.
 * Each call outside stream capture looks up the scratch address on the
 * current device; a call on a capturing stream uses the address of the last
 * call outside capture on that device (MX_ESTATE if there was none), so make
 * the first call on a device, and the first after a cudaDeviceReset, before
 * any stream capture.  On error the message goes to errbuf (may be NULL). */
#define MX_NOALLOC_MAX_CELLS 134217728
#define MX_NOALLOC_SCRATCH_BYTES 65792
int mx_brightness_temperature_noalloc(const mx_params* params,
                                      double redshift,
                                      const float* deltax,
                                      const float* xH,
                                      const float* TS_box,
                                      float* delta_T,
                                      double* volume_ave_Tb,
                                      void* stream,
                                      char* errbuf,
                                      size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* MX_REION_H */
