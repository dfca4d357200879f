/*
 * CPU oracle of the reionization grid step — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-snapshot grid step
 * (find_HII_bubbles, ComputeTs, ComputeBrightnessTemperatureBox) operating on
 * explicit host grids in the reference layouts (include/mx_reion.h).  Used by
 * the tests, the smoke check and the CPU baseline of the benchmark as the
 * checker; never linked by the product library.
 *
 * Parity pinning: this restatement is checked against the reference's own
 * sources compiled with the shims in oracle/shims (oracle/_ref, built by
 * `make ref` where the reference tree is present) and against the committed
 * fixtures in tests/golden/ that were produced by that build.
 */
#ifndef MX_ORACLE_H
#define MX_ORACLE_H

#include "../include/mx_reion.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mxo_ctx mxo_ctx;

int mxo_create(const mx_params* p, const char* tables_dir, mxo_ctx** out);
void mxo_destroy(mxo_ctx* c);
int mxo_set_redshifts(mxo_ctx* c, const double* zz, int n_snaps);
int mxo_n_sfr_histories(const mxo_ctx* c);
int mxo_find_HII_bubbles(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out);
int mxo_ComputeTs(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out);
int mxo_delta_T(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out);
/* Per-cell threshold margins of the last find_HII_bubbles call, two REAL
 * grids back to back: [0, N) the min over radii up to and including the first
 * crossing of |f_coll*eff / (nf*(1+rec)) - 1| (decides the ionised flag and the
 * first-crossing J_21 / Gamma12); [N, 2N) the same min over every radius
 * (decides r_bubble, which is overwritten at each ionising radius).  A cell
 * whose outputs can legitimately differ between two FP32 FFT implementations
 * has a small margin.  NULL before a call. */
/* construct_baryon_grids (reionization.c:1353-1615) on galaxy arrays, and
 * calculate_Mvir_crit (physics/reionization.c:10-59). */
int mxo_construct_baryon_grids(mxo_ctx* c, int snapshot, int n, const float* pos, const int* type, const double* fesc_gsm,
                               const double* gross_sm, const double* bhm, const double* ebhm, int flag_bh,
                               double bh_limit, double alpha_uv_bh, const mx_grids* g);
int mxo_calculate_Mvir_crit(mxo_ctx* c, double redshift, double m0, double a, double b, double cc, double d,
                            const float* J_21_at_ion, const float* z_at_ion, float* Mvir_crit);
/* Light cone (ConstructLightcone.c:12-166): returns LightconeLength. */
long long mxo_lightcone_init(mxo_ctx* c, double end_redshift, int last_output_snap, int* end_snapshot);
int mxo_construct_lightcone(mxo_ctx* c, int snapshot, const float* delta_T, float* delta_T_prev, float* lightcone,
                            float* lightcone_redshifts);
/* 21 cm power spectrum of a REAL delta_T grid (Initialise_PowerSpectrum and
 * Compute_PS, ComputePowerSpectrum.c:18-255); box_size in Mpc/h.  Returns the
 * number of k bins, or -1 if it exceeds cap. */
int mxo_ps_length(int D, double box_size_mpc_h, double hubble_h);
int mxo_power_spectrum(int D, double box_size_mpc_h, double hubble_h, const float* delta_T, float* ps_k, float* ps_data,
                       float* ps_error, int cap);
const float* mxo_last_margin(const mxo_ctx* c);

/* CPU timing of the benchmark (not used by the parity tests).  A timing
 * sample bounds the work of one call: find_HII_bubbles stops after its first
 * max_radii radii, ComputeTs smooths only its first max_shells shells (the
 * others repeat them, so the per-cell step still reads every shell) and
 * evolves only the first D / cell_div x planes.  The grids such a call leaves
 * are not the step's results.  0 (or 1 for cell_div) switches a limit off.
 * mxo_phase_times returns the wall seconds of the phases of the last calls,
 * indexed by MXO_PH_*, so that the sampled parts can be scaled to the full
 * counts.  The first radius and the first shell also touch freshly
 * allocated buffers for the first time and are left out of the per-radius and
 * per-shell times. */
#define MXO_PH_FORWARD 0       /* find_HII_bubbles: forward transforms + 1/N */
#define MXO_PH_RADII 1         /* the radius loop after its first radius */
#define MXO_PH_N_RADII 2       /* radii in MXO_PH_RADII */
#define MXO_PH_FHB_POST 3      /* global means and N_rec */
#define MXO_PH_SHELLS 4        /* ComputeTs: SFR reweighting + smoothing of the shells after the first */
#define MXO_PH_N_SHELLS 5      /* shells in MXO_PH_SHELLS */
#define MXO_PH_TABLES 6        /* frequency-integral tables and Ly-n sums */
#define MXO_PH_EVOLVE 7        /* per-cell evolution */
#define MXO_PH_EVOLVE_FRAC 8   /* fraction of the cells evolved */
#define MXO_PH_TS_POST 9       /* means */
#define MXO_PH_N_RADII_RUN 10  /* radii run (all of them without a sample) */
#define MXO_PH_N_SHELLS_RUN 11 /* shells smoothed */
#define MXO_PH_SHELL_COPIES 12 /* the repeated shells of a sample */
#define MXO_N_PHASES 13
void mxo_set_timing_sample(mxo_ctx* c, int max_radii, int max_shells, int cell_div);
const double* mxo_phase_times(const mxo_ctx* c);
/* dv/dx (padded layout) of the last delta_T with peculiar velocities, or NULL. */
const float* mxo_last_velocity_gradient(const mxo_ctx* c);

/* Table-level helpers (host physics) for tests. */
double mxo_recombination_rate_splined(mxo_ctx* c, double z_eff, double gamma12);
double mxo_dtdz(const mxo_ctx* c, float z);
double mxo_get_Ts(mxo_ctx* c, float z, float delta, float TK, float xe, float Jalpha, float* xalpha);
/* Frequency-integral tables of the last ComputeTs call: [3][14][n_shells]. */
const double* mxo_last_freq_tables(const mxo_ctx* c, int* n_shells);

#ifdef __cplusplus
}
#endif

#endif
