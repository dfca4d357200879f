/*
 * Driver for the reference's own reionization sources compiled against the
 * shims (oracle/_ref/libmxref.so) — TEST INFRASTRUCTURE ONLY.
 *
 * It sets up `run_globals` the way init_meraxes() / init_storage() do for the
 * fields the grid step reads (src/core/init.c:184-205 set_units,
 * init.c:292-313 set_sfr_history / init_MHR, reionization.c:518-952
 * malloc_reionization_grids), then calls the reference's entry points
 * find_HII_bubbles(), ComputeTs() and ComputeBrightnessTemperatureBox()
 * unmodified.  Used only to pin the C restatement in mx_oracle.c and to make
 * the golden fixtures under tests/golden/.
 */
#define _MAIN
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "meraxes.h"

#include "BrightnessTemperature.h"
#include "ComputeTs.h"
#include "XRayHeatingFunctions.h"
#include "find_HII_bubbles.h"
#include "recombinations.h"
#include "ComputePowerSpectrum.h"
#include "ConstructLightcone.h"
#include "physics/reionization.h"
#include "reionization.h"
#include "utils.h"

#include "../include/mx_reion.h"

static int g_ready = 0;

int mxref_init(const mx_params* p, const double* zz, int n_snaps, const char* tables_dir)
{
  memset(&run_globals, 0, sizeof(run_globals));
  run_params_t* rp = &run_globals.params;
  physics_params_t* ph = &rp->physics;
  run_units_t* u = &run_globals.units;

  run_globals.mpi_comm = MPI_COMM_WORLD;
  run_globals.mpi_rank = 0;
  run_globals.mpi_size = 1;

  rp->BoxSize = p->box_size;
  rp->Hubble_h = p->hubble_h;
  rp->OmegaM = p->omega_m;
  rp->OmegaLambda = p->omega_lambda;
  rp->OmegaR = p->omega_r;
  rp->OmegaK = p->omega_k;
  rp->BaryonFrac = p->baryon_frac;
  rp->wLambda = p->w_lambda;
  rp->ReionGridDim = p->grid_dim;
  rp->ReionFilterType = p->filter_type;
  rp->ReionRtoMFilterType = p->rtom_filter_type;
  rp->TsHeatingFilterType = p->ts_heating_filter_type;
  rp->TsNumFilterSteps = p->ts_num_filter_steps;
  rp->ReionUVBFlag = p->uvb_flag;
  rp->ReionDeltaRFactor = p->delta_r_factor;
  rp->TreesID = (enum tree_ids)p->trees_id;
  rp->Flag_PatchyReion = 1;
  rp->Flag_IncludeSpinTemp = p->flag_spin_temp;
  rp->Flag_IncludeRecombinations = p->flag_recombinations;
  rp->Flag_Compute21cmBrightTemp = p->flag_21cm;
  rp->Flag_IncludePecVelsFor21cm = p->flag_pecvel;
  rp->Flag_ComputePS = 0;
  rp->Flag_ConstructLightcone = 0;
  rp->ReionSfrTimescale = p->reion_sfr_timescale;
  strncpy(rp->TablesForXHeatingDir, tables_dir ? tables_dir : ".", STRLEN - 1);
  rp->FFTW3WisdomDir[0] = '\0';

  ph->ReionEfficiency = p->reion_efficiency;
  ph->ReionNionPhotPerBary = p->nion_phot_per_bary;
  ph->ReionGammaHaloBias = p->gamma_halo_bias;
  ph->ReionAlphaUV = p->alpha_uv;
  ph->Y_He = p->y_he;
  ph->ReionRBubbleMin = p->r_bubble_min;
  ph->ReionRBubbleMax = p->r_bubble_max;
  ph->ReionRBubbleMaxRecomb = p->r_bubble_max_recomb;
  ph->ReionMaxHeatingRedshift = p->max_heating_redshift;
  ph->LXrayGal = p->lx_gal;
  ph->NuXrayGalThreshold = p->nu_xray_gal_threshold;
  ph->SpecIndexXrayGal = p->spec_index_xray_gal;
  ph->NuXraySoftCut = p->nu_xray_soft_cut;
  ph->NuXrayMax = p->nu_xray_max;

  /* set_units (init.c:184-205) */
  u->UnitLength_in_cm = p->unit_length_cm;
  u->UnitMass_in_g = p->unit_mass_g;
  u->UnitVelocity_in_cm_per_s = p->unit_velocity_cm_s;
  u->UnitTime_in_s = u->UnitLength_in_cm / u->UnitVelocity_in_cm_per_s;
  u->UnitTime_in_Megayears = u->UnitTime_in_s / SEC_PER_MEGAYEAR;
  run_globals.G = GRAVITY / pow(u->UnitLength_in_cm, 3) * u->UnitMass_in_g * pow(u->UnitTime_in_s, 2);
  run_globals.Hubble = HUBBLE * u->UnitTime_in_s;
  run_globals.RhoCrit = 3 * run_globals.Hubble * run_globals.Hubble / (8 * M_PI * run_globals.G);

  run_globals.ZZ = (double*)malloc(sizeof(double) * (size_t)n_snaps);
  memcpy(run_globals.ZZ, zz, sizeof(double) * (size_t)n_snaps);
  run_globals.ListOutputSnaps = (int*)malloc(sizeof(int));
  run_globals.ListOutputSnaps[0] = n_snaps - 1;
  run_globals.NOutputSnaps = 1;
  run_globals.NStoreSnapshots = 1;

  if (rp->Flag_IncludeSpinTemp)
    run_globals.NstoreSnapshots_SFR = set_sfr_history();
  malloc_reionization_grids();
  if (rp->Flag_IncludeRecombinations)
    init_MHR();
  g_ready = 1;
  return 0;
}

int mxref_n_sfr_histories(void) { return run_globals.NstoreSnapshots_SFR; }

float* mxref_grid(const char* name)
{
  reion_grids_t* g = &run_globals.reion_grids;
#define G(n)                                                                                                           \
  if (!strcmp(name, #n))                                                                                               \
    return (float*)g->n;
  G(deltax) G(stars) G(weighted_sfr) G(sfr) G(sfr_histories) G(N_rec) G(x_e_box) G(x_e_box_prev) G(Tk_box)
  G(TS_box) G(xH) G(z_at_ionization) G(r_bubble) G(J_21) G(J_21_at_ionization) G(Gamma12) G(delta_T) G(vel)
#undef G
  return NULL;
}

void mxref_globals(mx_globals* out)
{
  reion_grids_t* g = &run_globals.reion_grids;
  memset(out, 0, sizeof(*out));
  out->volume_weighted_global_xH = g->volume_weighted_global_xH;
  out->volume_weighted_global_J_21 = g->volume_weighted_global_J_21;
  out->mass_weighted_global_xH = g->mass_weighted_global_xH;
  out->volume_ave_J_alpha = g->volume_ave_J_alpha;
  out->volume_ave_xalpha = g->volume_ave_xalpha;
  out->volume_ave_Xheat = g->volume_ave_Xheat;
  out->volume_ave_Xion = g->volume_ave_Xion;
  out->volume_ave_TS = g->volume_ave_TS;
  out->volume_ave_TK = g->volume_ave_TK;
  out->volume_ave_xe = g->volume_ave_xe;
  out->volume_ave_Tb = g->volume_ave_Tb;
  out->x_e_ave = x_e_ave;
}

double mxref_stored_fcoll(int snapshot) { return stored_fcoll[snapshot]; }

int mxref_find_HII_bubbles(int snapshot)
{
  timer_info t;
  timer_start(&t);
  find_HII_bubbles(snapshot, &t);
  return 0;
}

int mxref_ComputeTs(int snapshot)
{
  timer_info t;
  timer_start(&t);
  ComputeTs(snapshot, &t);
  return 0;
}

int mxref_delta_T(int snapshot)
{
  ComputeBrightnessTemperatureBox(snapshot);
  return 0;
}

/* Selected physics helpers of the reference, exposed for table-level tests. */
double mxref_splined_recombination_rate(double z_eff, double gamma12) { return splined_recombination_rate(z_eff, gamma12); }
double mxref_dtdz(float z) { return dtdz(z); }
double mxref_RtoM(double R) { return RtoM(R); }

/* Initialise_PowerSpectrum + Compute_PS on a REAL delta_T grid (needs a
 * context made with flag_21cm so that reion_grids.delta_T exists). */
int mxref_power_spectrum(const float* delta_T, float* ps_k, float* ps_data, float* ps_error, int cap)
{
  reion_grids_t* g = &run_globals.reion_grids;
  const int D = run_globals.params.ReionGridDim;
  if (!g->delta_T)
    return -2;
  Initialise_PowerSpectrum();
  const int nb = run_globals.params.PS_Length;
  if (nb > cap)
    return -1;
  memcpy(g->delta_T, delta_T, sizeof(float) * (size_t)D * D * D);
  g->PS_k = ps_k;
  g->PS_data = ps_data;
  g->PS_error = ps_error;
  Compute_PS(0);
  g->PS_k = g->PS_data = g->PS_error = NULL;
  return nb;
}

/* Initialise_ConstructLightcone with EndRedshiftLightcone and LastOutputSnap;
 * allocates delta_T_prev, LightconeBox and Lightcone_redshifts. */
long long mxref_lightcone_init(double end_redshift, int last_output_snap, int* end_snapshot)
{
  reion_grids_t* g = &run_globals.reion_grids;
  const int D = run_globals.params.ReionGridDim;
  run_globals.params.EndRedshiftLightcone = end_redshift;
  run_globals.LastOutputSnap = last_output_snap;
  Initialise_ConstructLightcone();
  const long long n = run_globals.params.LightconeLength;
  free(g->LightconeBox);
  free(g->Lightcone_redshifts);
  if (!g->delta_T_prev)
    g->delta_T_prev = (float*)calloc((size_t)D * D * D, sizeof(float));
  g->LightconeBox = (float*)calloc((size_t)D * D * (size_t)n, sizeof(float));
  g->Lightcone_redshifts = (float*)calloc((size_t)n, sizeof(float));
  *end_snapshot = run_globals.params.EndSnapshotLightcone;
  return n;
}

int mxref_construct_lightcone(int snapshot, const float* delta_T, float* delta_T_prev, float* lightcone, float* lc_z)
{
  reion_grids_t* g = &run_globals.reion_grids;
  const int D = run_globals.params.ReionGridDim;
  const long long n = run_globals.params.LightconeLength;
  memcpy(g->delta_T, delta_T, sizeof(float) * (size_t)D * D * D);
  memcpy(g->delta_T_prev, delta_T_prev, sizeof(float) * (size_t)D * D * D);
  ConstructLightcone(snapshot);
  memcpy(delta_T_prev, g->delta_T_prev, sizeof(float) * (size_t)D * D * D);
  memcpy(lightcone, g->LightconeBox, sizeof(float) * (size_t)D * D * (size_t)n);
  memcpy(lc_z, g->Lightcone_redshifts, sizeof(float) * (size_t)n);
  return 0;
}

/* construct_baryon_grids (reionization.c:1353-1615) on a galaxy list given
 * as arrays (Pos, Type, FescWeightedGSM, GrossStellarMass, BlackHoleMass,
 * EffectiveBHM; the last two may be NULL when flag_bh is 0). */
int mxref_construct_baryon_grids(int snapshot, int n, const float* pos, const int* type, const double* fesc_gsm,
                                 const double* gross_sm, const double* bhm, const double* ebhm, int flag_bh,
                                 double bh_limit, double alpha_uv_bh)
{
  reion_grids_t* g = &run_globals.reion_grids;
  const int D = run_globals.params.ReionGridDim;
  physics_params_t* ph = &run_globals.params.physics;
  ph->Flag_BHFeedback = flag_bh;
  ph->BlackHoleMassLimitReion = bh_limit;
  ph->ReionAlphaUVBH = alpha_uv_bh;
  galaxy_t* gals = (galaxy_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(galaxy_t));
  gal_to_slab_t* map = (gal_to_slab_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(gal_to_slab_t));
  int live = 0;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++)
      gals[i].Pos[k] = pos[3 * i + k];
    gals[i].Type = type[i];
    gals[i].FescWeightedGSM = fesc_gsm[i];
    gals[i].GrossStellarMass = gross_sm[i];
    gals[i].BlackHoleMass = bhm ? bhm[i] : 0.0;
    gals[i].EffectiveBHM = ebhm ? ebhm[i] : 0.0;
    map[i].index = i;
    map[i].galaxy = &gals[i];
    map[i].slab_ind = 0;
    if (type[i] <= 2)
      live++;
  }
  g->galaxy_to_slab_map = map;
  g->buffer_size = (int)((size_t)D * D * D);
  float* buf = (float*)calloc((size_t)D * D * D, sizeof(float));
  g->buffer = buf;
  construct_baryon_grids(snapshot, live);
  g->buffer = NULL;
  g->galaxy_to_slab_map = NULL;
  free(buf);
  free(map);
  free(gals);
  return 0;
}

/* calculate_Mvir_crit (physics/reionization.c:10-59) on given grids */
int mxref_calculate_Mvir_crit(double redshift, double m0, double a, double b, double c, double d,
                              const float* J_21_at_ion, const float* z_at_ion, float* out)
{
  reion_grids_t* g = &run_globals.reion_grids;
  const int D = run_globals.params.ReionGridDim;
  physics_params_t* ph = &run_globals.params.physics;
  ph->ReionSMParam_m0 = m0;
  ph->ReionSMParam_a = a;
  ph->ReionSMParam_b = b;
  ph->ReionSMParam_c = c;
  ph->ReionSMParam_d = d;
  const size_t n = (size_t)D * D * D;
  if (!g->Mvir_crit)
    g->Mvir_crit = (float*)calloc(n, sizeof(float));
  memcpy(g->J_21_at_ionization, J_21_at_ion, sizeof(float) * n);
  memcpy(g->z_at_ionization, z_at_ion, sizeof(float) * n);
  calculate_Mvir_crit(redshift);
  memcpy(out, g->Mvir_crit, sizeof(float) * n);
  return 0;
}
