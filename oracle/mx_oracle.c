/*
 * CPU oracle of the reionization grid step — TEST INFRASTRUCTURE ONLY.
 * See mx_oracle.h.  Every function cites the reference lines it restates
 * (paths relative to the Meraxes source tree).
 */
#include "mx_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#include "mx_numerics.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_E
#define M_E 2.7182818284590452354
#endif

/* ---- constants: src/meraxes.h:21-44, src/core/reionization.h:8-46,
 *      src/core/XRayHeatingFunctions.h:15-40, recombinations.h:17-33,
 *      ComputeTs.h:6 */
#define K_GRAVITY 6.672e-8
#define K_SOLAR_MASS 1.989e33
#define K_BOLTZMANN 1.3806e-16
#define K_C 2.9979e10
#define K_PLANCK 6.6262e-27
#define K_PROTONMASS 1.6726e-24
#define K_HUBBLE 3.2407789e-18
#define K_SEC_PER_YEAR 3.155e7
#define K_MPC 3.086e24
#define K_TCMB 2.728
#define K_REL_TOL ((float)1e-5)
#define K_ABS_TOL ((float)1e-8)
#define K_SIGMA_HI 6.3e-18
#define K_TINY 1e-30
#define K_FRACT_FLOAT_ERR 1e-7
#define K_MAX_TK ((float)5e4)
#define K_L_FACTOR 0.620350491
#define K_ALPHAB_10K 2.59e-13
#define K_T21 0.0628
#define K_A10 2.85e-15
#define K_LYA_HZ 2.46606727e15
#define K_NU_OVER_EV (1.60217646e-12 / K_PLANCK)
#define K_NU_HI (13.60 * K_NU_OVER_EV)
#define K_NU_HEI (24.59 * K_NU_OVER_EV)
#define K_NU_HEII (K_NU_HI * 4)
#define K_NSPEC_MAX 23
#define K_RECFAST_NPTS 501
#define K_KAPPA_10_NPTS 27
#define K_KAPPA_E_NPTS 20
#define K_KAPPA_P_NPTS 17
#define K_NXHII 14
#define K_NENERGY 258
#define K_R_XLY_MAX ((float)500)
#define K_A_NPTS 60
#define K_C_NPTS 12
#define K_BETA_NPTS 5
#define K_RR_Z_NPTS 300
#define K_RR_DEL_Z ((float)0.2)
#define K_RR_LNG_NPTS 150
#define K_RR_LNG_MIN (-10.0)
#define K_RR_DEL_LNG ((float)0.1)

struct mxo_ctx
{
  mx_params p;
  float* last_vel_grad; /* dv/dx of the last peculiar-velocity delta_T (padded), for tests */
  long long lc_length, lc_pos; /* LightconeLength, CurrentLCPos */
  int lc_end_snapshot;         /* EndSnapshotLightcone */
  double unit_time_s, G, hubble_int, rho_crit;
  double no, he_no, f_h, f_he, n_b0;
  double* zz;
  int n_snaps;
  int n_hist;
  double stored_fcoll[1000];
  double x_e_ave;
  /* recombination tables */
  int mhr_ready;
  mxo_spline A_sp, C_sp, beta_sp;
  mxo_spline rr_sp[K_RR_Z_NPTS];
  /* spin-temperature tables */
  int heat_ready;
  mxo_spline recfast_T, recfast_x;
  double recfast_zmax;
  mxo_spline kap10, kap_e, kap_p;
  double kap10_t[K_KAPPA_10_NPTS], kap10_k[K_KAPPA_10_NPTS];
  double kap_e_t[K_KAPPA_E_NPTS], kap_e_k[K_KAPPA_E_NPTS];
  double kap_p_t[K_KAPPA_P_NPTS], kap_p_k[K_KAPPA_P_NPTS];
  float spec_nu[K_NSPEC_MAX], spec_N0[K_NSPEC_MAX], spec_alpha[K_NSPEC_MAX];
  float x_xhii[K_NXHII];
  float x_energy[K_NENERGY];
  float x_fheat[K_NXHII][K_NENERGY], x_nlya[K_NXHII][K_NENERGY];
  float x_nion_hi[K_NXHII][K_NENERGY], x_nion_hei[K_NXHII][K_NENERGY], x_nion_heii[K_NXHII][K_NENERGY];
  /* per-call ComputeTs state (file-scope globals in XRayHeatingFunctions.h:43-60) */
  double* zpp_edge;
  double* sum_lyn;
  double growth_zp, dgrowth_dzp, dt_dzp, const_zp_prefactor;
  double* freq_tables; /* [3][14][S] */
  float* margin;
  /* grid buffers kept across calls, as the reference allocates its grids
   * once (reionization.c malloc_reionization_grids) */
  float* fhb_buf[10]; /* unfiltered and filtered spectra of the 5 fields */
  float* ts_buf[2];
  double* smoothed;
  double* contrib;
  int ts_shells;
  /* CPU-timing sample (mxo_set_timing_sample) and phase times */
  int sample_radii, sample_shells, sample_cell_div;
  double phase[MXO_N_PHASES];
};

/* ======================================================= cosmology helpers */

/* dtdz, XRayHeatingFunctions.c:377-392 */
static double c_dtdz(const mxo_ctx* c, float z)
{
  const double OMl = c->p.omega_lambda, OMm = c->p.omega_m;
  const double x = sqrt(OMl / OMm) * pow(1 + z, -3.0 / 2.0);
  const double dxdz = sqrt(OMl / OMm) * pow(1 + z, -5.0 / 2.0) * (-3.0 / 2.0);
  const double const1 = 2 * sqrt(1 + OMm / OMl) / (3.0 * K_HUBBLE * c->p.hubble_h);
  const double numer = dxdz * (1 + x * pow(pow(x, 2) + 1, -0.5));
  const double denom = x + sqrt(pow(x, 2) + 1);
  return (const1 * numer / denom);
}

/* hubble, XRayHeatingFunctions.c:395-404 */
static double c_hubble(const mxo_ctx* c, float z)
{
  return K_HUBBLE * c->p.hubble_h *
         sqrt(c->p.omega_m * pow(1 + z, 3) + c->p.omega_r * pow(1 + z, 4) + c->p.omega_lambda);
}

/* drdz, XRayHeatingFunctions.c:463-467 */
static double c_drdz(const mxo_ctx* c, float z) { return (1.0 + z) * K_C * c_dtdz(c, z); }

/* RtoM, find_HII_bubbles.c:26-45 */
static double c_RtoM(const mxo_ctx* c, double R)
{
  if (c->p.rtom_filter_type == 1)
    return pow(2 * M_PI, 1.5) * c->p.omega_m * c->rho_crit * pow(R, 3);
  return (4.0 / 3.0) * M_PI * pow(R, 3) * (c->p.omega_m * c->rho_crit);
}

/* dicke, XRayHeatingFunctions.c:1469-1503 (flat Lambda branch and EdS) */
static double c_dicke(const mxo_ctx* c, double z)
{
  const double OMm = c->p.omega_m, OMl = c->p.omega_lambda, OMr = c->p.omega_r;
  if (fabs(OMm - 1.0) < 1e-4)
    return 1.0 / (1.0 + z);
  const double omegaM_z = OMm * pow(1 + z, 3) / (OMl + OMm * pow(1 + z, 3) + OMr * pow(1 + z, 4));
  const double dick_z = 2.5 * omegaM_z / (1.0 / 70.0 + omegaM_z * (209 - omegaM_z) / 140.0 + pow(omegaM_z, 4.0 / 7.0));
  const double dick_0 = 2.5 * OMm / (1.0 / 70.0 + OMm * (209 - OMm) / 140.0 + pow(OMm, 4.0 / 7.0));
  return dick_z / (dick_0 * (1.0 + z));
}

/* ddicke_dz, XRayHeatingFunctions.c:1506-1511: forward difference with a
 * float step of 1e-10 */
static double c_ddicke_dz(const mxo_ctx* c, double z)
{
  const float dz = 1e-10f;
  return (c_dicke(c, z + dz) - c_dicke(c, z)) / dz;
}

/* ================================================================= filter */

/* filter(), reionization.c:2110-2170: W(kR) multiplied into the half
 * spectrum (interleaved float complex). */
static void c_filter(const mxo_ctx* c, float* box, int D, float R, int filter_type)
{
  const int middle = D / 2;
  const int H = D / 2 + 1;
  const float box_size = (float)c->p.box_size;
  const float delta_k = (float)(2.0 * M_PI / box_size);
#pragma omp parallel for schedule(static)
  for (int n_x = 0; n_x < D; n_x++) {
    const float k_x = (n_x > middle) ? (n_x - D) * delta_k : n_x * delta_k;
    for (int n_y = 0; n_y < D; n_y++) {
      const float k_y = (n_y > middle) ? (n_y - D) * delta_k : n_y * delta_k;
      for (int n_z = 0; n_z <= middle; n_z++) {
        const float k_z = n_z * delta_k;
        const float k_mag = sqrtf(k_x * k_x + k_y * k_y + k_z * k_z);
        float kR = k_mag * R;
        float* v = box + 2 * (((size_t)n_x * D + n_y) * H + n_z);
        if (filter_type == 0) {
          if (kR > 1e-4) {
            const float w = (float)(3.0 * (sinf(kR) / powf(kR, 3) - cosf(kR) / powf(kR, 2)));
            v[0] *= w;
            v[1] *= w;
          }
        } else if (filter_type == 1) {
          kR *= 0.413566994;
          if (kR > 1) {
            v[0] = 0.0f;
            v[1] = 0.0f;
          }
        } else if (filter_type == 2) {
          kR *= 0.643;
          const float w = powf((float)M_E, (float)(-kR * kR / 2.0));
          v[0] *= w;
          v[1] *= w;
        }
      }
    }
  }
}

static size_t pad_idx(int D, int i, int j, int k) { return (size_t)k + (size_t)(2 * (D / 2 + 1)) * ((size_t)j + (size_t)D * i); }
static size_t real_idx(int D, int i, int j, int k) { return (size_t)k + (size_t)D * ((size_t)j + (size_t)D * i); }

/* ========================================================= recombinations */

/* alpha_A, XRayHeatingFunctions.c:1450-1458 */
static double c_alpha_A(double T)
{
  const double logT = log(T / (double)1.1604505e4);
  return exp(-28.6130338 - 0.72411256 * logT - 2.02604473e-2 * pow(logT, 2) - 2.38086188e-3 * pow(logT, 3) -
             3.21260521e-4 * pow(logT, 4) - 1.42150291e-5 * pow(logT, 5) + 4.98910892e-6 * pow(logT, 6) +
             5.75561414e-7 * pow(logT, 7) - 1.85676704e-8 * pow(logT, 8) - 3.07113524e-9 * pow(logT, 9));
}

/* alpha_B, recombinations.c:359-363 */
static double c_alpha_B(double T) { return K_ALPHAB_10K * pow(T / 1.0e4, -0.75); }

/* neutral_fraction, recombinations.c:332-357 (case B) */
static double c_neutral_fraction(const mxo_ctx* c, double density, double T4, double gamma12)
{
  const double corr_He = 1.0 / (4.0 / c->p.y_he - 3);
  const double alpha = c_alpha_B(T4 * 1e4);
  gamma12 *= 1e-12;
  double chi = (1 + corr_He) * density * alpha / gamma12;
  if (chi < K_TINY)
    return 0;
  if (chi < 1e-5)
    return chi;
  const double b = -2 - gamma12 / (density * (1 + corr_He) * alpha);
  chi = (-b - sqrt(b * b - 4)) / 2.0;
  return chi;
}

/* Gamma_SS, recombinations.c:104-108 */
static double c_gamma_ss(double Gamma_bg, double Delta, double T_4, double z)
{
  const double D_ss = 26.7 * pow(T_4, 0.17) * pow((1 + z) / 10.0, -3) * pow(Gamma_bg, 2.0 / 3.0);
  return Gamma_bg * (0.98 * pow((1.0 + pow(Delta / D_ss, 1.64)), -2.28) + 0.02 * pow(1.0 + Delta / D_ss, -0.84));
}

/* C_MHR / beta_MHR / A_MHR, recombinations.c:190-316 */
static double c_C_MHR(const mxo_ctx* c, double z)
{
  if (z >= 13.0)
    return 1.0;
  if (z <= 2.0)
    return 0.558;
  return mxo_spline_eval(&c->C_sp, z);
}
static double c_beta_MHR(const mxo_ctx* c, double z)
{
  if (z >= 6.0)
    return -2.50;
  if (z <= 2.0)
    return -2.23;
  return mxo_spline_eval(&c->beta_sp, z);
}
static double c_A_MHR(const mxo_ctx* c, double z)
{
  if (z >= 2.0 + (float)K_A_NPTS)
    return mxo_spline_eval(&c->A_sp, 2.0 + (float)K_A_NPTS);
  if (z <= 2.0)
    return mxo_spline_eval(&c->A_sp, 2.0);
  return mxo_spline_eval(&c->A_sp, z);
}

typedef struct
{
  const mxo_ctx* c;
  double z;
} aux_par;

/* aux_function, recombinations.c:160-170 */
static double f_aux(double D, void* vp)
{
  const aux_par* a = (const aux_par*)vp;
  const double z = a->z;
  const double Cz = c_C_MHR(a->c, z);
  return exp(-(pow(D, -2.0 / 3.0) - Cz) * (pow(D, -2.0 / 3.0) - Cz) /
             (2.0 * (2.0 * 7.61 / (3.0 * (1.0 + z))) * (2.0 * 7.61 / (3.0 * (1.0 + z))))) *
         pow(D, c_beta_MHR(a->c, z));
}

typedef struct
{
  const mxo_ctx* c;
  double z, gamma12_bg, T4, A, C_0, beta, avenH;
} rr_par;

/* MHR_rr, recombinations.c:116-135 (case B) */
static double f_mhr_rr(double lnD, void* vp)
{
  const rr_par* p = (const rr_par*)vp;
  const double D = exp(lnD);
  const double z = p->z;
  const double gamma = c_gamma_ss(p->gamma12_bg, D, p->T4, z);
  const double n_H = p->avenH * D;
  const double x_e = 1.0 - c_neutral_fraction(p->c, n_H, p->T4, gamma);
  const double PDelta =
    p->A * exp(-0.5 * pow((pow(D, -2.0 / 3.0) - p->C_0) / ((2.0 * 7.61 / (3.0 * (1.0 + z)))), 2)) * pow(D, p->beta);
  const double alpha = c_alpha_B(p->T4 * 1e4);
  return n_H * PDelta * alpha * x_e * x_e * D * D;
}

/* init_MHR, recombinations.c:54-84 and the A/C/beta tables at :202-311 */
static void c_init_mhr(mxo_ctx* c)
{
  double xs[K_A_NPTS], ys[K_A_NPTS];
  static const double C_tab[K_C_NPTS] = { 0.558, 0.599, 0.611, 0.769, 0.868, 0.930,
                                          0.964, 0.983, 0.993, 0.998, 0.999, 1.00 };
  static const double beta_tab[K_BETA_NPTS] = { -2.23, -2.35, -2.48, -2.49, -2.50 };
  for (int i = 0; i < K_C_NPTS; i++)
    xs[i] = (float)i + 2.0;
  mxo_spline_init(&c->C_sp, xs, C_tab, K_C_NPTS);
  for (int i = 0; i < K_BETA_NPTS; i++)
    xs[i] = (float)i + 2.0;
  mxo_spline_init(&c->beta_sp, xs, beta_tab, K_BETA_NPTS);
  for (int i = 0; i < K_A_NPTS; i++) {
    aux_par ap = { c, 2.0 + (float)i };
    double res, err;
    mxo_qag61(f_aux, &ap, 1e-25, 1e25, 0, 0.001, 1000, &res, &err);
    xs[i] = 2.0 + (float)i;
    ys[i] = 1.0 / res;
  }
  mxo_spline_init(&c->A_sp, xs, ys, K_A_NPTS);

  double lng[K_RR_LNG_NPTS], rr[K_RR_LNG_NPTS];
  for (int z_ct = 0; z_ct < K_RR_Z_NPTS; z_ct++) {
    const float z = z_ct * K_RR_DEL_Z;
    for (int g = 0; g < K_RR_LNG_NPTS; g++) {
      lng[g] = K_RR_LNG_MIN + g * K_RR_DEL_LNG;
      const float gamma = (float)exp(lng[g]);
      /* recombination_rate(z, gamma, 1, 1), recombinations.c:141-158 */
      rr_par rp = { c, z, gamma, 1.0, c_A_MHR(c, z), c_C_MHR(c, z), c_beta_MHR(c, z), c->no * pow(1 + (double)z, 3) };
      double res, err;
      mxo_qag61(f_mhr_rr, &rp, log(0.01), log(200), 0, 0.01, 1000, &res, &err);
      rr[g] = res;
    }
    mxo_spline_init(&c->rr_sp[z_ct], lng, rr, K_RR_LNG_NPTS);
  }
  c->mhr_ready = 1;
}

/* splined_recombination_rate, recombinations.c:30-52 */
static double c_rr_splined(const mxo_ctx* c, double z_eff, double gamma12_bg)
{
  int z_ct = (int)(z_eff / K_RR_DEL_Z + 0.5);
  double lnGamma = log(gamma12_bg);
  if (z_ct < 0)
    z_ct = 0;
  else if (z_ct >= K_RR_Z_NPTS)
    z_ct = K_RR_Z_NPTS - 1;
  if (lnGamma < K_RR_LNG_MIN)
    return 0;
  else if (lnGamma >= (K_RR_LNG_MIN + K_RR_DEL_LNG * K_RR_LNG_NPTS))
    lnGamma = K_RR_LNG_MIN + K_RR_DEL_LNG * K_RR_LNG_NPTS - K_FRACT_FLOAT_ERR;
  return mxo_spline_eval(&c->rr_sp[z_ct], lnGamma);
}

/* ================================================================ context */

int mxo_create(const mx_params* p, const char* tables_dir, mxo_ctx** out)
{
  mxo_ctx* c = (mxo_ctx*)calloc(1, sizeof(mxo_ctx));
  c->p = *p;
  /* set_units, init.c:184-205 */
  c->unit_time_s = p->unit_length_cm / p->unit_velocity_cm_s;
  c->G = K_GRAVITY / pow(p->unit_length_cm, 3) * p->unit_mass_g * pow(c->unit_time_s, 2);
  c->hubble_int = K_HUBBLE * c->unit_time_s;
  c->rho_crit = 3 * c->hubble_int * c->hubble_int / (8 * M_PI * c->G);
  /* reionization.h:16-44 */
  const double rhocrit_cgs = 3.0 * K_HUBBLE * K_HUBBLE * p->hubble_h * p->hubble_h / (8.0 * M_PI * K_GRAVITY);
  const double omb = p->baryon_frac * p->omega_m;
  c->no = rhocrit_cgs * omb * (1 - p->y_he) / K_PROTONMASS;
  c->he_no = rhocrit_cgs * omb * p->y_he / (4.0 * K_PROTONMASS);
  c->f_h = c->no / (c->no + c->he_no);
  c->f_he = c->he_no / (c->no + c->he_no);
  c->n_b0 = c->no + c->he_no;
  if (p->flag_recombinations)
    c_init_mhr(c);
  if (p->flag_spin_temp) {
    /* init_heat tables, XRayHeatingFunctions.c:41-74 */
    char fn[1024];
    FILE* F;
    /* RECFAST, XRayHeatingFunctions.c:104-223 */
    snprintf(fn, sizeof fn, "%s/recfast_LCDM.dat", tables_dir);
    if (!(F = fopen(fn, "r"))) {
      free(c);
      return MX_ETABLE;
    }
    double zt[K_RECFAST_NPTS], tk[K_RECFAST_NPTS], xi[K_RECFAST_NPTS];
    for (int i = K_RECFAST_NPTS - 1; i >= 0; i--) {
      float cz, cx, trash, ct;
      if (fscanf(F, "%f %E %E %E", &cz, &cx, &trash, &ct) != 4) {
        fclose(F);
        free(c);
        return MX_ETABLE;
      }
      zt[i] = cz;
      xi[i] = cx;
      tk[i] = ct;
    }
    fclose(F);
    mxo_spline_init(&c->recfast_T, zt, tk, K_RECFAST_NPTS);
    mxo_spline_init(&c->recfast_x, zt, xi, K_RECFAST_NPTS);
    c->recfast_zmax = zt[K_RECFAST_NPTS - 1];
    /* kappa_10, XRayHeatingFunctions.c:1602-1696 (Zygelman 2005 table) */
    static const double tk10[K_KAPPA_10_NPTS] = { 1.0,   2.0,   4.0,   6.0,   8.0,   10.0,   15.0,   20.0,   25.0,
                                                  30.0,  40.0,  50.0,  60.0,  70.0,  80.0,   90.0,   100.0,  200.0,
                                                  300.0, 501.0, 701.0, 1000.0, 2000.0, 3000.0, 5000.0, 7000.0, 10000.0 };
    static const double k10[K_KAPPA_10_NPTS] = { 1.38e-13, 1.43e-13, 2.71e-13, 6.60e-13, 1.47e-12, 2.88e-12, 9.10e-12,
                                                 1.78e-11, 2.73e-11, 3.67e-11, 5.38e-11, 6.86e-11, 8.14e-11, 9.25e-11,
                                                 1.02e-10, 1.11e-10, 1.19e-10, 1.75e-10, 2.09e-10, 2.565e-10, 2.91e-10,
                                                 3.31e-10, 4.27e-10, 4.97e-10, 6.03e-10, 6.87e-10, 7.87e-10 };
    for (int i = 0; i < K_KAPPA_10_NPTS; i++) {
      c->kap10_t[i] = log(tk10[i]);
      c->kap10_k[i] = log(k10[i]);
    }
    mxo_spline_init(&c->kap10, c->kap10_t, c->kap10_k, K_KAPPA_10_NPTS);
    /* kappa_10_elec / kappa_10_pH, XRayHeatingFunctions.c:1701-1840 */
    const char* kf[2] = { "kappa_eH_table.dat", "kappa_pH_table.dat" };
    const int kn[2] = { K_KAPPA_E_NPTS, K_KAPPA_P_NPTS };
    double* kt[2] = { c->kap_e_t, c->kap_p_t };
    double* kk[2] = { c->kap_e_k, c->kap_p_k };
    for (int t = 0; t < 2; t++) {
      snprintf(fn, sizeof fn, "%s/%s", tables_dir, kf[t]);
      if (!(F = fopen(fn, "r"))) {
        free(c);
        return MX_ETABLE;
      }
      for (int i = 0; i < kn[t]; i++) {
        float a, b;
        if (fscanf(F, "%f %e", &a, &b) != 2) {
          fclose(F);
          free(c);
          return MX_ETABLE;
        }
        kt[t][i] = log((double)a);
        kk[t][i] = log((double)b);
      }
      fclose(F);
    }
    mxo_spline_init(&c->kap_e, c->kap_e_t, c->kap_e_k, K_KAPPA_E_NPTS);
    mxo_spline_init(&c->kap_p, c->kap_p_t, c->kap_p_k, K_KAPPA_P_NPTS);
    /* spectral_emissivity table, XRayHeatingFunctions.c:586-650 (Pop II) */
    snprintf(fn, sizeof fn, "%s/stellar_spectra.dat", tables_dir);
    if (!(F = fopen(fn, "r"))) {
      free(c);
      return MX_ETABLE;
    }
    int nidx[K_NSPEC_MAX];
    for (int i = 1; i < K_NSPEC_MAX; i++) {
      float n2, a2, n3, a3;
      if (fscanf(F, "%i %e %e %e %e", &nidx[i], &n2, &a2, &n3, &a3) != 5) {
        fclose(F);
        free(c);
        return MX_ETABLE;
      }
      c->spec_N0[i] = n2;
      c->spec_alpha[i] = a2;
    }
    fclose(F);
    for (int i = 1; i < K_NSPEC_MAX; i++)
      c->spec_nu[i] = (float)(4.0 / 3.0 * (1.0 - 1.0 / pow(nidx[i], 2.0)));
    for (int i = 1; i < (K_NSPEC_MAX - 1); i++) {
      const double n0_fac = (pow(c->spec_nu[i + 1], c->spec_alpha[i] + 1) - pow(c->spec_nu[i], c->spec_alpha[i] + 1));
      c->spec_N0[i] *= (c->spec_alpha[i] + 1) / n0_fac * p->nion_phot_per_bary;
    }
    /* x_int tables, initialize_interp_arrays, XRayHeatingFunctions.c:805-905 */
    static const float xh[K_NXHII] = { 1.0e-4f, 2.318e-4f, 4.677e-4f, 1.0e-3f, 2.318e-3f, 4.677e-3f, 1.0e-2f,
                                      2.318e-2f, 4.677e-2f, 1.0e-1f, 0.5f, 0.9f, 0.99f, 0.999f };
    memcpy(c->x_xhii, xh, sizeof xh);
    for (int n = 0; n < K_NXHII; n++) {
      if (c->x_xhii[n] < 0.3)
        snprintf(fn, sizeof fn, "%s/x_int_tables/log_xi_%1.1f.dat", tables_dir, log10(c->x_xhii[n]));
      else
        snprintf(fn, sizeof fn, "%s/x_int_tables/xi_%1.3f.dat", tables_dir, c->x_xhii[n]);
      if (!(F = fopen(fn, "r"))) {
        free(c);
        return MX_ETABLE;
      }
      char label[64];
      float f1, f2, f3, f4, f5, trash;
      for (int i = 1; i <= 5; i++)
        if (fscanf(F, "%63s", label) != 1)
          goto bad;
      if (fscanf(F, "%g %g %g %g %g", &f1, &f2, &f3, &f4, &f5) != 5)
        goto bad;
      for (int i = 1; i <= 11; i++)
        if (fscanf(F, "%63s", label) != 1)
          goto bad;
      for (int i = 0; i < K_NENERGY; i++)
        if (fscanf(F, "%g %g %g %g %g %g %g %g %g", &c->x_energy[i], &trash, &c->x_fheat[n][i], &trash,
                   &c->x_nlya[n][i], &c->x_nion_hi[n][i], &c->x_nion_hei[n][i], &c->x_nion_heii[n][i], &trash) != 9)
          goto bad;
      fclose(F);
      continue;
    bad:
      fclose(F);
      free(c);
      return MX_ETABLE;
    }
    c->heat_ready = 1;
  }
  *out = c;
  return 0;
}

void mxo_destroy(mxo_ctx* c)
{
  if (!c)
    return;
  free(c->last_vel_grad);
  if (c->mhr_ready) {
    mxo_spline_free(&c->A_sp);
    mxo_spline_free(&c->C_sp);
    mxo_spline_free(&c->beta_sp);
    for (int i = 0; i < K_RR_Z_NPTS; i++)
      mxo_spline_free(&c->rr_sp[i]);
  }
  if (c->heat_ready) {
    mxo_spline_free(&c->recfast_T);
    mxo_spline_free(&c->recfast_x);
    mxo_spline_free(&c->kap10);
    mxo_spline_free(&c->kap_e);
    mxo_spline_free(&c->kap_p);
  }
  free(c->zz);
  free(c->zpp_edge);
  free(c->sum_lyn);
  free(c->freq_tables);
  free(c->margin);
  for (int i = 0; i < 10; i++)
    free(c->fhb_buf[i]);
  free(c->ts_buf[0]);
  free(c->ts_buf[1]);
  free(c->smoothed);
  free(c->contrib);
  free(c);
}

/* A buffer of the context, allocated on first use (the grid size of a
 * context is fixed). */
static void* ctx_buf(void** slot, size_t bytes)
{
  if (!*slot)
    *slot = malloc(bytes);
  return *slot;
}

/* set_sfr_history, ComputeTs.c:32-76 */
static int c_set_sfr_history(const mxo_ctx* c)
{
  const double box_size = c->p.box_size / c->p.hubble_h;
  const int D = c->p.grid_dim;
  const int S = c->p.ts_num_filter_steps;
  const int last_snap = c->n_snaps - 1;
  int max_snaps = 0;
  for (int snapshot = 1; snapshot <= last_snap; snapshot++) {
    const double zp = c->zz[snapshot];
    double R = K_L_FACTOR * box_size / (float)D;
    const double R_factor = pow(K_R_XLY_MAX / R, 1 / (float)S);
    int scb = 1;
    double prev_R = 0, prev_zpp = zp, zpp_edge;
    for (int R_ct = 0; R_ct < S; R_ct++) {
      zpp_edge = prev_zpp - (R - prev_R) * K_MPC / (c_drdz(c, (float)prev_zpp));
      while (zpp_edge > c->zz[snapshot - scb]) {
        if (snapshot - scb == 0)
          break;
        scb += 1;
      }
      prev_R = R;
      prev_zpp = zpp_edge;
      R *= R_factor;
    }
    if (max_snaps < scb)
      max_snaps = scb;
  }
  return max_snaps;
}

int mxo_set_redshifts(mxo_ctx* c, const double* zz, int n_snaps)
{
  free(c->zz);
  c->zz = (double*)malloc(sizeof(double) * (size_t)n_snaps);
  memcpy(c->zz, zz, sizeof(double) * (size_t)n_snaps);
  c->n_snaps = n_snaps;
  c->n_hist = c->p.flag_spin_temp ? c_set_sfr_history(c) : 0;
  return 0;
}

int mxo_n_sfr_histories(const mxo_ctx* c) { return c->n_hist; }
const float* mxo_last_margin(const mxo_ctx* c) { return c->margin; }
void mxo_set_timing_sample(mxo_ctx* c, int max_radii, int max_shells, int cell_div)
{
  c->sample_radii = max_radii > 0 ? max_radii : 0;
  c->sample_shells = max_shells > 0 ? max_shells : 0;
  c->sample_cell_div = cell_div > 1 ? cell_div : 0;
}
const double* mxo_phase_times(const mxo_ctx* c) { return c->phase; }
double mxo_dtdz(const mxo_ctx* c, float z) { return c_dtdz(c, z); }
double mxo_recombination_rate_splined(mxo_ctx* c, double z_eff, double gamma12)
{
  if (!c->mhr_ready)
    c_init_mhr(c);
  return c_rr_splined(c, z_eff, gamma12);
}
const double* mxo_last_freq_tables(const mxo_ctx* c, int* n_shells)
{
  *n_shells = c->p.ts_num_filter_steps;
  return c->freq_tables;
}

/* ======================================================= find_HII_bubbles */

/* _find_HII_bubbles, find_HII_bubbles.c:47-495 (no mini-halos) */
int mxo_find_HII_bubbles(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out)
{
  const mx_params* p = &c->p;
  const int D = p->grid_dim;
  const int H = D / 2 + 1;
  const size_t nc = (size_t)D * D * H;
  const double box_size = p->box_size;
  const double pixel_volume = pow(box_size / (double)D, 3);
  double cell_length_factor = K_L_FACTOR;
  const double total_n_cells = pow((double)D, 3);
  const int uvb = p->uvb_flag;
  const int recomb = p->flag_recombinations;
  const int spin = p->flag_spin_temp;
  const double eff = p->reion_efficiency;
  const double unit_len = p->unit_length_cm, unit_mass = p->unit_mass_g, unit_time = c->unit_time_s;

  if (snapshot < 0 || snapshot >= c->n_snaps)
    return MX_ESTATE;
  const double redshift = c->zz[snapshot];
  const double prev_redshift = (snapshot == 0) ? c->zz[snapshot] : c->zz[snapshot - 1];
  const float zstep = (float)(prev_redshift - redshift);
  const float fabs_dtdz = (float)fabs(c_dtdz(c, (float)redshift) / p->hubble_h);

  if ((box_size / (double)D) < 1.0)
    cell_length_factor = 1.0;

  const size_t nreal = (size_t)D * D * D;
  if (uvb)
    for (size_t i = 0; i < nreal; i++)
      g->J_21[i] = 0.0f;
  for (size_t i = 0; i < nreal; i++) {
    g->xH[i] = 1.0f;
    g->r_bubble[i] = 0.0f;
  }
  c->margin = (float*)ctx_buf((void**)&c->margin, sizeof(float) * 2 * nreal);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < 2 * nreal; i++)
    c->margin[i] = INFINITY;

  /* fields: deltax, stars, weighted_sfr, [x_e], [N_rec] */
  enum { F_DX, F_ST, F_WS, F_XE, F_NR, F_N };
  const float* src[F_N] = { g->deltax, g->stars, g->weighted_sfr, spin ? g->x_e_box : NULL,
                            recomb ? g->N_rec : NULL };
  float* unf[F_N] = { 0 };
  float* fil[F_N] = { 0 };
  double tp = omp_get_wtime();
  for (int f = 0; f < F_N; f++) {
    if (!src[f])
      continue;
    unf[f] = (float*)ctx_buf((void**)&c->fhb_buf[2 * f], sizeof(float) * 2 * nc);
    fil[f] = (float*)ctx_buf((void**)&c->fhb_buf[2 * f + 1], sizeof(float) * 2 * nc);
    mxo_r2c_3d(D, src[f], 1, unf[f]);
    /* ×1/N: float complex /= double (find_HII_bubbles.c:168-182) */
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < 2 * nc; i++)
      unf[f][i] = (float)((double)unf[f][i] / total_n_cells);
  }

  const double Rmax = recomb ? p->r_bubble_max_recomb : p->r_bubble_max;
  double R = fmin(Rmax, K_L_FACTOR * box_size);
  int last = 0;
  int n_radii = 0;
  c->phase[MXO_PH_FORWARD] = omp_get_wtime() - tp;
  double t_radii = 0.0;
  while (!last) {
    tp = omp_get_wtime();
    if (c->sample_radii > 0 && n_radii == c->sample_radii)
      break; /* timing sample: the first sample_radii radii only */
    if (((R / p->delta_r_factor) <= (cell_length_factor * box_size / (double)D)) ||
        ((R / p->delta_r_factor) <= p->r_bubble_min)) {
      last = 1;
      R = cell_length_factor * box_size / (double)D;
    }
    n_radii++;
    for (int f = 0; f < F_N; f++) {
      if (!unf[f])
        continue;
      memcpy(fil[f], unf[f], sizeof(float) * 2 * nc);
      if (!last)
        c_filter(c, fil[f], D, (float)R, p->filter_type);
      mxo_c2r_3d(D, fil[f], fil[f]);
    }
    /* aliasing clamps, find_HII_bubbles.c:271-311 */
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ip = pad_idx(D, ix, iy, iz);
          fil[F_DX][ip] = fmaxf(fil[F_DX][ip], -1 + K_REL_TOL);
          for (int f = F_ST; f < F_N; f++) {
            if (!fil[f])
              continue;
            fil[f][ip] = fmaxf(fil[f][ip], 0.0);
            if (fil[f][ip] < K_ABS_TOL)
              fil[f][ip] = 0;
            if (f == F_XE)
              fil[f][ip] = fminf(fil[f][ip], 0.999);
          }
        }

    /* find_HII_bubbles.c:317-340 */
    const double J_21_aux_constant = (1.0 + redshift) * (1.0 + redshift) / (4.0 * M_PI) * p->alpha_uv * K_PLANCK *
                                     1e21 * R * unit_len * p->nion_phot_per_bary / K_PROTONMASS * unit_mass /
                                     pow(unit_len, 3) / unit_time;
    double Gamma_R_prefactor = 0.0;
    if (recomb) {
      Gamma_R_prefactor = (1.0 + redshift) * (1.0 + redshift) * R * (unit_len / p->hubble_h) * K_SIGMA_HI *
                          p->alpha_uv / (p->alpha_uv + 2.75) / 1.0e-12;
      Gamma_R_prefactor *= (unit_mass / unit_time) * pow(unit_len / p->hubble_h, -3.) * p->nion_phot_per_bary /
                           K_PROTONMASS;
    }
    const double M_mean = c_RtoM(c, R);
    const double R_cubed = R * R * R;

    /* threshold loop, find_HII_bubbles.c:342-443 (cells are independent) */
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ir = real_idx(D, ix, iy, iz);
          const size_t ip = pad_idx(D, ix, iy, iz);
          const double dom = 1.0 + (double)fil[F_DX][ip];
          const double f_coll_stars =
            (double)fil[F_ST][ip] / (M_mean * dom) * (4.0 / 3.0) * M_PI * R_cubed / pixel_volume;
          const double wsd = (double)fil[F_WS][ip] / pixel_volume;
          double rec = 0.0;
          if (recomb)
            rec = (double)fil[F_NR][ip] / dom;
          const double nf = spin ? 1.0 - fil[F_XE][ip] : 1.0;
          float J_21_aux = 0;
          if (uvb)
            J_21_aux = (float)(wsd * J_21_aux_constant);
          const double lhs = f_coll_stars * eff, rhs = nf * (1. + rec);
          const float mrel = (float)fabs(lhs / rhs - 1.0);
          if (g->xH[ir] > K_REL_TOL)
            c->margin[ir] = fminf(c->margin[ir], mrel);
          c->margin[nreal + ir] = fminf(c->margin[nreal + ir], mrel);
          if (lhs > rhs) {
            if (g->xH[ir] > K_REL_TOL) {
              if (uvb)
                g->J_21[ir] = J_21_aux;
              if (recomb)
                g->Gamma12[ir] = (float)(Gamma_R_prefactor * wsd);
            }
            g->xH[ir] = 0;
            g->r_bubble[ir] = (float)R;
          } else {
            if (last && (g->xH[ir] > K_REL_TOL)) {
              g->xH[ir] = (float)(nf - f_coll_stars * eff);
              if (g->xH[ir] < 0.)
                g->xH[ir] = (float)0.;
              else if (g->xH[ir] > 1.0)
                g->xH[ir] = (float)1.;
            }
          }
          if ((g->xH[ir] < K_REL_TOL) && (g->z_at_ionization[ir] < 0)) {
            g->z_at_ionization[ir] = (float)redshift;
            if (uvb)
              g->J_21_at_ionization[ir] = J_21_aux * (float)p->gamma_halo_bias;
          }
        }
    R /= p->delta_r_factor;
    if (n_radii > 1) /* the first radius also first touches the buffers */
      t_radii += omp_get_wtime() - tp;
  }

  c->phase[MXO_PH_RADII] = t_radii;
  c->phase[MXO_PH_N_RADII] = n_radii > 1 ? n_radii - 1 : 0;
  c->phase[MXO_PH_N_RADII_RUN] = n_radii;
  tp = omp_get_wtime();
  /* global means + N_rec, find_HII_bubbles.c:451-494: the N_rec update of
   * each cell in parallel, the sums in the reference's cell order */
  if (recomb) {
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ir = real_idx(D, ix, iy, iz);
          const size_t ip = pad_idx(D, ix, iy, iz);
          const double cell_xH = (double)g->xH[ir];
          const double dom = 1.0 + (double)g->deltax[ip];
          const float z_eff = (float)((1. + redshift) * pow(dom, 1.0 / 3.0) - 1);
          const double dNrec = c_rr_splined(c, z_eff, g->Gamma12[ir]) * fabs_dtdz * zstep * (1. - cell_xH);
          g->N_rec[ip] += dNrec;
        }
  }
  double vol_xH = 0.0, mass_xH = 0.0, mass_weight = 0.0, vol_J21 = 0.0;
  for (int ix = 0; ix < D; ix++)
    for (int iy = 0; iy < D; iy++)
      for (int iz = 0; iz < D; iz++) {
        const size_t ir = real_idx(D, ix, iy, iz);
        const size_t ip = pad_idx(D, ix, iy, iz);
        const double cell_xH = (double)g->xH[ir];
        vol_xH += cell_xH;
        if (uvb)
          vol_J21 += (double)g->J_21[ir];
        const double dom = 1.0 + (double)g->deltax[ip];
        mass_xH += cell_xH * dom;
        mass_weight += dom;
      }
  vol_xH /= total_n_cells;
  if (uvb)
    vol_J21 /= total_n_cells;
  mass_xH /= mass_weight;
  c->phase[MXO_PH_FHB_POST] = omp_get_wtime() - tp;
  if (out) {
    out->volume_weighted_global_xH = vol_xH;
    out->volume_weighted_global_J_21 = vol_J21;
    out->mass_weighted_global_xH = mass_xH;
    out->n_radii = n_radii;
  }
  return 0;
}

/* ======================================================= X-ray / spin temp */

static double c_T_RECFAST(const mxo_ctx* c, float z)
{
  if (z > c->recfast_zmax)
    return -1;
  return mxo_spline_eval(&c->recfast_T, z);
}
static double c_xion_RECFAST(const mxo_ctx* c, float z)
{
  if (z > c->recfast_zmax)
    return -1;
  return mxo_spline_eval(&c->recfast_x, z);
}

/* cross sections, XRayHeatingFunctions.c:420-460 */
static double c_HeI_xs(double nu)
{
  if (nu < K_NU_HEI)
    return 0;
  const double x = nu / K_NU_OVER_EV / 13.61 - 0.4434;
  const double y = sqrt(x * x + pow(2.136, 2));
  return 9.492e-16 * ((x - 1) * (x - 1) + 2.039 * 2.039) * pow(y, (0.5 * 3.188 - 5.5)) *
         pow(1.0 + sqrt(y / 1.469), -3.188);
}
static double c_HeII_xs(double nu)
{
  const double Z = 2;
  if (nu < K_NU_HEII)
    return 0;
  if (nu == K_NU_HEII)
    nu += K_TINY;
  const double eps = sqrt(nu / K_NU_HEII - 1);
  return (6.3e-18) / Z / Z * pow(K_NU_HEII / nu, 4) * exp(4 - (4 * atan(eps) / eps)) / (1 - exp(-2 * M_PI / eps));
}
static double c_HI_xs(double nu)
{
  const double Z = 1;
  if (nu < K_NU_HI)
    return 0;
  if (nu == K_NU_HI)
    nu += K_TINY;
  const double eps = sqrt(nu / K_NU_HI - 1);
  return K_SIGMA_HI / Z / Z * pow(K_NU_HI / nu, 4) * exp(4 - (4 * atan(eps) / eps)) / (1 - exp(-2 * M_PI / eps));
}
static double c_species_xs(const mxo_ctx* c, double nu, double x_e)
{
  return c->f_h * (1 - x_e) * c_HI_xs(nu) + c->f_he * (1 - x_e) * c_HeI_xs(nu) + c->f_he * x_e * c_HeII_xs(nu);
}

/* interpolate_fcoll, XRayHeatingFunctions.c:1884-1917 (Pop II) */
static double c_interp_fcoll(const mxo_ctx* c, double redshift, int snap_i)
{
  double v;
  if (snap_i == 0)
    v = c->stored_fcoll[snap_i];
  else
    v = c->stored_fcoll[snap_i - 1] + (redshift - c->zz[snap_i - 1]) *
                                        (c->stored_fcoll[snap_i] - c->stored_fcoll[snap_i - 1]) /
                                        (c->zz[snap_i] - c->zz[snap_i - 1]);
  if (v < 0.0)
    v = 0.0;
  return v;
}

typedef struct
{
  const mxo_ctx* c;
  double nu_0, x_e, ion_eff;
  int snap_i;
} taux_par;

/* tauX_integrand, XRayHeatingFunctions.c:307-344 */
static double f_taux(double zhat, void* vp)
{
  const taux_par* p = (const taux_par*)vp;
  const mxo_ctx* c = p->c;
  const double drpropdz = K_C * c_dtdz(c, (float)zhat);
  const double n = c->n_b0 * pow(1 + zhat, 3);
  const double nuhat = p->nu_0 * (1 + zhat);
  const double fcoll = c_interp_fcoll(c, zhat, p->snap_i);
  double HI;
  if (fcoll < 1e-20)
    HI = 1;
  else
    HI = 1 - (p->ion_eff * fcoll) / (1.0 - c->x_e_ave);
  if (HI < 1e-4)
    HI = 1e-4;
  return drpropdz * n * HI * c_species_xs(c, nuhat, p->x_e);
}

/* tauX, XRayHeatingFunctions.c:345-375 */
static double c_tauX(const mxo_ctx* c, double nu, double x_e, double zp, double zpp, int snap_i)
{
  taux_par tp = { c, nu / (1 + zp), x_e, c->p.reion_efficiency, snap_i };
  double res, err;
  mxo_qag61(f_taux, &tp, zpp, zp, 0, 0.005, 1000, &res, &err);
  return res;
}

typedef struct
{
  const mxo_ctx* c;
  double x_e, zp, zpp;
  int snap_i;
} ntau_par;
static double f_ntau(double nu, void* vp)
{
  const ntau_par* p = (const ntau_par*)vp;
  return c_tauX(p->c, nu, p->x_e, p->zp, p->zpp, p->snap_i) - 1;
}

/* nu_tau_one, XRayHeatingFunctions.c:229-297 */
static double c_nu_tau_one(const mxo_ctx* c, double zp, double zpp, double x_e, int snap_i)
{
  if (x_e > 0.9999)
    return -1;
  if (c_tauX(c, K_NU_HEI, x_e, zp, zpp, snap_i) < 1)
    return K_NU_HEI;
  ntau_par np = { c, x_e, zp, zpp, snap_i };
  mxo_brent s;
  double x_lo = K_NU_HEI, x_hi = 1e6 * K_NU_OVER_EV, r = 0;
  mxo_brent_set(&s, f_ntau, &np, x_lo, x_hi);
  int iter = 0, status;
  do {
    iter++;
    mxo_brent_iterate(&s);
    r = s.root;
    x_lo = s.x_lower;
    x_hi = s.x_upper;
    status = mxo_root_test_interval(x_lo, x_hi, 0, 0.02);
  } while (status == 1 && iter < 100);
  return r;
}

/* locate_energy_index / locate_xHII_index, XRayHeatingFunctions.c:1193-1219 */
static int c_loc_energy(float En)
{
  if (En < 1008.88)
    return (int)(log(En / 10.0) / 1.98026273e-2);
  return 232 + (int)(log(En / 1008.88) / 9.53101798e-2);
}
static int c_loc_xhii(const mxo_ctx* c, float x)
{
  int m = K_NXHII - 1;
  while (x < c->x_xhii[m])
    m--;
  return m;
}

/* interp_fheat / interp_n_Lya / interp_nion_*, XRayHeatingFunctions.c:914-1190:
 * bilinear in (energy, x_HII) with float arithmetic. */
static float c_interp_tab(const mxo_ctx* c, const float (*tab)[K_NENERGY], float below, float En, float xHII_call)
{
  if (En > 0.999 * c->x_energy[K_NENERGY - 1])
    En = (float)(c->x_energy[K_NENERGY - 1] * 0.999);
  else if (En < c->x_energy[0])
    return below;
  if (xHII_call > c->x_xhii[K_NXHII - 1] * 0.999)
    xHII_call = (float)(c->x_xhii[K_NXHII - 1] * 0.999);
  else if (xHII_call < c->x_xhii[0])
    xHII_call = (float)(1.001 * c->x_xhii[0]);
  const int n_low = c_loc_energy(En), n_high = n_low + 1;
  const int m_low = c_loc_xhii(c, xHII_call), m_high = m_low + 1;
  const float* E = c->x_energy;
  float elow = ((tab[m_low][n_high] - tab[m_low][n_low]) / (E[n_high] - E[n_low]));
  elow *= (En - E[n_low]);
  elow += tab[m_low][n_low];
  float ehigh = ((tab[m_high][n_high] - tab[m_high][n_low]) / (E[n_high] - E[n_low]));
  ehigh *= (En - E[n_low]);
  ehigh += tab[m_high][n_low];
  float fin = (ehigh - elow) / (c->x_xhii[m_high] - c->x_xhii[m_low]);
  fin *= (xHII_call - c->x_xhii[m_low]);
  fin += elow;
  return fin;
}

typedef struct
{
  const mxo_ctx* c;
  double x_e, thresh, alpha;
} nu_par;

/* integrand_in_nu_heat_integral, XRayHeatingFunctions.c:672-695 */
static double f_nu_heat(double nu, void* vp)
{
  const nu_par* p = (const nu_par*)vp;
  const mxo_ctx* c = p->c;
  const float xe = (float)p->x_e;
  double s = c_interp_tab(c, c->x_fheat, 1.0f, (float)((nu - K_NU_HI) / K_NU_OVER_EV), xe) * K_PLANCK *
             (nu - K_NU_HI) * c->f_h * (1 - p->x_e) * c_HI_xs(nu);
  s += c_interp_tab(c, c->x_fheat, 1.0f, (float)((nu - K_NU_HEI) / K_NU_OVER_EV), xe) * K_PLANCK * (nu - K_NU_HEI) *
       c->f_he * (1 - p->x_e) * c_HeI_xs(nu);
  s += c_interp_tab(c, c->x_fheat, 1.0f, (float)((nu - K_NU_HEII) / K_NU_OVER_EV), xe) * K_PLANCK *
       (nu - K_NU_HEII) * c->f_he * p->x_e * c_HeII_xs(nu);
  return s * pow(nu / (p->thresh * K_NU_OVER_EV), -p->alpha - 1);
}

/* integrand_in_nu_ion_integral, XRayHeatingFunctions.c:697-723 */
static double f_nu_ion(double nu, void* vp)
{
  const nu_par* p = (const nu_par*)vp;
  const mxo_ctx* c = p->c;
  const float xe = (float)p->x_e;
  const double nus[3] = { K_NU_HI, K_NU_HEI, K_NU_HEII };
  double s = 0;
  for (int k = 0; k < 3; k++) {
    const float En = (float)((nu - nus[k]) / K_NU_OVER_EV);
    const double F_i = c_interp_tab(c, c->x_nion_hi, 0.0f, En, xe) + c_interp_tab(c, c->x_nion_hei, 0.0f, En, xe) +
                       c_interp_tab(c, c->x_nion_heii, 0.0f, En, xe) + 1;
    if (k == 0)
      s = F_i * c->f_h * (1 - p->x_e) * c_HI_xs(nu);
    else if (k == 1)
      s += F_i * c->f_he * (1 - p->x_e) * c_HeI_xs(nu);
    else
      s += F_i * c->f_he * p->x_e * c_HeII_xs(nu);
  }
  return s * pow(nu / (p->thresh * K_NU_OVER_EV), -p->alpha - 1);
}

/* integrand_in_nu_lya_integral, XRayHeatingFunctions.c:725-744 */
static double f_nu_lya(double nu, void* vp)
{
  const nu_par* p = (const nu_par*)vp;
  const mxo_ctx* c = p->c;
  const float xe = (float)p->x_e;
  double s = c_interp_tab(c, c->x_nlya, 0.0f, (float)((nu - K_NU_HI) / K_NU_OVER_EV), xe) * c->f_h * (1 - p->x_e) *
             c_HI_xs(nu);
  s += c_interp_tab(c, c->x_nlya, 0.0f, (float)((nu - K_NU_HEI) / K_NU_OVER_EV), xe) * c->f_he * (1 - p->x_e) *
       c_HeI_xs(nu);
  s += c_interp_tab(c, c->x_nlya, 0.0f, (float)((nu - K_NU_HEII) / K_NU_OVER_EV), xe) * c->f_he * p->x_e *
       c_HeII_xs(nu);
  return s * pow(nu / (p->thresh * K_NU_OVER_EV), -p->alpha - 1);
}

/* integrate_over_nu, XRayHeatingFunctions.c:746-800 */
static double c_integrate_over_nu(const mxo_ctx* c, double zp, double local_x_e, double lower, int flag)
{
  nu_par np = { c, local_x_e, c->p.nu_xray_gal_threshold, c->p.spec_index_xray_gal };
  mxo_fn fn = flag == 0 ? f_nu_heat : (flag == 1 ? f_nu_ion : f_nu_lya);
  double res, err;
  mxo_qag61(fn, &np, lower, c->p.nu_xray_max * K_NU_OVER_EV, 0, 0.01, 1000, &res, &err);
  if (flag == 2)
    return res * K_C / (4 * M_PI) / K_LYA_HZ / c_hubble(c, (float)zp);
  return res;
}

/* zmax / nu_n / frecycle / spectral_emissivity, XRayHeatingFunctions.c:477-584, 632-670 */
static float c_zmax(float z, int n)
{
  const double num = 1 - pow(n + 1, -2);
  const double denom = 1 - pow(n, -2);
  return (float)((1 + z) * num / denom - 1);
}
static double c_nu_n(int n) { return (1.0 - pow(n, -2.0)) / 0.75; }
static double c_frecycle(int n)
{
  static const double t[31] = { 1,      1,      1,      0,      0.2609, 0.3078, 0.3259, 0.3353, 0.3410, 0.3448, 0.3476,
                                0.3496, 0.3512, 0.3524, 0.3535, 0.3543, 0.3550, 0.3556, 0.3561, 0.3565, 0.3569, 0.3572,
                                0.3575, 0.3578, 0.3580, 0.3582, 0.3584, 0.3586, 0.3587, 0.3589, 0.3590 };
  return (n >= 0 && n <= 30) ? t[n] : 0;
}
static double c_spectral_emissivity(const mxo_ctx* c, double nu_norm)
{
  for (int i = 1; i < (K_NSPEC_MAX - 1); i++)
    if ((nu_norm >= c->spec_nu[i]) && (nu_norm < c->spec_nu[i + 1]))
      return c->spec_N0[i] * pow(nu_norm, c->spec_alpha[i]) / K_LYA_HZ;
  const int i = K_NSPEC_MAX - 1;
  return c->spec_N0[i] * pow(nu_norm, c->spec_alpha[i]) / K_LYA_HZ;
}

/* dT_comp, XRayHeatingFunctions.c:1437-1448 */
static double c_dT_comp(const mxo_ctx* c, double z, double TK, double xe)
{
  const double Trad = K_TCMB * (1.0 + z);
  double ans = (-1.51e-4) * (xe / (1.0 + xe + c->f_he)) / (c_hubble(c, (float)z) / (K_HUBBLE * c->p.hubble_h)) /
               c->p.hubble_h * pow(Trad, 4.0) / (1.0 + z);
  ans *= Trad - TK;
  return ans;
}

/* kappa_10 / kappa_10_elec / kappa_10_pH, XRayHeatingFunctions.c:1686-1695, 1755-1766, 1827-1839 */
static double c_kappa_10(const mxo_ctx* c, double TK)
{
  double ans;
  const int n = K_KAPPA_10_NPTS;
  if (log(TK) < c->kap10_t[0])
    ans = c->kap10_k[0];
  else if (log(TK) > c->kap10_t[n - 1])
    ans = log(exp(c->kap10_k[n - 1]) * pow(TK / exp(c->kap10_t[n - 1]), 0.381));
  else
    ans = mxo_spline_eval(&c->kap10, log(TK));
  return exp(ans);
}
static double c_kappa_tab(const mxo_spline* sp, const double* t, const double* k, int n, double T)
{
  double ans;
  T = log(T);
  if (T < t[0])
    ans = k[0];
  else if (T > t[n - 1])
    ans = k[n - 1] + ((k[n - 1] - k[n - 2]) / (t[n - 1] - t[n - 2]) * (T - t[n - 1]));
  else
    ans = mxo_spline_eval(sp, T);
  return exp(ans);
}

/* xcoll and helpers, XRayHeatingFunctions.c:1560-1600 */
static double c_xcoll(const mxo_ctx* c, double z, double TK, double delta, double xe)
{
  const double Trad = K_TCMB * (1.0 + z);
  const double nH = (1.0 - xe) * c->no * pow(1.0 + z, 3.0) * (1.0 + delta);
  const double x_hi = K_T21 / Trad * nH * c_kappa_10(c, TK) / K_A10;
  const double ne = xe * c->n_b0 * pow(1.0 + z, 3.0) * (1.0 + delta);
  const double x_el =
    K_T21 / Trad * ne * c_kappa_tab(&c->kap_e, c->kap_e_t, c->kap_e_k, K_KAPPA_E_NPTS, TK) / K_A10;
  const double np = xe * c->no * pow(1.0 + z, 3.0) * (1.0 + delta);
  const double x_pr =
    K_T21 / Trad * np * c_kappa_tab(&c->kap_p, c->kap_p_t, c->kap_p_k, K_KAPPA_P_NPTS, TK) / K_A10;
  return x_hi + x_el + x_pr;
}

/* get_Ts, XRayHeatingFunctions.c:1513-1558 with xalpha_tilde / taugp /
 * Salpha_tilde / Tc_eff at :1847-1882 */
static float c_get_Ts(const mxo_ctx* c, float z, float delta, float TK, float xe, float Jalpha, float* curr_xalpha)
{
  const double Trad = K_TCMB * (1.0 + z);
  const double xc = c_xcoll(c, z, TK, delta, xe);
  double TS, TSold, TSinv, xa_tilde = 0, Tceff;
  if (Jalpha > 1.0e-20) {
    TS = Trad;
    TSold = 0.0;
    while (fabs(TS - TSold) / TS > 1.0e-3) {
      TSold = TS;
      const double tgp =
        1.342881e-7 / c_hubble(c, (float)z) * c->no * pow(1 + (double)z, 3) * (1.0 + (double)delta) * (1.0 - (double)xe);
      const double xi = pow(1.0e-7 * tgp / TK / TK, 1.0 / 3.0);
      double St = 1.0 - 0.0631789 / TK + 0.115995 / TK / TK - 0.401403 / TS / TK;
      St += 0.336463 / TS / TK / TK;
      St /= 1.0 + 2.98394 * xi + 1.53583 * xi * xi + 3.85289 * xi * xi * xi;
      xa_tilde = 1.66e11 / (1.0 + z) * St * Jalpha;
      Tceff = 1.0 / (1.0 / TK + 0.405535 / TK * (1.0 / TS - 1.0 / TK));
      TSinv = (1.0 / Trad + xa_tilde / Tceff + xc / TK) / (1.0 + xa_tilde + xc);
      TS = 1.0 / TSinv;
    }
    *curr_xalpha = (float)xa_tilde;
  } else {
    TSinv = (1.0 / Trad + xc / TK) / (1.0 + xc);
    TS = 1.0 / TSinv;
    *curr_xalpha = 0;
  }
  if (TS < 0.)
    TS = fabs(TS);
  return (float)TS;
}

double mxo_get_Ts(mxo_ctx* c, float z, float delta, float TK, float xe, float Jalpha, float* xalpha)
{
  return c_get_Ts(c, z, delta, TK, xe, Jalpha, xalpha);
}

/* evolveInt (no mini-halos), XRayHeatingFunctions.c:1241-1435 */
static void c_evolve(const mxo_ctx* c,
                     float zp,
                     float curr_delNL0,
                     const double* SFR,
                     const double* fheat,
                     const double* fion,
                     const double* flya,
                     int NO_LIGHT,
                     const double* y,
                     double* deriv)
{
  const int S = c->p.ts_num_filter_steps;
  const double Conversion_factor = (K_C / (4. * M_PI)) / (K_PROTONMASS / K_SOLAR_MASS);
  const double x_e = y[0], T = y[1];
  const double n_b = c->n_b0 * pow(1 + zp, 3) * (1 + curr_delNL0);
  double dxheat_dt = 0, dxion_source_dt = 0, dxlya_dt = 0, dstarlya_dt = 0;
  if (!NO_LIGHT) {
    for (int k = 0; k < S; k++) {
      double zpp, dzpp;
      if (k == 0) {
        zpp = (c->zpp_edge[0] + zp) * 0.5;
        dzpp = zp - c->zpp_edge[0];
      } else {
        zpp = (c->zpp_edge[k] + c->zpp_edge[k - 1]) * 0.5;
        dzpp = c->zpp_edge[k - 1] - c->zpp_edge[k];
      }
      const double dt_dzpp = c_dtdz(c, (float)zpp);
      const double integrand = SFR[k] * pow(1 + zpp, -c->p.spec_index_xray_gal);
      dxheat_dt += dt_dzpp * dzpp * integrand * fheat[k];
      dxion_source_dt += dt_dzpp * dzpp * integrand * fion[k];
      dxlya_dt += dt_dzpp * dzpp * integrand * flya[k];
      dstarlya_dt += SFR[k] * pow(1 + zp, 2) * (1 + zpp) * c->sum_lyn[k] * dt_dzpp * dzpp;
    }
    dxheat_dt *= c->const_zp_prefactor;
    dxion_source_dt *= c->const_zp_prefactor;
    dxlya_dt *= c->const_zp_prefactor * n_b;
    dstarlya_dt *= Conversion_factor;
  }
  const double dxion_sink_dt = c_alpha_A(T) * c->p.clumping_factor * x_e * x_e * c->f_h * n_b;
  const double dxe_dzp = c->dt_dzp * (dxion_source_dt - dxion_sink_dt);
  deriv[0] = dxe_dzp;
  double dadia_dzp = 3 / (1.0 + zp);
  if (fabs(curr_delNL0) > K_FRACT_FLOAT_ERR)
    dadia_dzp += c->dgrowth_dzp / (1.0 / curr_delNL0 + c->growth_zp);
  dadia_dzp *= (2.0 / 3.0) * T;
  const double dspec_dzp = -dxe_dzp * T / (1 + x_e);
  const double dcomp_dzp = c_dT_comp(c, zp, T, x_e);
  const double dxheat_dzp = dxheat_dt * c->dt_dzp * 2.0 / 3.0 / K_BOLTZMANN / (1.0 + x_e);
  deriv[1] = dxheat_dzp + dcomp_dzp + dspec_dzp + dadia_dzp;
  deriv[2] = dxlya_dt + dstarlya_dt;
  deriv[3] = dxheat_dzp;
  deriv[4] = c->dt_dzp * dxion_source_dt;
}

/* load_reion_sfr_grids, reionization.c:1756-1784 (REAL indexing into the
 * stored slice, PADDED indexing into sfr) */
static void c_load_sfr(const mxo_ctx* c, const mx_grids* g, int scb, float weight, int new_load)
{
  const int D = c->p.grid_dim;
  const size_t nc2 = (size_t)D * D * (D / 2 + 1) * 2;
  const float* h = g->sfr_histories + (size_t)scb * nc2;
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++)
      for (int k = 0; k < D; k++) {
        const size_t ip = pad_idx(D, i, j, k);
        const float v = h[real_idx(D, i, j, k)] * weight;
        if (new_load)
          g->sfr[ip] = v;
        else
          g->sfr[ip] += v;
      }
}

/* _ComputeTs, ComputeTs.c:78-1020 (no mini-halos) */
int mxo_ComputeTs(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out)
{
  const mx_params* p = &c->p;
  if (!c->heat_ready)
    return MX_ESTATE;
  if (snapshot < 0 || snapshot >= c->n_snaps)
    return MX_ESTATE;
  const double box_size = p->box_size / p->hubble_h;
  const int D = p->grid_dim;
  const int H = D / 2 + 1;
  const size_t nc = (size_t)D * D * H;
  const double pixel_volume = pow(box_size / (double)D, 3);
  const double total_n_cells = pow((double)D, 3);
  const double eff = p->reion_efficiency;
  const int S = p->ts_num_filter_steps;
  const double redshift = c->zz[snapshot];
  const double prev_redshift = (snapshot == 0) ? c->zz[snapshot] : c->zz[snapshot - 1];
  const double sfr_unit = (p->unit_mass_g / c->unit_time_s) * pow(p->unit_length_cm, -3.) / K_SOLAR_MASS;
  float curr_xalpha;
  size_t i_padded = 0;

  free(c->zpp_edge);
  free(c->sum_lyn);
  free(c->freq_tables);
  c->zpp_edge = (double*)calloc((size_t)S, sizeof(double));
  c->sum_lyn = (double*)calloc((size_t)S, sizeof(double));
  c->freq_tables = (double*)calloc((size_t)3 * K_NXHII * S, sizeof(double));
  c->x_e_ave = 0.0;

  double J_alpha_ave = 0, xalpha_ave = 0, Xheat_ave = 0, Xion_ave = 0;
  const double zp = redshift;
  const double dzp = zp - prev_redshift;
  c->dt_dzp = c_dtdz(c, (float)(float)zp);
  double collapse_fraction = 0.;

  if ((zp - p->max_heating_redshift) >= -0.0001) {
    /* homogeneous branch, ComputeTs.c:189-262 */
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ir = real_idx(D, ix, iy, iz);
          i_padded = pad_idx(D, ix, iy, iz);
          g->x_e_box_prev[i_padded] = (float)(float)c_xion_RECFAST(c, (float)zp);
          g->Tk_box[ir] = (float)(float)c_T_RECFAST(c, (float)zp);
          g->TS_box[ir] = c_get_Ts(c, (float)zp, g->deltax[i_padded], g->Tk_box[ir], g->x_e_box_prev[i_padded], 0,
                                   &curr_xalpha);
        }
    const double R = K_L_FACTOR * box_size / (float)D;
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          i_padded = pad_idx(D, ix, iy, iz);
          const double dom = 1.0 + g->deltax[i_padded];
          double cf = g->stars[i_padded] / (c_RtoM(c, R) * p->hubble_h * p->hubble_h * dom) * (4.0 / 3.0) * M_PI *
                      pow(R, 3.0) / pixel_volume;
          if (cf > 1.0)
            cf = 1.0;
          collapse_fraction += cf;
        }
    collapse_fraction = collapse_fraction / total_n_cells;
  } else {
    /* shells, ComputeTs.c:270-503 */
    double R = K_L_FACTOR * box_size / (float)D;
    const double R_factor = pow(K_R_XLY_MAX / R, 1 / (float)S);
    double* R_values = (double*)malloc(sizeof(double) * (size_t)S);
    int* scb = (int*)malloc(sizeof(int) * (size_t)S);
    if (c->smoothed && c->ts_buf[0] && S > c->ts_shells) {
      free(c->smoothed);
      c->smoothed = NULL;
    }
    double* smoothed = (double*)ctx_buf((void**)&c->smoothed, sizeof(double) * (size_t)S * D * D * D);
    c->ts_shells = S;
    float* unf = (float*)ctx_buf((void**)&c->ts_buf[0], sizeof(float) * 2 * nc);
    float* fil = (float*)ctx_buf((void**)&c->ts_buf[1], sizeof(float) * 2 * nc);
    const double* ZZ = c->zz;
    double weight = 1;
    scb[0] = 1;
    double tp = omp_get_wtime(), t_shells = 0.0, t_copies = 0.0;
    int n_shells_done = 0;
    for (int R_ct = 0; R_ct < S; R_ct++) {
      double prev_zpp, prev_R;
      R_values[R_ct] = R;
      if (R_ct == 0) {
        prev_zpp = zp;
        prev_R = 0;
      } else {
        prev_zpp = c->zpp_edge[R_ct - 1];
        prev_R = R_values[R_ct - 1];
        scb[R_ct] = scb[R_ct - 1];
      }
      c->zpp_edge[R_ct] = prev_zpp - (R - prev_R) * K_MPC / (c_drdz(c, (float)prev_zpp));
      const double zpp = (c->zpp_edge[R_ct] + prev_zpp) * 0.5;
      const double total_weight = (prev_zpp - c->zpp_edge[R_ct]) * c_dtdz(c, (float)zpp);

      /* SFR-history reweighting, ComputeTs.c:288-377 */
      if (snapshot - scb[R_ct] >= 0) {
        if (snapshot - scb[R_ct] == 0 && weight < 0) {
          for (size_t ii = 0; ii < nc; ii++)
            g->sfr[ii] = 0;
          scb[R_ct] += 1;
        } else if (c->zpp_edge[R_ct] > ZZ[snapshot - scb[R_ct]]) {
          if (R_ct == 0) {
            weight = c->dt_dzp * dzp / total_weight;
            for (size_t ii = 0; ii < nc; ii++)
              g->sfr[ii] *= weight;
          } else {
            if (ZZ[snapshot - scb[R_ct]] > c->zpp_edge[R_ct - 1]) {
              weight = -c_dtdz(c, (float)(0.5 * (ZZ[snapshot - scb[R_ct]] + c->zpp_edge[R_ct - 1])));
              weight *= (ZZ[snapshot - scb[R_ct]] - c->zpp_edge[R_ct - 1]);
              weight /= total_weight;
              c_load_sfr(c, g, scb[R_ct] - 1, (float)weight, 1);
            } else {
              for (size_t ii = 0; ii < nc; ii++)
                g->sfr[ii] = 0;
            }
          }
          while (c->zpp_edge[R_ct] > ZZ[snapshot - scb[R_ct]]) {
            if (snapshot - scb[R_ct] == 0) {
              weight = -1;
              break;
            }
            if (c->zpp_edge[R_ct] < ZZ[snapshot - scb[R_ct] - 1]) {
              /* the ternary of ComputeTs.c:345 as written */
              const double zprev = R_ct > 0 ? c->zpp_edge[R_ct - 1] : 0.0;
              const double zedge = zprev ? ZZ[snapshot - scb[R_ct]] : (double)(zprev > ZZ[snapshot - scb[R_ct]]);
              weight = c->zpp_edge[R_ct] - zedge;
              weight *= -c_dtdz(c, (float)(0.5 * (c->zpp_edge[R_ct] + zedge)));
            } else {
              weight = ZZ[snapshot - scb[R_ct] - 1] - ZZ[snapshot - scb[R_ct]];
              weight *= -c_dtdz(c, (float)(0.5 * (ZZ[snapshot - scb[R_ct] - 1] + ZZ[snapshot - scb[R_ct]])));
            }
            weight /= total_weight;
            c_load_sfr(c, g, scb[R_ct], (float)weight, 0);
            scb[R_ct] += 1;
          }
        } else {
          if (R_ct > 0 && weight != 1) {
            weight = 1;
            c_load_sfr(c, g, scb[R_ct] - 1, (float)weight, 1);
          }
        }
      }

      if (c->sample_shells > 0 && R_ct >= c->sample_shells) {
        /* timing sample: this shell repeats a smoothed one (the per-cell
         * work below still reads every shell) */
        const int from = R_ct % c->sample_shells;
        const double t0 = omp_get_wtime();
        /* only the cells that the sampled per-cell step reads */
        const size_t n_read = (size_t)(c->sample_cell_div > 1 ? D / c->sample_cell_div : D) * D * D;
#pragma omp parallel for schedule(static)
        for (size_t ir = 0; ir < n_read; ir++)
          smoothed[(size_t)R_ct + (size_t)S * ir] = smoothed[(size_t)from + (size_t)S * ir];
        t_copies += omp_get_wtime() - t0;
        R *= R_factor;
        continue;
      }
      n_shells_done++;
      const double t_shell0 = omp_get_wtime();
      /* R2C, ×1/N (float division), filter, C2R: ComputeTs.c:379-409 */
      mxo_r2c_3d(D, g->sfr, 1, unf);
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < 2 * nc; i++)
        unf[i] = unf[i] / (float)total_n_cells;
      memcpy(fil, unf, sizeof(float) * 2 * nc);
      if (R_ct > 0)
        c_filter(c, fil, D, (float)R, p->ts_heating_filter_type);
      mxo_c2r_3d(D, fil, fil);

      /* ComputeTs.c:413-500 (stores in parallel, sums in the reference order) */
#pragma omp parallel for schedule(static)
      for (int ix = 0; ix < D; ix++)
        for (int iy = 0; iy < D; iy++)
          for (int iz = 0; iz < D; iz++) {
            const size_t ip = pad_idx(D, ix, iy, iz);
            const size_t ir = real_idx(D, ix, iy, iz);
            fil[ip] = fmaxf(fil[ip], 0.0);
            smoothed[(size_t)R_ct + (size_t)S * ir] = ((fil[ip] / pixel_volume) * sfr_unit);
          }
      if (R_ct == 0)
        for (int ix = 0; ix < D; ix++)
          for (int iy = 0; iy < D; iy++)
            for (int iz = 0; iz < D; iz++) {
              const size_t ip = pad_idx(D, ix, iy, iz);
              const double dom = 1.0 + g->deltax[ip];
              double cf = g->stars[ip] / (c_RtoM(c, R) * p->hubble_h * p->hubble_h * dom) * (4.0 / 3.0) * M_PI *
                          pow(R, 3.0) / pixel_volume;
              if (cf > 1.0)
                cf = 1.0;
              collapse_fraction += cf;
              c->x_e_ave += g->x_e_box_prev[ip];
            }
      if (R_ct == 0) {
        collapse_fraction = collapse_fraction / total_n_cells;
        c->x_e_ave = c->x_e_ave / total_n_cells;
        c->stored_fcoll[snapshot] = collapse_fraction;
      } else { /* shell 0 also first touches the buffers */
        t_shells += omp_get_wtime() - t_shell0;
      }
      R *= R_factor;
    }
    const int NO_LIGHT = (collapse_fraction > 0.0) ? 0 : 1;
    c->phase[MXO_PH_SHELLS] = t_shells;
    c->phase[MXO_PH_N_SHELLS] = n_shells_done > 1 ? n_shells_done - 1 : 0;
    c->phase[MXO_PH_N_SHELLS_RUN] = n_shells_done;
    c->phase[MXO_PH_SHELL_COPIES] = t_copies;
    (void)tp;
    tp = omp_get_wtime();

    /* frequency-integral tables and Ly-n sums, ComputeTs.c:517-663 */
    int first_radii = 1, first_zero = 1;
    const int n_pts_radii = 1000;
    double* tH = c->freq_tables;
    double* tI = c->freq_tables + (size_t)K_NXHII * S;
    double* tL = c->freq_tables + (size_t)2 * K_NXHII * S;
    /* the integrals of different shells are independent */
#pragma omp parallel for schedule(dynamic, 1)
    for (int R_ct = 0; R_ct < S; R_ct++) {
      const double prev_zpp = R_ct == 0 ? zp : c->zpp_edge[R_ct - 1];
      const double zpp = (c->zpp_edge[R_ct] + prev_zpp) * 0.5;
      const double lower = fmax(c_nu_tau_one(c, zp, zpp, c->x_e_ave, snapshot), p->nu_xray_gal_threshold * K_NU_OVER_EV);
      for (int x = 0; x < K_NXHII; x++) {
        tH[(size_t)x * S + R_ct] = c_integrate_over_nu(c, zp, c->x_xhii[x], lower, 0);
        tI[(size_t)x * S + R_ct] = c_integrate_over_nu(c, zp, c->x_xhii[x], lower, 1);
        tL[(size_t)x * S + R_ct] = c_integrate_over_nu(c, zp, c->x_xhii[x], lower, 2);
      }
    }
    for (int R_ct = 0; R_ct < S; R_ct++) {
      double prev_zpp, prev_R;
      if (R_ct == 0) {
        prev_zpp = zp;
        prev_R = 0;
      } else {
        prev_zpp = c->zpp_edge[R_ct - 1];
        prev_R = R_values[R_ct - 1];
      }
      const double zpp = (c->zpp_edge[R_ct] + prev_zpp) * 0.5;
      c->sum_lyn[R_ct] = 0;
      for (int n_ct = K_NSPEC_MAX; n_ct >= 2; n_ct--) {
        if (zpp > c_zmax((float)zp, n_ct))
          continue;
        const double nuprime = c_nu_n(n_ct) * (1 + zpp) / (1.0 + zp);
        c->sum_lyn[R_ct] += c_frecycle(n_ct) * c_spectral_emissivity(c, nuprime);
      }
      if (R_ct > 2 && c->sum_lyn[R_ct] == 0.0 && c->sum_lyn[R_ct - 1] > 0. && first_radii) {
        const double trial_zpp_max =
          (prev_zpp - (R_values[R_ct] - prev_R) * K_MPC / c_drdz(c, (float)prev_zpp) + prev_zpp) * 0.5;
        const double trial_zpp_min = (c->zpp_edge[R_ct - 2] -
                                      (R_values[R_ct - 1] - R_values[R_ct - 2]) * K_MPC /
                                        c_drdz(c, (float)c->zpp_edge[R_ct - 2]) +
                                      c->zpp_edge[R_ct - 2]) *
                                     0.5;
        for (int ii = 0; ii < n_pts_radii; ii++) {
          const double trial_zpp =
            trial_zpp_min + (trial_zpp_max - trial_zpp_min) * (float)ii / ((float)n_pts_radii - 1.);
          int counter = 0;
          for (int n_ct = K_NSPEC_MAX; n_ct >= 2; n_ct--) {
            if (trial_zpp > c_zmax((float)zp, n_ct))
              continue;
            counter += 1;
          }
          if (counter == 0 && first_zero) {
            first_zero = 0;
            weight = (float)ii / (float)n_pts_radii;
          }
        }
        c->sum_lyn[R_ct] = weight * c->sum_lyn[R_ct - 1];
        first_radii = 0;
      }
    }

    c->phase[MXO_PH_TABLES] = omp_get_wtime() - tp;
    tp = omp_get_wtime();
    c->growth_zp = c_dicke(c, zp);
    c->dgrowth_dzp = c_ddicke_dz(c, zp);
    c->dt_dzp = c_dtdz(c, (float)zp);
    /* luminosity conversion, ComputeTs.c:675-724 */
    const double E0 = p->nu_xray_gal_threshold, alpha = p->spec_index_xray_gal;
    double Lconv;
    if (fabs(alpha - 1.0) < 0.000001) {
      Lconv = (E0 * K_NU_OVER_EV) * log(p->nu_xray_soft_cut / E0);
      Lconv = 1. / Lconv;
    } else {
      Lconv = pow(p->nu_xray_soft_cut * K_NU_OVER_EV, 1. - alpha) - pow(E0 * K_NU_OVER_EV, 1. - alpha);
      Lconv = 1. / Lconv;
      Lconv *= pow(E0 * K_NU_OVER_EV, -alpha) * (1 - alpha);
    }
    Lconv *= (K_SEC_PER_YEAR) / (K_PLANCK);
    c->const_zp_prefactor = (p->lx_gal * Lconv) / (E0 * K_NU_OVER_EV) * K_C * pow(1 + zp, alpha + 3);

    /* per-cell evolution, ComputeTs.c:743-900: cells in parallel, the
     * volume averages summed afterwards in the reference's cell order */
    double* contrib = (double*)ctx_buf((void**)&c->contrib, sizeof(double) * 4 * (size_t)D * D * D);
    /* timing sample: the first D / sample_cell_div x planes only; the x and
     * y loops are shared out together, so that a sample of fewer x planes
     * than threads still keeps every thread busy */
    const int nx_cells = c->sample_cell_div > 1 ? D / c->sample_cell_div : D;
#pragma omp parallel
    {
    double* SFR = (double*)malloc(sizeof(double) * (size_t)S);
    double* fh = (double*)malloc(sizeof(double) * (size_t)S);
    double* fi = (double*)malloc(sizeof(double) * (size_t)S);
    double* fl = (double*)malloc(sizeof(double) * (size_t)S);
#pragma omp for collapse(2) schedule(static)
    for (int ix = 0; ix < nx_cells; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ir = real_idx(D, ix, iy, iz);
          const size_t i_padded = pad_idx(D, ix, iy, iz);
          float curr_xalpha;
          double ans[2], dansdz[5];
          ans[0] = g->x_e_box_prev[i_padded];
          ans[1] = g->Tk_box[ir];
          for (int R_ct = 0; R_ct < S; R_ct++) {
            SFR[R_ct] = smoothed[(size_t)R_ct + (size_t)S * ir];
            double xHII_call = g->x_e_box_prev[i_padded];
            if (xHII_call > c->x_xhii[K_NXHII - 1] * 0.999)
              xHII_call = c->x_xhii[K_NXHII - 1] * 0.999;
            else if (xHII_call < c->x_xhii[0])
              xHII_call = 1.001 * c->x_xhii[0];
            const int lo = c_loc_xhii(c, (float)xHII_call), hi = lo + 1;
            const double* T3[3] = { tH, tI, tL };
            double* O3[3] = { fh, fi, fl };
            for (int t = 0; t < 3; t++) {
              double v = (T3[t][(size_t)hi * S + R_ct] - T3[t][(size_t)lo * S + R_ct]) / (c->x_xhii[hi] - c->x_xhii[lo]);
              v *= (xHII_call - c->x_xhii[lo]);
              v += T3[t][(size_t)lo * S + R_ct];
              O3[t][R_ct] = v;
            }
          }
          c_evolve(c, (float)zp, g->deltax[i_padded], SFR, fh, fi, fl, NO_LIGHT, ans, dansdz);
          g->x_e_box_prev[i_padded] += dansdz[0] * dzp;
          if (g->x_e_box_prev[i_padded] > 1)
            g->x_e_box_prev[i_padded] = (float)(1 - K_FRACT_FLOAT_ERR);
          else if (g->x_e_box_prev[i_padded] < 0)
            g->x_e_box_prev[i_padded] = 0;
          if (g->Tk_box[ir] < K_MAX_TK)
            g->Tk_box[ir] += dansdz[1] * dzp;
          if (g->Tk_box[ir] < 0)
            g->Tk_box[ir] = (float)(K_TCMB * (1 + zp));
          g->TS_box[ir] = c_get_Ts(c, (float)zp, g->deltax[i_padded], g->Tk_box[ir], g->x_e_box_prev[i_padded],
                                   (float)dansdz[2], &curr_xalpha);
          contrib[4 * ir + 0] = dansdz[2];
          contrib[4 * ir + 1] = curr_xalpha;
          contrib[4 * ir + 2] = dansdz[3];
          contrib[4 * ir + 3] = dansdz[4];
        }
    free(SFR);
    free(fh);
    free(fi);
    free(fl);
    }
    c->phase[MXO_PH_EVOLVE] = omp_get_wtime() - tp;
    c->phase[MXO_PH_EVOLVE_FRAC] = (double)nx_cells / (double)D;
    for (size_t ir = 0; ir < (size_t)D * D * D; ir++) {
      J_alpha_ave += contrib[4 * ir + 0];
      xalpha_ave += contrib[4 * ir + 1];
      Xheat_ave += contrib[4 * ir + 2];
      Xion_ave += contrib[4 * ir + 3];
    }

    i_padded = pad_idx(D, D - 1, D - 1, D - 1); /* last cell visited */
    free(R_values);
    free(scb);

    J_alpha_ave /= total_n_cells;
    xalpha_ave /= total_n_cells;
    Xheat_ave /= total_n_cells;
    Xion_ave /= total_n_cells;
  }

  /* ComputeTs.c:940-974 */
  const double tpost = omp_get_wtime();
  memcpy(g->x_e_box, g->x_e_box_prev, sizeof(float) * 2 * nc);
  double Ave_Ts = 0.0, Ave_x_e = 0.0, Ave_Tk = 0.0;
  for (int ix = 0; ix < D; ix++)
    for (int iy = 0; iy < D; iy++)
      for (int iz = 0; iz < D; iz++) {
        const size_t ir = real_idx(D, ix, iy, iz);
        Ave_Ts += (double)g->TS_box[ir];
        Ave_Tk += (double)g->Tk_box[ir];
        Ave_x_e += (double)g->x_e_box_prev[i_padded]; /* stale index, ComputeTs.c:957 */
      }
  Ave_Ts /= total_n_cells;
  Ave_Tk /= total_n_cells;
  Ave_x_e /= total_n_cells;
  c->phase[MXO_PH_TS_POST] = omp_get_wtime() - tpost;
  if (out) {
    if ((zp - p->max_heating_redshift) < -0.0001) {
      out->volume_ave_J_alpha = J_alpha_ave;
      out->volume_ave_xalpha = xalpha_ave;
      out->volume_ave_Xheat = Xheat_ave;
      out->volume_ave_Xion = Xion_ave;
    }
    out->volume_ave_TS = Ave_Ts;
    out->volume_ave_TK = Ave_Tk;
    out->volume_ave_xe = Ave_x_e;
    out->x_e_ave = c->x_e_ave;
    out->collapse_fraction = collapse_fraction;
  }
  return 0;
}

/* ==================================================== brightness temperature */

/* ComputeBrightnessTemperatureBox, BrightnessTemperature.c:24-124, 512-548
 * (peculiar-velocity modes are not restated here) */
#define MXO_N_RSD_STEPS 50
#define MXO_MAX_DVDR 0.2f
#define MXO_FRACT_FLOAT_ERR 1e-7
#define MXO_MPC 3.086e24

/* One z column of the line-of-sight remap (BrightnessTemperature.c:325-499):
 * the sub-cells of every cell are displaced by the interpolated velocity and
 * deposited, with the reference's float / double mix, into los[0..D). */
void mxo_rsd_column(int D, double BoxSize, double subcell_width, double x_val1, double x_val2, const float* x_pos,
                    const float* x_pos_offset, float H_z, const float* vel, const float* delta_T, const float* xH,
                    float* los)
{
  const int N = MXO_N_RSD_STEPS;
  for (int kk = 0; kk < D; kk++)
    los[kk] = 0.0;
  for (int kk = 0; kk < D; kk++) {
    if (!((fabs(delta_T[kk]) >= MXO_FRACT_FLOAT_ERR) && (xH[kk] >= MXO_FRACT_FLOAT_ERR)))
      continue;
    double d1_low, d2_low, d1_high, d2_high;
    if (kk == 0) {
      d1_low = vel[D - 1] / H_z;
      d2_low = vel[kk] / H_z;
    } else {
      d1_low = vel[kk - 1] / H_z;
      d2_low = vel[kk] / H_z;
    }
    if (kk == (D - 1)) {
      d1_high = vel[kk] / H_z;
      d2_high = vel[0] / H_z;
    } else {
      d1_high = vel[kk] / H_z;
      d2_high = vel[kk + 1] / H_z;
    }
    const float dT = delta_T[kk];
    for (int iii = 0; iii < N; iii++) {
      double subcell_displacement;
      if (x_pos[iii] <= 0.5)
        subcell_displacement = d1_low + ((x_pos[iii] + 0.5) - x_val1) * (d2_low - d1_low) / (x_val2 - x_val1);
      else
        subcell_displacement = d1_high + ((x_pos[iii] - 0.5) - x_val1) * (d2_high - d1_high) / (x_val2 - x_val1);
      const double RSD_pos_new = (x_pos_offset[iii] + subcell_displacement) / (BoxSize / (float)D);
      const double lo = RSD_pos_new - (subcell_width / 2.) / (BoxSize / (float)D);
      const double hi = RSD_pos_new + (subcell_width / 2.) / (BoxSize / (float)D);
      if (lo >= 0.0 && hi < 1.0) {
        los[kk] += dT / (float)N;
      } else if (lo < 0.0 && hi < 0.0) {
        const double cell_distance = ceil(fabs(lo)) - 1.;
        const int cd = (int)cell_distance;
        if (fabs(hi) > cell_distance) {
          if (kk < (cd + 1))
            los[kk - (cd + 1) + D] += dT / (float)N;
          else
            los[kk - (cd + 1)] += dT / (float)N;
        } else {
          const double fraction_outside = (fabs(lo) - cell_distance) / (subcell_width / (BoxSize / (float)D));
          const double fraction_within = 1. - fraction_outside;
          if (kk < cd)
            los[kk - cd + D] += fraction_within * dT / (float)N;
          else
            los[kk - cd] += fraction_within * dT / (float)N;
          if (kk < (cd + 1))
            los[kk - (cd + 1) + D] += fraction_outside * dT / (float)N;
          else
            los[kk - (cd + 1)] += fraction_outside * dT / (float)N;
        }
      } else if (lo < 0.0 && (hi > 0.0 && hi < 1.0)) {
        const double fraction_within = hi / (subcell_width / (BoxSize / (float)D));
        const double fraction_outside = 1. - fraction_within;
        if (kk == 0) {
          los[D - 1] += fraction_outside * dT / (float)N;
          los[kk] += fraction_within * dT / (float)N;
        } else {
          los[kk - 1] += fraction_outside * dT / (float)N;
          los[kk] += fraction_within * dT / (float)N;
        }
      } else if ((lo >= 0.0 && lo < 1.0) && (hi >= 1.0)) {
        const double fraction_outside = (hi - 1.) / (subcell_width / (BoxSize / (float)D));
        const double fraction_within = 1. - fraction_outside;
        if (kk == (D - 1)) {
          los[kk] += fraction_within * dT / (float)N;
          los[0] += fraction_outside * dT / (float)N;
        } else {
          los[kk] += fraction_within * dT / (float)N;
          los[kk + 1] += fraction_outside * dT / (float)N;
        }
      } else {
        const double cell_distance = floor(fabs(hi));
        const int cd = (int)cell_distance;
        if (lo >= cell_distance) {
          if (kk > (D - 1 - cd))
            los[kk + cd - D] += dT / (float)N;
          else
            los[kk + cd] += dT / (float)N;
        } else {
          const double fraction_outside = (hi - cell_distance) / (subcell_width / (BoxSize / (float)D));
          const double fraction_within = 1. - fraction_outside;
          if (kk > (D - 1 - (cd - 1)))
            los[kk + cd - 1 - D] += fraction_within * dT / (float)N;
          else
            los[kk + cd - 1] += fraction_within * dT / (float)N;
          if (kk > (D - 1 - cd))
            los[kk + cd - D] += fraction_outside * dT / (float)N;
          else
            los[kk + cd] += fraction_outside * dT / (float)N;
        }
      }
    }
  }
}

/* Peculiar-velocity corrections of the brightness temperature,
 * BrightnessTemperature.c:158-509 (spin temperature on,
 * Flag_IncludePecVelsFor21cm 1-3); vel is converted in place like the
 * reference does. */
static void pecvel_correction(mxo_ctx* c, const mx_grids* g, float redshift, double T_rad)
{
  const mx_params* p = &c->p;
  const int D = p->grid_dim, H = D / 2 + 1;
  const double total_n_cells = pow((double)D, 3);
  const double BoxSize = p->box_size / p->hubble_h;
  const float H_z = (float)(float)c_hubble(c, redshift);
  float* vel = g->vel;
  float* delta_T = g->delta_T;
  /* :180-209 velocity units */
  for (int ii = 0; ii < D; ii++)
    for (int jj = 0; jj < D; jj++)
      for (int kk = 0; kk < D; kk++) {
        const size_t ip = pad_idx(D, ii, jj, kk);
        switch (p->trees_id) {
          case 1: /* GBPTREES_TREES */
            vel[ip] = (float)(sqrt(1. / (1. + redshift)) * vel[ip] / 1000.);
            break;
          case 0: /* VELOCIRAPTOR_TREES */
          case 2: /* VELOCIRAPTOR_TREES_AUG */
            vel[ip] = (float)((1. + redshift) * vel[ip]);
            break;
        }
        vel[ip] *= 1000. * 100. / MXO_MPC;
        vel[ip] = (float)(vel[ip] / (1. / (1. + redshift)));
      }
  /* :212-228 gradient along z in k-space */
  const size_t nc = (size_t)D * D * H;
  float* spec = (float*)malloc(sizeof(float) * 2 * nc);
  float* grad = (float*)malloc(sizeof(float) * 2 * nc);
  mxo_r2c_3d(D, vel, 1, spec);
  for (size_t i = 0; i < nc; i++) {
    float complex v = spec[2 * i] + I * spec[2 * i + 1];
    v /= total_n_cells;
    v *= p->hubble_h;
    spec[2 * i] = crealf(v);
    spec[2 * i + 1] = cimagf(v);
  }
  {
    /* velocity_gradient, reionization.c:2172-2187 (k from BoxSize in Mpc/h) */
    const float box_size = (float)p->box_size;
    const float delta_k = (float)(2.0 * M_PI / box_size);
    for (int n_x = 0; n_x < D; n_x++)
      for (int n_y = 0; n_y < D; n_y++)
        for (int n_z = 0; n_z <= D / 2; n_z++) {
          const float k_z = n_z * delta_k;
          const size_t ih = ((size_t)n_x * D + n_y) * H + n_z;
          float complex v = spec[2 * ih] + I * spec[2 * ih + 1];
          v *= (float complex)(k_z * I);
          spec[2 * ih] = crealf(v);
          spec[2 * ih + 1] = cimagf(v);
        }
  }
  mxo_c2r_3d(D, spec, grad); /* padded real */
  free(spec);
  free(c->last_vel_grad);
  c->last_vel_grad = grad;
  const double max_v_deriv = fabs(MXO_MAX_DVDR * H_z);
  if (p->flag_pecvel == 1) {
    /* :232-257 */
    for (int ii = 0; ii < D; ii++)
      for (int jj = 0; jj < D; jj++)
        for (int kk = 0; kk < D; kk++) {
          const size_t ir = real_idx(D, ii, jj, kk), ip = pad_idx(D, ii, jj, kk);
          double dvdx = (double)grad[ip];
          if (fabs(dvdx) > max_v_deriv)
            dvdx = dvdx < 0 ? -max_v_deriv : max_v_deriv;
          delta_T[ir] /= (dvdx / H_z + 1.0);
        }
  }
  if (p->flag_pecvel > 1) {
    /* :261-315 (spin temperature on) */
    for (int ii = 0; ii < D; ii++)
      for (int jj = 0; jj < D; jj++)
        for (int kk = 0; kk < D; kk++) {
          const size_t ir = real_idx(D, ii, jj, kk), ip = pad_idx(D, ii, jj, kk);
          const double gradient_component = fabs((double)grad[ip] / H_z + 1.0);
          if (gradient_component < MXO_FRACT_FLOAT_ERR)
            delta_T[ir] = (float)(1000. * (g->TS_box[ir] - T_rad) / (1. + redshift));
          else
            delta_T[ir] = (float)((1. - exp(-delta_T[ir] / gradient_component)) * 1000. * (g->TS_box[ir] - T_rad) /
                                  (1. + redshift));
        }
  }
  if (p->flag_pecvel == 3) {
    /* :317-505 line-of-sight redshift-space distortions along z */
    const double subcell_width = (BoxSize / ((double)D)) / (double)MXO_N_RSD_STEPS;
    float x_pos[MXO_N_RSD_STEPS], x_pos_offset[MXO_N_RSD_STEPS];
    for (int iii = 0; iii < MXO_N_RSD_STEPS; iii++) {
      x_pos_offset[iii] = (float)(subcell_width * (float)iii + subcell_width / 2.);
      x_pos[iii] = (float)(x_pos_offset[iii] / (BoxSize / (float)D));
    }
    float* los = (float*)malloc(sizeof(float) * (size_t)D);
    for (int ii = 0; ii < D; ii++)
      for (int jj = 0; jj < D; jj++) {
        mxo_rsd_column(D, BoxSize, subcell_width, 0., 1., x_pos, x_pos_offset, H_z, vel + pad_idx(D, ii, jj, 0),
                       delta_T + real_idx(D, ii, jj, 0), g->xH + real_idx(D, ii, jj, 0), los);
        for (int kk = 0; kk < D; kk++)
          delta_T[real_idx(D, ii, jj, kk)] = los[kk];
      }
    free(los);
  }
}

int mxo_delta_T(mxo_ctx* c, int snapshot, const mx_grids* g, mx_globals* out)
{
  const mx_params* p = &c->p;
  const int D = p->grid_dim;
  if (snapshot < 0 || snapshot >= c->n_snaps)
    return MX_ESTATE;
  if (p->flag_pecvel < 0 || p->flag_pecvel > 3)
    return MX_EINVAL;
  if (p->flag_pecvel != 0 && p->flag_spin_temp && (!g->vel || !g->TS_box))
    return MX_EINVAL;
  const double total_n_cells = pow((double)D, 3);
  const float redshift = (float)(float)c->zz[snapshot];
  const float Hubble_h = (float)(float)p->hubble_h;
  const float OmegaM = (float)(float)p->omega_m;
  const float OmegaB = (float)(OmegaM * p->baryon_frac);
  const float const_factor =
    (float)(27.0 * (OmegaB * Hubble_h * Hubble_h / 0.023) * sqrt((0.15 / OmegaM / Hubble_h / Hubble_h) * (1.0 + redshift) / 10.0));
  const double T_rad = K_TCMB * (1. + redshift);
  for (int ii = 0; ii < D; ii++)
    for (int jj = 0; jj < D; jj++)
      for (int kk = 0; kk < D; kk++) {
        const size_t ir = real_idx(D, ii, jj, kk);
        const size_t ip = pad_idx(D, ii, jj, kk);
        const double pixel_deltax = g->deltax[ip];
        const double pixel_x_HI = g->xH[ir];
        g->delta_T[ir] = (float)(const_factor * pixel_x_HI * (1.0 + pixel_deltax));
        if (p->flag_spin_temp) {
          if (p->flag_pecvel > 1)
            g->delta_T[ir] *= (1. + redshift) / (1000. * g->TS_box[ir]);
          else {
            const double pixel_Ts_factor = (1 - T_rad / g->TS_box[ir]);
            g->delta_T[ir] *= pixel_Ts_factor;
          }
        }
      }
  if (p->flag_spin_temp && p->flag_pecvel > 0)
    pecvel_correction(c, g, redshift, T_rad);
  double Ave_Tb = 0.0;
  for (size_t i = 0; i < (size_t)D * D * D; i++)
    Ave_Tb += (double)g->delta_T[i];
  Ave_Tb /= total_n_cells;
  if (out)
    out->volume_ave_Tb = Ave_Tb;
  return 0;
}

/* ------------------------------------------------------------------------
 * 21 cm power spectrum: Initialise_PowerSpectrum (ComputePowerSpectrum.c:18-42)
 * and Compute_PS (:44-255), single rank, without the Pop III field.
 * ---------------------------------------------------------------------- */
int mxo_ps_length(int D, double box_size_mpc_h, double hubble_h)
{
  const double box_size = box_size_mpc_h / hubble_h; /* Mpc */
  const float k_factor = 1.35f;
  const float delta_k = (float)(2. * M_PI / box_size);
  const float k_max = delta_k * D;
  float k_ceil = delta_k;
  int n = 0;
  while (k_ceil < k_max) {
    n++;
    k_ceil *= k_factor;
  }
  return n;
}

int mxo_power_spectrum(int D, double box_size_mpc_h, double hubble_h, const float* delta_T, float* ps_k, float* ps_data,
                       float* ps_error, int cap)
{
  const int nb = mxo_ps_length(D, box_size_mpc_h, hubble_h);
  if (nb > cap)
    return -1;
  const double box_size = box_size_mpc_h / hubble_h;
  const float volume = powf((float)box_size, 3);
  const double total_n_cells = pow((double)D, 3);
  const int H = D / 2 + 1;
  /* :74-83 mean of delta_T */
  double ave = 0.0;
  for (size_t i = 0; i < (size_t)D * D * D; i++)
    ave += delta_T[i];
  ave /= total_n_cells;
  /* :94-110 the field (delta_T / ave - 1) * V / N * ave in the padded layout */
  float* deldel = (float*)calloc((size_t)D * D * 2 * H, sizeof(float));
  float* spec = (float*)malloc(sizeof(float) * 2 * (size_t)D * D * H);
  for (int ii = 0; ii < D; ii++)
    for (int jj = 0; jj < D; jj++)
      for (int kk = 0; kk < D; kk++) {
        const size_t ip = pad_idx(D, ii, jj, kk);
        deldel[ip] = (float)((delta_T[real_idx(D, ii, jj, kk)] / ave - 1) * volume / (float)total_n_cells);
        deldel[ip] *= ave;
      }
  mxo_r2c_3d(D, deldel, 1, spec);
  free(deldel);
  /* :130-215 binning */
  const float k_factor = 1.35f;
  const float delta_k = (float)(2. * M_PI / box_size);
  const float k_first_bin_ceil = delta_k;
  const float k_max = delta_k * D;
  double* p_box = (double*)calloc((size_t)nb, sizeof(double));
  double* k_ave = (double*)calloc((size_t)nb, sizeof(double));
  unsigned long long* in_bin_ct = (unsigned long long*)calloc((size_t)nb, sizeof(unsigned long long));
  const int middle = D / 2;
  for (int n_x = 0; n_x < D; n_x++) {
    float k_x = n_x * delta_k;
    if (n_x > middle)
      k_x = (n_x - D) * delta_k;
    for (int n_y = 0; n_y < D; n_y++) {
      float k_y = n_y * delta_k;
      if (n_y > middle)
        k_y = (n_y - D) * delta_k;
      for (int n_z = 0; n_z <= middle; n_z++) {
        const float k_z = n_z * delta_k;
        const float k_mag = (float)sqrt(k_x * k_x + k_y * k_y + k_z * k_z);
        int ct = 0;
        float k_floor = 0;
        float k_ceil = k_first_bin_ceil;
        while (k_ceil < k_max) {
          if ((k_mag >= k_floor) && (k_mag < k_ceil)) {
            const size_t ih = ((size_t)n_x * D + n_y) * H + n_z;
            const float complex X = spec[2 * ih] + I * spec[2 * ih + 1];
            in_bin_ct[ct]++;
            p_box[ct] += pow(k_mag, 3) * pow(cabs(X), 2.) / (2.0 * M_PI * M_PI * volume);
            k_ave[ct] += k_mag;
            break;
          }
          ct++;
          k_floor = k_ceil;
          k_ceil *= k_factor;
        }
      }
    }
  }
  /* :228-240 */
  for (int i = 0; i < nb; i++) {
    ps_k[i] = (float)(k_ave[i] / (double)in_bin_ct[i]);
    ps_data[i] = (float)(p_box[i] / (double)in_bin_ct[i]);
    ps_error[i] = (float)((p_box[i] / (double)in_bin_ct[i]) / sqrt((double)in_bin_ct[i]));
  }
  free(spec);
  free(p_box);
  free(k_ave);
  free(in_bin_ct);
  return nb;
}

const float* mxo_last_velocity_gradient(const mxo_ctx* c) { return c->last_vel_grad; }

/* ------------------------------------------------------------------------
 * Light cone: Initialise_ConstructLightcone (ConstructLightcone.c:12-67) and
 * ConstructLightcone (:69-166), single rank.
 * ---------------------------------------------------------------------- */
/* gettime, XRayHeatingFunctions.c:483-494 (zero curvature, Weinberg 1989) */
static double c_gettime(const mxo_ctx* c, double z)
{
  const double OMl = c->p.omega_lambda, OMm = c->p.omega_m;
  const double x = sqrt(OMl / OMm) * pow(1 + z, -3.0 / 2.0);
  const double term1 = log(x + sqrt(pow(x, 2) + 1));
  const double const1 = 2 * sqrt(1 + OMm / OMl) / (3 * K_HUBBLE * c->p.hubble_h);
  return term1 * const1;
}

long long mxo_lightcone_init(mxo_ctx* c, double end_redshift, int last_output_snap, int* end_snapshot)
{
  const double box_size = c->p.box_size / c->p.hubble_h;
  const double dR = (box_size / (double)c->p.grid_dim) * MXO_MPC;
  const double start_redshift = c->zz[0];
  int i = 0;
  while (c->zz[i] > end_redshift)
    i++;
  int closest = i;
  if (closest > last_output_snap)
    closest = last_output_snap;
  double z1 = c->zz[closest], z_LC = z1;
  long long total = 0;
  i = 0;
  while (z1 < start_redshift) {
    const double z2 = c->zz[closest - 1 - i];
    while (z_LC < z2) {
      total++;
      z_LC -= dR / c_drdz(c, (float)z_LC);
    }
    z1 = z2;
    i += 1;
  }
  c->lc_length = total;
  c->lc_end_snapshot = closest;
  if (end_snapshot)
    *end_snapshot = closest;
  return total;
}

int mxo_construct_lightcone(mxo_ctx* c, int snapshot, const float* delta_T, float* delta_T_prev, float* lightcone,
                            float* lightcone_redshifts)
{
  const int D = c->p.grid_dim;
  const double box_size = c->p.box_size / c->p.hubble_h;
  const double dR = (box_size / (double)D) * MXO_MPC;
  if (snapshot > 0) {
    const double z2_LC = c->zz[snapshot - 1], t_z2 = c_gettime(c, z2_LC);
    const double z1_LC = c->zz[snapshot], t_z1 = c_gettime(c, z1_LC);
    double z_LC = c->zz[c->lc_end_snapshot];
    long long n_snap = 0;
    while (z_LC < z2_LC) {
      if (z_LC >= c->zz[snapshot] && z_LC < c->zz[snapshot - 1])
        n_snap++;
      z_LC -= dR / c_drdz(c, (float)z_LC);
    }
    z_LC = c->zz[c->lc_end_snapshot];
    c->lc_pos -= n_snap;
    long long slice_ct = c->lc_pos;
    int iz = (int)(slice_ct % D);
    while (z_LC < z2_LC) {
      if (z_LC >= c->zz[snapshot] && z_LC < c->zz[snapshot - 1]) {
        const double t_slice = c_gettime(c, z_LC);
        lightcone_redshifts[slice_ct] = (float)z_LC;
        if (iz >= D)
          iz = 0;
        for (int ii = 0; ii < D; ii++)
          for (int jj = 0; jj < D; jj++) {
            const size_t i_lc = (size_t)slice_ct + (size_t)c->lc_length * ((size_t)jj + (size_t)D * ii);
            const size_t ir = real_idx(D, ii, jj, iz);
            const double fz1 = delta_T[ir], fz2 = delta_T_prev[ir];
            lightcone[i_lc] = (float)((fz2 - fz1) / (t_z2 - t_z1) * (t_slice - t_z1) + fz1);
          }
        iz++;
        slice_ct++;
      }
      z_LC -= dR / c_drdz(c, (float)z_LC);
    }
  } else {
    c->lc_pos = c->lc_length;
  }
  memcpy(delta_T_prev, delta_T, sizeof(float) * (size_t)D * D * D);
  return 0;
}

/* ------------------------------------------------------------------------
 * Galaxy -> grid deposit: construct_baryon_grids (reionization.c:1353-1615),
 * single rank, no mini-haloes; and the grid -> galaxy feedback mass
 * calculate_Mvir_crit (physics/reionization.c:10-59).
 * ---------------------------------------------------------------------- */
/* pos_to_ngp, misc_tools.c:163-173; -1 for a negative index */
static int ngp(double x, double side, int nx)
{
  int ind = (int)nearbyint(x / side * (double)nx);
  if (ind > nx - 1)
    ind = 0;
  return ind > -1 ? ind : -1;
}

/* hubble_time, virial_properties.c:79-93 (internal time units) */
static double c_hubble_time(const mxo_ctx* c, int snapshot)
{
  const double zplus1 = c->zz[snapshot] + 1;
  return 1.0 / (c->hubble_int * sqrt(c->p.omega_m * zplus1 * zplus1 * zplus1 + c->p.omega_k * zplus1 * zplus1 +
                                     c->p.omega_lambda));
}

int mxo_construct_baryon_grids(mxo_ctx* c, int snapshot, int n, const float* pos, const int* type, const double* fesc_gsm,
                               const double* gross_sm, const double* bhm, const double* ebhm, int flag_bh,
                               double bh_limit, double alpha_uv_bh, const mx_grids* g)
{
  const mx_params* p = &c->p;
  const int D = p->grid_dim, H = D / 2 + 1;
  const size_t np = (size_t)D * D * 2 * H, nr = (size_t)D * D * D;
  const double box_size = p->box_size;
  const double sfr_timescale = p->reion_sfr_timescale * c_hubble_time(c, snapshot);
  /* :1375-1397 */
  memset(g->stars, 0, sizeof(float) * np);
  memset(g->weighted_sfr, 0, sizeof(float) * np);
  if (p->flag_spin_temp) {
    memset(g->sfr, 0, sizeof(float) * np);
    for (int snap = c->n_hist - 2; snap >= 0; snap--)
      memcpy(g->sfr_histories + (size_t)(snap + 1) * np, g->sfr_histories + (size_t)snap * np, sizeof(float) * np);
  }
  float* buffer = (float*)malloc(sizeof(float) * nr);
  int rc = 0;
  for (int prop = 0; prop < 3; prop++) { /* stellar, weighted_sfr, sfr */
    if (!p->flag_spin_temp && prop == 2)
      continue;
    memset(buffer, 0, sizeof(float) * nr);
    for (int i = 0; i < n; i++) {
      if (type[i] > 2)
        continue;
      const int ix = ngp(pos[3 * i], box_size, D), iy = ngp(pos[3 * i + 1], box_size, D),
                iz = ngp(pos[3 * i + 2], box_size, D);
      if (ix < 0 || iy < 0 || iz < 0) {
        rc = MX_EINVAL;
        continue;
      }
      const size_t ind = real_idx(D, ix, iy, iz);
      if (prop == 0) {
        buffer[ind] += fesc_gsm[i];
        if (flag_bh && bhm[i] >= bh_limit)
          buffer[ind] += ebhm[i];
      } else if (prop == 1) {
        buffer[ind] += (fesc_gsm[i]);
        if (flag_bh && bhm[i] >= bh_limit)
          buffer[ind] += ebhm[i] * alpha_uv_bh / p->alpha_uv;
      } else {
        buffer[ind] += gross_sm[i];
      }
    }
    for (int ix = 0; ix < D; ix++)
      for (int iy = 0; iy < D; iy++)
        for (int iz = 0; iz < D; iz++) {
          const size_t ir = real_idx(D, ix, iy, iz), ip = pad_idx(D, ix, iy, iz);
          if (prop == 0) {
            float val = buffer[ir];
            if (val < 0)
              val = 0;
            g->stars[ip] = val;
          } else {
            double val = (double)buffer[ir];
            val = (val > 0) ? val / sfr_timescale : 0;
            if (prop == 1) {
              g->weighted_sfr[ip] = (float)val;
            } else {
              g->sfr[ip] = (float)val;
              g->sfr_histories[ip] = (float)val;
            }
          }
        }
  }
  free(buffer);
  return rc;
}

int mxo_calculate_Mvir_crit(mxo_ctx* c, double redshift, double m0, double a, double b, double cc, double d,
                            const float* J_21_at_ion, const float* z_at_ion, float* Mvir_crit)
{
  const int D = c->p.grid_dim;
  const double Hubble_h = c->p.hubble_h;
  for (size_t i = 0; i < (size_t)D * D * D; i++) {
    double cell = 0.0;
    if (z_at_ion[i] > redshift)
      cell = m0 * pow((double)(J_21_at_ion[i]) * Hubble_h * Hubble_h, a) * pow((1.0 + redshift) / 10.0, b) *
             pow((1.0 - pow((1.0 + redshift) / (1.0 + (double)(z_at_ion[i])), cc)), d);
    Mvir_crit[i] = (float)cell;
  }
  return 0;
}
