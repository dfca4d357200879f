// Host-side FP64 physics tables of the reionization step.
//
// These are the small, grid-independent pieces of the step that the
// reference evaluates on the host: the recombination-rate table
// (src/core/recombinations.c), the RECFAST / collisional-coupling / stellar
// spectrum tables and the X-ray frequency integrals
// (src/core/XRayHeatingFunctions.c), the filter-radius schedule
// (src/core/find_HII_bubbles.c:184-207) and the spin-temperature shell
// schedule with its SFR-history weights (src/core/ComputeTs.c:32-76, 270-377).
// The third-party numerics they rely on (GSL natural cubic spline, QUADPACK
// QAG with the 61-point Gauss-Kronrod rule, Brent's root bracketing) are
// implemented here from the published algorithms.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "mx_reion.h"

namespace mx {

// ---------------------------------------------------------------- constants
// src/meraxes.h:21-44, src/core/reionization.h:8-46,
// src/core/XRayHeatingFunctions.h:15-40, src/core/recombinations.h:17-33
namespace k {
constexpr double GRAVITY = 6.672e-8;
constexpr double SOLAR_MASS = 1.989e33;
constexpr double BOLTZMANN = 1.3806e-16;
constexpr double C = 2.9979e10;
constexpr double PLANCK = 6.6262e-27;
constexpr double PROTONMASS = 1.6726e-24;
constexpr double HUBBLE = 3.2407789e-18;
constexpr double SEC_PER_YEAR = 3.155e7;
constexpr double MPC = 3.086e24;
constexpr double TCMB = 2.728;
constexpr float REL_TOL = 1e-5f;
constexpr float ABS_TOL = 1e-8f;
constexpr double SIGMA_HI = 6.3e-18;
constexpr double TINY = 1e-30;
constexpr double FRACT_FLOAT_ERR = 1e-7;
constexpr float MAX_TK = 5e4f;
constexpr double L_FACTOR = 0.620350491;
constexpr double ALPHAB_10K = 2.59e-13;
constexpr double T21 = 0.0628;
constexpr double A10 = 2.85e-15;
constexpr double LYA_HZ = 2.46606727e15;
constexpr double NU_OVER_EV = 1.60217646e-12 / PLANCK;
constexpr double NU_HI = 13.60 * NU_OVER_EV;
constexpr double NU_HEI = 24.59 * NU_OVER_EV;
constexpr double NU_HEII = NU_HI * 4;
constexpr int NSPEC_MAX = 23;
constexpr int RECFAST_NPTS = 501;
constexpr int KAPPA_10_NPTS = 27;
constexpr int KAPPA_E_NPTS = 20;
constexpr int KAPPA_P_NPTS = 17;
constexpr int NXHII = 14;
constexpr int NENERGY = 258;
constexpr float R_XLY_MAX = 500.0f;
constexpr int A_NPTS = 60;
constexpr int C_NPTS = 12;
constexpr int BETA_NPTS = 5;
constexpr int RR_Z_NPTS = 300;
constexpr float RR_DEL_Z = 0.2f;
constexpr int RR_LNG_NPTS = 150;
constexpr double RR_LNG_MIN = -10.0;
constexpr float RR_DEL_LNG = 0.1f;
constexpr double PI = 3.14159265358979323846;
}  // namespace k

// ------------------------------------------------------- numerics (GSL-like)
struct NaturalSpline
{
  std::vector<double> x, y, c;  // c = second derivative / 2
  void init(const double* xs, const double* ys, int n);
  double eval(double xv) const;  // NaN outside [x0, xn-1]
};

using Integrand = std::function<double(double)>;
// QUADPACK QAG with the 61-point Gauss-Kronrod rule (GSL semantics).
int qag61(const Integrand& f, double a, double b, double epsabs, double epsrel, size_t limit, double* result,
          double* abserr);
// Brent bracketing + interval test with relative tolerance `epsrel`, up to
// `max_iter` iterations (XRayHeatingFunctions.c:266-292 uses 0.02 / 100).
double brent_root(const std::function<double(double)>& f, double lo, double hi, double epsrel, int max_iter);

// ------------------------------------------------------------ derived units
struct Derived
{
  double unit_time_s, G, hubble_int, rho_crit;  // init.c:184-205
  double no, he_no, f_h, f_he, n_b0;            // reionization.h:16-44
  void init(const mx_params& p);
};

double dtdz(const mx_params& p, float z);
double hubble(const mx_params& p, float z);
double drdz(const mx_params& p, float z);
double gettime(const mx_params& p, double z);
double RtoM(const mx_params& p, const Derived& d, double R);
double dicke(const mx_params& p, double z);
double ddicke_dz(const mx_params& p, double z);

// Radius schedule of find_HII_bubbles (largest first; last entry is the
// unfiltered cell-scale step).
std::vector<double> filter_radii(const mx_params& p);

// ------------------------------------------------- recombination-rate table
struct RecombTable
{
  // RR(z_ct, lnGamma) natural splines, 300 rows x 150 points
  std::vector<double> lng;  // 150
  std::vector<double> y;    // 300*150
  std::vector<double> c;    // 300*150
  bool ready = false;
  void build(const mx_params& p, const Derived& d, int nthreads);
};

// ------------------------------------------------------ spin-temperature data
struct HeatTables
{
  NaturalSpline recfast_T, recfast_x;
  double recfast_zmax = 0;
  // collisional coupling splines in (ln T, ln kappa)
  NaturalSpline kap10, kap_e, kap_p;
  float spec_nu[k::NSPEC_MAX], spec_N0[k::NSPEC_MAX], spec_alpha[k::NSPEC_MAX];
  float xhii[k::NXHII];
  float energy[k::NENERGY];
  float fheat[k::NXHII][k::NENERGY], nlya[k::NXHII][k::NENERGY];
  float nion_hi[k::NXHII][k::NENERGY], nion_hei[k::NXHII][k::NENERGY], nion_heii[k::NXHII][k::NENERGY];
  bool ready = false;
  int load(const mx_params& p, const std::string& dir, std::string* err);
  double T_recfast(float z) const;
  double xion_recfast(float z) const;
};

// One SFR-grid operation of the shell loop (ComputeTs.c:288-377,
// reionization.c:1756-1784), applied to the PADDED sfr grid in order.
struct SfrOp
{
  enum Kind : int32_t { SCALE_HALF = 0, ZERO_HALF = 1, LOAD = 2, ADD = 3 } kind;
  int32_t slice;  // history slice for LOAD / ADD
  float weight;   // float, as load_reion_sfr_grids takes it
  double dweight; // SCALE_HALF multiplies by a double
};

struct ShellPlan
{
  int S = 0;
  bool homogeneous = false;
  std::vector<double> R;         // filter radius of each shell [Mpc]
  std::vector<double> zpp_edge;  // shell redshift edges
  std::vector<std::vector<SfrOp>> ops;  // ops before the R2C of each shell
  // per-shell factors of evolveInt (XRayHeatingFunctions.c:1289-1330)
  std::vector<double> a_dt_dz;   // dt_dzpp * dzpp
  std::vector<double> b_pow;     // pow(1 + zpp, -alpha)
  std::vector<double> zpp1;      // 1 + zpp
  std::vector<double> dt_dzpp;   // dt_dzpp
  std::vector<double> dzpp;      // dzpp
  double weight_after = 1.0;     // value of the shell-loop `weight` at the end
};

// Builds the shell schedule of _ComputeTs for `snapshot`.
ShellPlan plan_shells(const mx_params& p, const std::vector<double>& zz, int snapshot);
// set_sfr_history (ComputeTs.c:32-76)
int n_sfr_histories(const mx_params& p, const std::vector<double>& zz);

// Frequency-integral tables and Ly-n sums for one snapshot
// (ComputeTs.c:517-663).  tables[3][14][S] (heat, ion, lya), sum_lyn[S].
struct FreqTables
{
  std::vector<double> tab;  // 3*14*S
  std::vector<double> sum_lyn;
  double const_zp_prefactor = 0;
  double growth_zp = 0, dgrowth_dzp = 0, dt_dzp = 0;
};
void build_freq_tables(const mx_params& p,
                       const Derived& d,
                       const HeatTables& ht,
                       const std::vector<double>& zz,
                       const double* stored_fcoll,
                       int snapshot,
                       const ShellPlan& sp,
                       double x_e_ave,
                       double weight_in,
                       int nthreads,
                       FreqTables* out);

}  // namespace mx
