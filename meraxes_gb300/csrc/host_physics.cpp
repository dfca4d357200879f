// Host-side FP64 physics tables of the reionization step (see host_physics.h).
#include "host_physics.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>

namespace mx {

// ======================================================== natural spline
// gsl_interp_cspline semantics: second derivatives from the symmetric
// tridiagonal system with zero end curvature; evaluation by the cubic
// y_lo + dx (b + dx (c + dx d)) on the bracketing interval.
void NaturalSpline::init(const double* xs, const double* ys, int n)
{
  x.assign(xs, xs + n);
  y.assign(ys, ys + n);
  c.assign(n, 0.0);
  if (n < 3)
    return;
  const int m = n - 2;
  std::vector<double> diag(m), off(m), rhs(m);
  for (int i = 0; i < m; i++) {
    const double h0 = xs[i + 1] - xs[i], h1 = xs[i + 2] - xs[i + 1];
    const double g0 = h0 != 0.0 ? 1.0 / h0 : 0.0, g1 = h1 != 0.0 ? 1.0 / h1 : 0.0;
    off[i] = h1;
    diag[i] = 2.0 * (h1 + h0);
    rhs[i] = 3.0 * ((ys[i + 2] - ys[i + 1]) * g1 - (ys[i + 1] - ys[i]) * g0);
  }
  if (m == 1) {
    c[1] = rhs[0] / diag[0];
    return;
  }
  std::vector<double> cp(m), dp(m);
  cp[0] = off[0] / diag[0];
  dp[0] = rhs[0] / diag[0];
  for (int i = 1; i < m; i++) {
    const double den = diag[i] - off[i - 1] * cp[i - 1];
    cp[i] = (i < m - 1) ? off[i] / den : 0.0;
    dp[i] = (rhs[i] - off[i - 1] * dp[i - 1]) / den;
  }
  c[m] = dp[m - 1];
  for (int i = m - 2; i >= 0; i--)
    c[i + 1] = dp[i] - cp[i] * c[i + 2];
}

double NaturalSpline::eval(double xv) const
{
  const int n = (int)x.size();
  if (!(xv >= x[0] && xv <= x[n - 1]))
    return NAN;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) / 2;
    if (x[mid] > xv)
      hi = mid;
    else
      lo = mid;
  }
  const double h = x[lo + 1] - x[lo];
  if (h <= 0.0)
    return NAN;
  const double dx = xv - x[lo];
  const double b = (y[lo + 1] - y[lo]) / h - h * (c[lo + 1] + 2.0 * c[lo]) / 3.0;
  const double dd = (c[lo + 1] - c[lo]) / (3.0 * h);
  return y[lo] + dx * (b + dx * (c[lo] + dx * dd));
}

// ================================================================ QAG-GK61
namespace {
// Kronrod abscissae (xk), Kronrod weights (wk) and Gauss weights (wg) of the
// 61-point rule, QUADPACK (Piessens et al. 1983), qk61.
const double XK[31] = {
  0.999484410050490637571325895705811, 0.996893484074649540271630050918695, 0.991630996870404594858628366109486,
  0.983668123279747209970032581605663, 0.973116322501126268374693868423707, 0.960021864968307512216871025581798,
  0.944374444748559979415831324037439, 0.926200047429274325879324277080474, 0.905573307699907798546522558925958,
  0.882560535792052681543116462530226, 0.857205233546061098958658510658944, 0.829565762382768397442898119732502,
  0.799727835821839083013668942322683, 0.767777432104826194917977340974503, 0.733790062453226804726171131369528,
  0.697850494793315796932292388026640, 0.660061064126626961370053668149271, 0.620526182989242861140477556431189,
  0.579345235826361691756024932172540, 0.536624148142019899264169793311073, 0.492480467861778574993693061207709,
  0.447033769538089176780609900322854, 0.400401254830394392535476211542661, 0.352704725530878113471037207089374,
  0.304073202273625077372677107199257, 0.254636926167889846439805129817805, 0.204525116682309891438957671002025,
  0.153869913608583546963794672743256, 0.102806937966737030147096751318001, 0.051471842555317695833025213166723,
  0.000000000000000000000000000000000
};
const double WG[15] = {
  0.007968192496166605615465883474674, 0.018466468311090959142302131912047, 0.028784707883323369349719179611292,
  0.038799192569627049596801936446348, 0.048402672830594052902938140422808, 0.057493156217619066481721689402056,
  0.065974229882180495128128515115962, 0.073755974737705206268243850022191, 0.080755895229420215354694938460530,
  0.086899787201082979802387530715126, 0.092122522237786128717632707087619, 0.096368737174644259639468626351810,
  0.099593420586795267062780282103569, 0.101762389748405504596428952168554, 0.102852652893558840341285636705415
};
const double WK[31] = {
  0.001389013698677007624551591226760, 0.003890461127099884051267201844516, 0.006630703915931292173319826369750,
  0.009273279659517763428441146892024, 0.011823015253496341742232898853251, 0.014369729507045804812451432443580,
  0.016920889189053272627572289420322, 0.019414141193942381173408951050128, 0.021828035821609192297167485738339,
  0.024191162078080601365686370725232, 0.026509954882333101610601709335075, 0.028754048765041292843978785354334,
  0.030907257562387762472884252943092, 0.032981447057483726031814191016854, 0.034979338028060024137499670731468,
  0.036882364651821229223911065617136, 0.038678945624727592950348651532281, 0.040374538951535959111995279752468,
  0.041969810215164246147147541285970, 0.043452539701356069316831728117073, 0.044814800133162663192355551616723,
  0.046059238271006988116271735559374, 0.047185546569299153945261478181099, 0.048185861757087129140779492298305,
  0.049055434555029778887528165367238, 0.049795683427074206357811569379942, 0.050405921402782346840893085653585,
  0.050881795898749606492297473049805, 0.051221547849258772170656282604944, 0.051426128537459025933862879215781,
  0.051494729429451567558340433647099
};

double rescale_err(double err, double res_abs, double res_asc)
{
  err = std::fabs(err);
  if (res_asc != 0 && err != 0) {
    const double scale = std::pow(200 * err / res_asc, 1.5);
    err = scale < 1 ? res_asc * scale : res_asc;
  }
  if (res_abs > DBL_MIN / (50 * DBL_EPSILON)) {
    const double min_err = 50 * DBL_EPSILON * res_abs;
    if (min_err > err)
      err = min_err;
  }
  return err;
}

struct Panel
{
  double result, abserr, resabs, resasc;
};

Panel gk61(const Integrand& f, double a, double b)
{
  double fv1[31], fv2[31];
  const double center = 0.5 * (a + b), half = 0.5 * (b - a), ahalf = std::fabs(half);
  const double fc = f(center);
  double rg = 0, rk = fc * WK[30], rabs = std::fabs(rk);
  for (int j = 0; j < 15; j++) {
    const int jtw = 2 * j + 1;
    const double dx = half * XK[jtw];
    const double f1 = f(center - dx), f2 = f(center + dx);
    fv1[jtw] = f1;
    fv2[jtw] = f2;
    rg += WG[j] * (f1 + f2);
    rk += WK[jtw] * (f1 + f2);
    rabs += WK[jtw] * (std::fabs(f1) + std::fabs(f2));
  }
  for (int j = 0; j < 15; j++) {
    const int jtwm1 = 2 * j;
    const double dx = half * XK[jtwm1];
    const double f1 = f(center - dx), f2 = f(center + dx);
    fv1[jtwm1] = f1;
    fv2[jtwm1] = f2;
    rk += WK[jtwm1] * (f1 + f2);
    rabs += WK[jtwm1] * (std::fabs(f1) + std::fabs(f2));
  }
  const double mean = rk * 0.5;
  double rasc = WK[30] * std::fabs(fc - mean);
  for (int j = 0; j < 30; j++)
    rasc += WK[j] * (std::fabs(fv1[j] - mean) + std::fabs(fv2[j] - mean));
  Panel p;
  const double err = (rk - rg) * half;
  p.result = rk * half;
  p.resabs = rabs * ahalf;
  p.resasc = rasc * ahalf;
  p.abserr = rescale_err(err, p.resabs, p.resasc);
  return p;
}

// Interval list kept in QUADPACK's partially sorted order (qpsrt).
struct IntervalList
{
  size_t limit, size = 0, nrmax = 0, i = 0;
  std::vector<double> a, b, r, e;
  std::vector<size_t> order, level;
  explicit IntervalList(size_t lim) : limit(lim), a(lim), b(lim), r(lim), e(lim), order(lim), level(lim) {}

  void sort_errors()
  {
    const size_t last = size - 1;
    size_t i_nrmax = nrmax;
    size_t i_maxerr = order[i_nrmax];
    if (last < 2) {
      order[0] = 0;
      order[1] = 1;
      i = i_maxerr;
      return;
    }
    const double errmax = e[i_maxerr];
    while (i_nrmax > 0 && errmax > e[order[i_nrmax - 1]]) {
      order[i_nrmax] = order[i_nrmax - 1];
      i_nrmax--;
    }
    const long top = (last < (limit / 2 + 2)) ? (long)last : (long)(limit - last + 1);
    long ii = (long)i_nrmax + 1;
    while (ii < top && errmax < e[order[ii]]) {
      order[ii - 1] = order[ii];
      ii++;
    }
    order[ii - 1] = i_maxerr;
    const double errmin = e[last];
    long kk = top - 1;
    while (kk > ii - 2 && errmin >= e[order[kk]]) {
      order[kk + 1] = order[kk];
      kk--;
    }
    order[kk + 1] = last;
    i = order[i_nrmax];
    nrmax = i_nrmax;
  }

  void split(double a1, double b1, double r1, double e1, double a2, double b2, double r2, double e2)
  {
    const size_t imax = i, inew = size, lev = level[imax] + 1;
    if (e2 > e1) {
      a[imax] = a2;
      r[imax] = r2;
      e[imax] = e2;
      level[imax] = lev;
      a[inew] = a1;
      b[inew] = b1;
      r[inew] = r1;
      e[inew] = e1;
      level[inew] = lev;
    } else {
      b[imax] = b1;
      r[imax] = r1;
      e[imax] = e1;
      level[imax] = lev;
      a[inew] = a2;
      b[inew] = b2;
      r[inew] = r2;
      e[inew] = e2;
      level[inew] = lev;
    }
    size++;
    sort_errors();
  }
};
}  // namespace

int qag61(const Integrand& f, double a, double b, double epsabs, double epsrel, size_t limit, double* result,
          double* abserr)
{
  const Panel p0 = gk61(f, a, b);
  double tol = std::max(epsabs, epsrel * std::fabs(p0.result));
  const double round_off = 50 * DBL_EPSILON * p0.resabs;
  *result = p0.result;
  *abserr = p0.abserr;
  if (p0.abserr <= round_off && p0.abserr > tol)
    return 18;
  if ((p0.abserr <= tol && p0.abserr != p0.resasc) || p0.abserr == 0.0)
    return 0;
  if (limit == 1)
    return 11;

  IntervalList w(limit);
  w.a[0] = a;
  w.b[0] = b;
  w.r[0] = p0.result;
  w.e[0] = p0.abserr;
  w.order[0] = 0;
  w.level[0] = 0;
  w.size = 1;
  double area = p0.result, errsum = p0.abserr;
  size_t it = 1;
  int rt1 = 0, rt2 = 0, etype = 0;
  do {
    const double ai = w.a[w.i], bi = w.b[w.i], ri = w.r[w.i], ei = w.e[w.i];
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    const Panel p1 = gk61(f, a1, b1), p2 = gk61(f, a2, b2);
    const double area12 = p1.result + p2.result, err12 = p1.abserr + p2.abserr;
    errsum += err12 - ei;
    area += area12 - ri;
    if (p1.resasc != p1.abserr && p2.resasc != p2.abserr) {
      const double delta = ri - area12;
      if (std::fabs(delta) <= 1.0e-5 * std::fabs(area12) && err12 >= 0.99 * ei)
        rt1++;
      if (it >= 10 && err12 > ei)
        rt2++;
    }
    tol = std::max(epsabs, epsrel * std::fabs(area));
    if (errsum > tol) {
      if (rt1 >= 6 || rt2 >= 20)
        etype = 2;
      const double tmp = (1 + 100 * DBL_EPSILON) * (std::fabs(a2) + 1000 * DBL_MIN);
      if (std::fabs(a1) <= tmp && std::fabs(b2) <= tmp)
        etype = 3;
    }
    w.split(a1, b1, p1.result, p1.abserr, a2, b2, p2.result, p2.abserr);
    it++;
  } while (it < limit && !etype && errsum > tol);
  double sum = 0;
  for (size_t q = 0; q < w.size; q++)
    sum += w.r[q];
  *result = sum;
  *abserr = errsum;
  if (errsum <= tol)
    return 0;
  return etype == 2 ? 18 : (etype == 3 ? 21 : (it == limit ? 11 : 5));
}

// ================================================================= Brent
// Brent (1973) bracketing iteration with inverse quadratic / secant steps and
// bisection fallback; the bracket [lower, upper] is tested after each step
// with |upper - lower| < epsrel * min(|lower|, |upper|).
double brent_root(const std::function<double(double)>& f, double lo, double hi, double epsrel, int max_iter)
{
  double a = lo, b = hi, fa = f(lo), fb = f(hi);
  double c = hi, fc = fb, d = hi - lo, e = hi - lo;
  double root = 0.5 * (lo + hi), xl = lo, xu = hi;
  for (int iter = 1; iter <= max_iter; iter++) {
    bool ac_equal = false;
    bool done_now = false;
    double na = a, nb = b, nc = c, nfa = fa, nfb = fb, nfc = fc, nd = d, ne = e;
    if ((nfb < 0 && nfc < 0) || (nfb > 0 && nfc > 0)) {
      ac_equal = true;
      nc = na;
      nfc = nfa;
      nd = nb - na;
      ne = nb - na;
    }
    if (std::fabs(nfc) < std::fabs(nfb)) {
      ac_equal = true;
      na = nb;
      nb = nc;
      nc = na;
      nfa = nfb;
      nfb = nfc;
      nfc = nfa;
    }
    const double tol = 0.5 * DBL_EPSILON * std::fabs(nb);
    const double m = 0.5 * (nc - nb);
    if (nfb == 0) {
      root = nb;
      xl = nb;
      xu = nb;
      done_now = true;
    } else if (std::fabs(m) <= tol) {
      root = nb;
      xl = std::min(nb, nc);
      xu = std::max(nb, nc);
      if (!(nb < nc)) {
        xl = nc;
        xu = nb;
      } else {
        xl = nb;
        xu = nc;
      }
      done_now = true;
    }
    if (!done_now) {
      if (std::fabs(ne) < tol || std::fabs(nfa) <= std::fabs(nfb)) {
        nd = m;
        ne = m;
      } else {
        double p, q, r;
        const double s = nfb / nfa;
        if (ac_equal) {
          p = 2 * m * s;
          q = 1 - s;
        } else {
          q = nfa / nfc;
          r = nfb / nfc;
          p = s * (2 * m * q * (q - r) - (nb - na) * (r - 1));
          q = (q - 1) * (r - 1) * (s - 1);
        }
        if (p > 0)
          q = -q;
        else
          p = -p;
        if (2 * p < std::min(3 * m * q - std::fabs(tol * q), std::fabs(ne * q))) {
          ne = nd;
          nd = p / q;
        } else {
          nd = m;
          ne = m;
        }
      }
      na = nb;
      nfa = nfb;
      if (std::fabs(nd) > tol)
        nb += nd;
      else
        nb += (m > 0 ? +tol : -tol);
      nfb = f(nb);
      root = nb;
      if ((nfb < 0 && nfc < 0) || (nfb > 0 && nfc > 0))
        nc = na;
      if (nb < nc) {
        xl = nb;
        xu = nc;
      } else {
        xl = nc;
        xu = nb;
      }
      a = na;
      b = nb;
      c = nc;
      fa = nfa;
      fb = nfb;
      fc = nfc;
      d = nd;
      e = ne;
    }
    // interval test (absolute tolerance 0)
    double min_abs = 0;
    if ((xl > 0 && xu > 0) || (xl < 0 && xu < 0))
      min_abs = std::min(std::fabs(xl), std::fabs(xu));
    if (std::fabs(xu - xl) < epsrel * min_abs)
      break;
  }
  return root;
}

// =========================================================== cosmology
void Derived::init(const mx_params& p)
{
  unit_time_s = p.unit_length_cm / p.unit_velocity_cm_s;
  G = k::GRAVITY / std::pow(p.unit_length_cm, 3) * p.unit_mass_g * std::pow(unit_time_s, 2);
  hubble_int = k::HUBBLE * unit_time_s;
  rho_crit = 3 * hubble_int * hubble_int / (8 * k::PI * G);
  const double rhocrit_cgs = 3.0 * k::HUBBLE * k::HUBBLE * p.hubble_h * p.hubble_h / (8.0 * k::PI * k::GRAVITY);
  const double omb = p.baryon_frac * p.omega_m;
  no = rhocrit_cgs * omb * (1 - p.y_he) / k::PROTONMASS;
  he_no = rhocrit_cgs * omb * p.y_he / (4.0 * k::PROTONMASS);
  f_h = no / (no + he_no);
  f_he = he_no / (no + he_no);
  n_b0 = no + he_no;
}

// XRayHeatingFunctions.c:377-392
double dtdz(const mx_params& p, float z)
{
  const double OMl = p.omega_lambda, OMm = p.omega_m;
  const double x = std::sqrt(OMl / OMm) * std::pow(1 + z, -3.0 / 2.0);
  const double dxdz = std::sqrt(OMl / OMm) * std::pow(1 + z, -5.0 / 2.0) * (-3.0 / 2.0);
  const double const1 = 2 * std::sqrt(1 + OMm / OMl) / (3.0 * k::HUBBLE * p.hubble_h);
  const double numer = dxdz * (1 + x * std::pow(std::pow(x, 2) + 1, -0.5));
  const double denom = x + std::sqrt(std::pow(x, 2) + 1);
  return const1 * numer / denom;
}

// XRayHeatingFunctions.c:395-404
double hubble(const mx_params& p, float z)
{
  return k::HUBBLE * p.hubble_h *
         std::sqrt(p.omega_m * std::pow(1 + z, 3) + p.omega_r * std::pow(1 + z, 4) + p.omega_lambda);
}

double drdz(const mx_params& p, float z) { return (1.0 + z) * k::C * dtdz(p, z); }

// gettime, XRayHeatingFunctions.c:483-494: age of a flat universe at z (s)
double gettime(const mx_params& p, double z)
{
  const double OMl = p.omega_lambda, OMm = p.omega_m;
  const double x = std::sqrt(OMl / OMm) * std::pow(1 + z, -3.0 / 2.0);
  const double term1 = std::log(x + std::sqrt(std::pow(x, 2) + 1));
  const double const1 = 2 * std::sqrt(1 + OMm / OMl) / (3 * k::HUBBLE * p.hubble_h);
  return term1 * const1;
}

// find_HII_bubbles.c:26-45
double RtoM(const mx_params& p, const Derived& d, double R)
{
  if (p.rtom_filter_type == 1)
    return std::pow(2 * k::PI, 1.5) * p.omega_m * d.rho_crit * std::pow(R, 3);
  return (4.0 / 3.0) * k::PI * std::pow(R, 3) * (p.omega_m * d.rho_crit);
}

// XRayHeatingFunctions.c:1469-1503
double dicke(const mx_params& p, double z)
{
  const double OMm = p.omega_m, OMl = p.omega_lambda, OMr = p.omega_r;
  if (std::fabs(OMm - 1.0) < 1e-4)
    return 1.0 / (1.0 + z);
  const double om_z = OMm * std::pow(1 + z, 3) / (OMl + OMm * std::pow(1 + z, 3) + OMr * std::pow(1 + z, 4));
  const double dz = 2.5 * om_z / (1.0 / 70.0 + om_z * (209 - om_z) / 140.0 + std::pow(om_z, 4.0 / 7.0));
  const double d0 = 2.5 * OMm / (1.0 / 70.0 + OMm * (209 - OMm) / 140.0 + std::pow(OMm, 4.0 / 7.0));
  return dz / (d0 * (1.0 + z));
}

// XRayHeatingFunctions.c:1506-1511 (float step)
double ddicke_dz(const mx_params& p, double z)
{
  const float dz = 1e-10f;
  return (dicke(p, z + dz) - dicke(p, z)) / dz;
}

// find_HII_bubbles.c:97-100, 184-207, 445
std::vector<double> filter_radii(const mx_params& p)
{
  const double L = p.box_size, D = p.grid_dim;
  double clf = k::L_FACTOR;
  if (L / D < 1.0)
    clf = 1.0;
  const double rmax = p.flag_recombinations ? p.r_bubble_max_recomb : p.r_bubble_max;
  double R = std::fmin(rmax, k::L_FACTOR * L);
  std::vector<double> out;
  for (;;) {
    const bool last = ((R / p.delta_r_factor) <= (clf * L / D)) || ((R / p.delta_r_factor) <= p.r_bubble_min);
    if (last)
      R = clf * L / D;
    out.push_back(R);
    if (last)
      break;
    R /= p.delta_r_factor;
    if (out.size() > 100000)
      break;
  }
  return out;
}

// ===================================================== recombination table
namespace {
double alpha_B(double T) { return k::ALPHAB_10K * std::pow(T / 1.0e4, -0.75); }

struct Mhr
{
  const mx_params* p;
  NaturalSpline A, C, beta;
  double C_at(double z) const
  {
    if (z >= 13.0)
      return 1.0;
    if (z <= 2.0)
      return 0.558;
    return C.eval(z);
  }
  double beta_at(double z) const
  {
    if (z >= 6.0)
      return -2.50;
    if (z <= 2.0)
      return -2.23;
    return beta.eval(z);
  }
  double A_at(double z) const
  {
    if (z >= 2.0 + (float)k::A_NPTS)
      return A.eval(2.0 + (float)k::A_NPTS);
    if (z <= 2.0)
      return A.eval(2.0);
    return A.eval(z);
  }
};

// recombinations.c:332-357 (case B)
double neutral_fraction_B(double y_he, double density, double T4, double gamma12)
{
  const double corr_He = 1.0 / (4.0 / y_he - 3);
  const double alpha = alpha_B(T4 * 1e4);
  gamma12 *= 1e-12;
  double chi = (1 + corr_He) * density * alpha / gamma12;
  if (chi < k::TINY)
    return 0;
  if (chi < 1e-5)
    return chi;
  const double b = -2 - gamma12 / (density * (1 + corr_He) * alpha);
  return (-b - std::sqrt(b * b - 4)) / 2.0;
}
}  // namespace

void RecombTable::build(const mx_params& p, const Derived& d, int nthreads)
{
  Mhr m;
  m.p = &p;
  double xs[k::A_NPTS], ys[k::A_NPTS];
  static const double C_tab[k::C_NPTS] = { 0.558, 0.599, 0.611, 0.769, 0.868, 0.930,
                                           0.964, 0.983, 0.993, 0.998, 0.999, 1.00 };
  static const double beta_tab[k::BETA_NPTS] = { -2.23, -2.35, -2.48, -2.49, -2.50 };
  for (int i = 0; i < k::C_NPTS; i++)
    xs[i] = (float)i + 2.0;
  m.C.init(xs, C_tab, k::C_NPTS);
  for (int i = 0; i < k::BETA_NPTS; i++)
    xs[i] = (float)i + 2.0;
  m.beta.init(xs, beta_tab, k::BETA_NPTS);
  // A parameter: 1 / integral of the MHR00 PDF shape (recombinations.c:160-216)
  for (int i = 0; i < k::A_NPTS; i++) {
    const double z = 2.0 + (float)i;
    const double Cz = m.C_at(z), bz = m.beta_at(z);
    const double s = 2.0 * 7.61 / (3.0 * (1.0 + z));
    auto aux = [&](double D) {
      return std::exp(-(std::pow(D, -2.0 / 3.0) - Cz) * (std::pow(D, -2.0 / 3.0) - Cz) / (2.0 * s * s)) *
             std::pow(D, bz);
    };
    double res, err;
    qag61(aux, 1e-25, 1e25, 0, 0.001, 1000, &res, &err);
    xs[i] = z;
    ys[i] = 1.0 / res;
  }
  m.A.init(xs, ys, k::A_NPTS);

  lng.resize(k::RR_LNG_NPTS);
  for (int g = 0; g < k::RR_LNG_NPTS; g++)
    lng[g] = k::RR_LNG_MIN + g * k::RR_DEL_LNG;
  y.assign((size_t)k::RR_Z_NPTS * k::RR_LNG_NPTS, 0.0);
  c.assign((size_t)k::RR_Z_NPTS * k::RR_LNG_NPTS, 0.0);
  const double y_he = p.y_he;
  const double no = d.no;
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (;;) {
      const int z_ct = next.fetch_add(1);
      if (z_ct >= k::RR_Z_NPTS)
        break;
      const float z = z_ct * k::RR_DEL_Z;
      const double zd = z;
      const double A = m.A_at(zd), C0 = m.C_at(zd), beta = m.beta_at(zd), avenH = no * std::pow(1 + zd, 3);
      std::vector<double> row(k::RR_LNG_NPTS);
      for (int g = 0; g < k::RR_LNG_NPTS; g++) {
        const float gamma = (float)std::exp(lng[g]);
        const double gbg = gamma, T4 = 1.0;
        // MHR_rr, recombinations.c:116-135, integrated over ln Delta in [ln 0.01, ln 200]
        auto rr = [&](double lnD) {
          const double D = std::exp(lnD);
          const double Dss = 26.7 * std::pow(T4, 0.17) * std::pow((1 + zd) / 10.0, -3) * std::pow(gbg, 2.0 / 3.0);
          const double gam =
            gbg * (0.98 * std::pow((1.0 + std::pow(D / Dss, 1.64)), -2.28) + 0.02 * std::pow(1.0 + D / Dss, -0.84));
          const double n_H = avenH * D;
          const double x_e = 1.0 - neutral_fraction_B(y_he, n_H, T4, gam);
          const double PDelta =
            A * std::exp(-0.5 * std::pow((std::pow(D, -2.0 / 3.0) - C0) / ((2.0 * 7.61 / (3.0 * (1.0 + zd)))), 2)) *
            std::pow(D, beta);
          return n_H * PDelta * alpha_B(T4 * 1e4) * x_e * x_e * D * D;
        };
        double res, err;
        qag61(rr, std::log(0.01), std::log(200), 0, 0.01, 1000, &res, &err);
        row[g] = res;
      }
      NaturalSpline sp;
      sp.init(lng.data(), row.data(), k::RR_LNG_NPTS);
      std::memcpy(&y[(size_t)z_ct * k::RR_LNG_NPTS], sp.y.data(), sizeof(double) * k::RR_LNG_NPTS);
      std::memcpy(&c[(size_t)z_ct * k::RR_LNG_NPTS], sp.c.data(), sizeof(double) * k::RR_LNG_NPTS);
    }
  };
  std::vector<std::thread> pool;
  const int nt = std::max(1, nthreads);
  for (int t = 0; t < nt; t++)
    pool.emplace_back(worker);
  for (auto& t : pool)
    t.join();
  ready = true;
}

// ========================================================== heat tables
int HeatTables::load(const mx_params& p, const std::string& dir, std::string* err)
{
  char fn[2048];
  FILE* F;
  auto fail = [&](const char* what) {
    if (err)
      *err = std::string("cannot read ") + what;
    return MX_ETABLE;
  };
  // recfast_LCDM.dat, read bottom-up into ascending z (XRayHeatingFunctions.c:104-148)
  std::snprintf(fn, sizeof fn, "%s/recfast_LCDM.dat", dir.c_str());
  if (!(F = std::fopen(fn, "r")))
    return fail(fn);
  std::vector<double> zt(k::RECFAST_NPTS), tk(k::RECFAST_NPTS), xi(k::RECFAST_NPTS);
  for (int i = k::RECFAST_NPTS - 1; i >= 0; i--) {
    float cz, cx, trash, ct;
    if (std::fscanf(F, "%f %E %E %E", &cz, &cx, &trash, &ct) != 4) {
      std::fclose(F);
      return fail(fn);
    }
    zt[i] = cz;
    xi[i] = cx;
    tk[i] = ct;
  }
  std::fclose(F);
  recfast_T.init(zt.data(), tk.data(), k::RECFAST_NPTS);
  recfast_x.init(zt.data(), xi.data(), k::RECFAST_NPTS);
  recfast_zmax = zt[k::RECFAST_NPTS - 1];

  // Zygelman (2005) kappa_10^HH table, XRayHeatingFunctions.c:1612-1676
  static const double tk10[k::KAPPA_10_NPTS] = { 1.0,   2.0,   4.0,   6.0,   8.0,    10.0,   15.0,   20.0,   25.0,
                                                 30.0,  40.0,  50.0,  60.0,  70.0,   80.0,   90.0,   100.0,  200.0,
                                                 300.0, 501.0, 701.0, 1000.0, 2000.0, 3000.0, 5000.0, 7000.0, 10000.0 };
  static const double k10[k::KAPPA_10_NPTS] = { 1.38e-13, 1.43e-13, 2.71e-13, 6.60e-13, 1.47e-12, 2.88e-12, 9.10e-12,
                                                1.78e-11, 2.73e-11, 3.67e-11, 5.38e-11, 6.86e-11, 8.14e-11, 9.25e-11,
                                                1.02e-10, 1.11e-10, 1.19e-10, 1.75e-10, 2.09e-10, 2.565e-10, 2.91e-10,
                                                3.31e-10, 4.27e-10, 4.97e-10, 6.03e-10, 6.87e-10, 7.87e-10 };
  double lt[k::KAPPA_10_NPTS], lk[k::KAPPA_10_NPTS];
  for (int i = 0; i < k::KAPPA_10_NPTS; i++) {
    lt[i] = std::log(tk10[i]);
    lk[i] = std::log(k10[i]);
  }
  kap10.init(lt, lk, k::KAPPA_10_NPTS);
  const char* names[2] = { "kappa_eH_table.dat", "kappa_pH_table.dat" };
  const int counts[2] = { k::KAPPA_E_NPTS, k::KAPPA_P_NPTS };
  NaturalSpline* dst[2] = { &kap_e, &kap_p };
  for (int t = 0; t < 2; t++) {
    std::snprintf(fn, sizeof fn, "%s/%s", dir.c_str(), names[t]);
    if (!(F = std::fopen(fn, "r")))
      return fail(fn);
    std::vector<double> a(counts[t]), b(counts[t]);
    for (int i = 0; i < counts[t]; i++) {
      float x0, y0;
      if (std::fscanf(F, "%f %e", &x0, &y0) != 2) {
        std::fclose(F);
        return fail(fn);
      }
      a[i] = std::log((double)x0);
      b[i] = std::log((double)y0);
    }
    std::fclose(F);
    dst[t]->init(a.data(), b.data(), counts[t]);
  }

  // Pop II stellar spectra, XRayHeatingFunctions.c:618-650
  std::snprintf(fn, sizeof fn, "%s/stellar_spectra.dat", dir.c_str());
  if (!(F = std::fopen(fn, "r")))
    return fail(fn);
  int nidx[k::NSPEC_MAX] = { 0 };
  for (int i = 1; i < k::NSPEC_MAX; i++) {
    float n2, a2, n3, a3;
    if (std::fscanf(F, "%i %e %e %e %e", &nidx[i], &n2, &a2, &n3, &a3) != 5) {
      std::fclose(F);
      return fail(fn);
    }
    spec_N0[i] = n2;
    spec_alpha[i] = a2;
  }
  std::fclose(F);
  for (int i = 1; i < k::NSPEC_MAX; i++)
    spec_nu[i] = (float)(4.0 / 3.0 * (1.0 - 1.0 / std::pow(nidx[i], 2.0)));
  for (int i = 1; i < k::NSPEC_MAX - 1; i++) {
    const double n0_fac = std::pow(spec_nu[i + 1], spec_alpha[i] + 1) - std::pow(spec_nu[i], spec_alpha[i] + 1);
    spec_N0[i] *= (spec_alpha[i] + 1) / n0_fac * p.nion_phot_per_bary;
  }

  // secondary-electron tables, XRayHeatingFunctions.c:805-905
  static const float xh[k::NXHII] = { 1.0e-4f, 2.318e-4f, 4.677e-4f, 1.0e-3f, 2.318e-3f, 4.677e-3f, 1.0e-2f,
                                     2.318e-2f, 4.677e-2f, 1.0e-1f, 0.5f, 0.9f, 0.99f, 0.999f };
  std::memcpy(xhii, xh, sizeof xh);
  for (int n = 0; n < k::NXHII; n++) {
    if (xhii[n] < 0.3)
      std::snprintf(fn, sizeof fn, "%s/x_int_tables/log_xi_%1.1f.dat", dir.c_str(), std::log10(xhii[n]));
    else
      std::snprintf(fn, sizeof fn, "%s/x_int_tables/xi_%1.3f.dat", dir.c_str(), xhii[n]);
    if (!(F = std::fopen(fn, "r")))
      return fail(fn);
    char label[64];
    float f1, f2, f3, f4, f5, trash;
    bool ok = true;
    for (int i = 0; i < 5 && ok; i++)
      ok = std::fscanf(F, "%63s", label) == 1;
    ok = ok && std::fscanf(F, "%g %g %g %g %g", &f1, &f2, &f3, &f4, &f5) == 5;
    for (int i = 0; i < 11 && ok; i++)
      ok = std::fscanf(F, "%63s", label) == 1;
    for (int i = 0; i < k::NENERGY && ok; i++)
      ok = std::fscanf(F, "%g %g %g %g %g %g %g %g %g", &energy[i], &trash, &fheat[n][i], &trash, &nlya[n][i],
                       &nion_hi[n][i], &nion_hei[n][i], &nion_heii[n][i], &trash) == 9;
    std::fclose(F);
    if (!ok)
      return fail(fn);
  }
  ready = true;
  return 0;
}

double HeatTables::T_recfast(float z) const { return z > recfast_zmax ? -1 : recfast_T.eval(z); }
double HeatTables::xion_recfast(float z) const { return z > recfast_zmax ? -1 : recfast_x.eval(z); }

// ============================================================ shell plan
// set_sfr_history, ComputeTs.c:32-76
int n_sfr_histories(const mx_params& p, const std::vector<double>& zz)
{
  const double box = p.box_size / p.hubble_h;
  const int D = p.grid_dim, S = p.ts_num_filter_steps;
  int max_snaps = 0;
  for (int s = 1; s < (int)zz.size(); s++) {
    const double zp = zz[s];
    double R = k::L_FACTOR * box / (float)D;
    const double Rf = std::pow(k::R_XLY_MAX / R, 1 / (float)S);
    int scb = 1;
    double prev_R = 0, prev_zpp = zp;
    for (int r = 0; r < S; r++) {
      const double edge = prev_zpp - (R - prev_R) * k::MPC / drdz(p, (float)prev_zpp);
      while (edge > zz[s - scb]) {
        if (s - scb == 0)
          break;
        scb++;
      }
      prev_R = R;
      prev_zpp = edge;
      R *= Rf;
    }
    max_snaps = std::max(max_snaps, scb);
  }
  return max_snaps;
}

// The scalar control flow of _ComputeTs' shell loop, ComputeTs.c:270-377:
// shell radii and redshift edges, and the sequence of operations applied to
// the sfr grid before each shell's forward FFT.
ShellPlan plan_shells(const mx_params& p, const std::vector<double>& zz, int snapshot)
{
  ShellPlan sp;
  const int S = p.ts_num_filter_steps;
  const int D = p.grid_dim;
  sp.S = S;
  const double zp = zz[snapshot];
  const double prev_z = snapshot == 0 ? zz[snapshot] : zz[snapshot - 1];
  const double dzp = zp - prev_z;
  sp.homogeneous = (zp - p.max_heating_redshift) >= -0.0001;
  if (sp.homogeneous)
    return sp;
  const double dt_dzp = dtdz(p, (float)zp);
  const double box = p.box_size / p.hubble_h;
  double R = k::L_FACTOR * box / (float)D;
  const double Rf = std::pow(k::R_XLY_MAX / R, 1 / (float)S);
  sp.R.resize(S);
  sp.zpp_edge.resize(S);
  sp.ops.resize(S);
  std::vector<int> scb(S);
  scb[0] = 1;
  double weight = 1;
  const double* ZZ = zz.data();
  for (int r = 0; r < S; r++) {
    double prev_zpp, prev_R;
    sp.R[r] = R;
    if (r == 0) {
      prev_zpp = zp;
      prev_R = 0;
    } else {
      prev_zpp = sp.zpp_edge[r - 1];
      prev_R = sp.R[r - 1];
      scb[r] = scb[r - 1];
    }
    sp.zpp_edge[r] = prev_zpp - (R - prev_R) * k::MPC / drdz(p, (float)prev_zpp);
    const double zpp = (sp.zpp_edge[r] + prev_zpp) * 0.5;
    const double total_weight = (prev_zpp - sp.zpp_edge[r]) * dtdz(p, (float)zpp);
    auto& ops = sp.ops[r];
    if (snapshot - scb[r] >= 0) {
      if (snapshot - scb[r] == 0 && weight < 0) {
        ops.push_back({ SfrOp::ZERO_HALF, 0, 0.f, 0.0 });
        scb[r] += 1;
      } else if (sp.zpp_edge[r] > ZZ[snapshot - scb[r]]) {
        if (r == 0) {
          weight = dt_dzp * dzp / total_weight;
          ops.push_back({ SfrOp::SCALE_HALF, 0, 0.f, weight });
        } else {
          if (ZZ[snapshot - scb[r]] > sp.zpp_edge[r - 1]) {
            weight = -dtdz(p, (float)(0.5 * (ZZ[snapshot - scb[r]] + sp.zpp_edge[r - 1])));
            weight *= (ZZ[snapshot - scb[r]] - sp.zpp_edge[r - 1]);
            weight /= total_weight;
            ops.push_back({ SfrOp::LOAD, scb[r] - 1, (float)weight, 0.0 });
          } else {
            ops.push_back({ SfrOp::ZERO_HALF, 0, 0.f, 0.0 });
          }
        }
        while (sp.zpp_edge[r] > ZZ[snapshot - scb[r]]) {
          if (snapshot - scb[r] == 0) {
            weight = -1;
            break;
          }
          if (sp.zpp_edge[r] < ZZ[snapshot - scb[r] - 1]) {
            // the conditional expression of ComputeTs.c:345, as written
            const double zprev = r > 0 ? sp.zpp_edge[r - 1] : 0.0;
            const double zedge = zprev ? ZZ[snapshot - scb[r]] : (double)(zprev > ZZ[snapshot - scb[r]]);
            weight = sp.zpp_edge[r] - zedge;
            weight *= -dtdz(p, (float)(0.5 * (sp.zpp_edge[r] + zedge)));
          } else {
            weight = ZZ[snapshot - scb[r] - 1] - ZZ[snapshot - scb[r]];
            weight *= -dtdz(p, (float)(0.5 * (ZZ[snapshot - scb[r] - 1] + ZZ[snapshot - scb[r]])));
          }
          weight /= total_weight;
          ops.push_back({ SfrOp::ADD, scb[r], (float)weight, 0.0 });
          scb[r] += 1;
        }
      } else if (r > 0 && weight != 1) {
        weight = 1;
        ops.push_back({ SfrOp::LOAD, scb[r] - 1, (float)weight, 0.0 });
      }
    }
    R *= Rf;
  }
  sp.weight_after = weight;
  // evolveInt shell factors (XRayHeatingFunctions.c:1289-1330)
  sp.a_dt_dz.resize(S);
  sp.b_pow.resize(S);
  sp.zpp1.resize(S);
  sp.dt_dzpp.resize(S);
  sp.dzpp.resize(S);
  const float zpf = (float)zp;
  for (int r = 0; r < S; r++) {
    double zpp, dzpp;
    if (r == 0) {
      zpp = (sp.zpp_edge[0] + zpf) * 0.5;
      dzpp = zpf - sp.zpp_edge[0];
    } else {
      zpp = (sp.zpp_edge[r] + sp.zpp_edge[r - 1]) * 0.5;
      dzpp = sp.zpp_edge[r - 1] - sp.zpp_edge[r];
    }
    sp.dt_dzpp[r] = dtdz(p, (float)zpp);
    sp.dzpp[r] = dzpp;
    sp.a_dt_dz[r] = sp.dt_dzpp[r] * dzpp;
    sp.b_pow[r] = std::pow(1 + zpp, -p.spec_index_xray_gal);
    sp.zpp1[r] = 1 + zpp;
  }
  return sp;
}

// ====================================================== frequency tables
namespace {
double xs_HI(double nu)
{
  if (nu < k::NU_HI)
    return 0;
  if (nu == k::NU_HI)
    nu += k::TINY;
  const double eps = std::sqrt(nu / k::NU_HI - 1);
  return k::SIGMA_HI * std::pow(k::NU_HI / nu, 4) * std::exp(4 - (4 * std::atan(eps) / eps)) /
         (1 - std::exp(-2 * k::PI / eps));
}
double xs_HeII(double nu)
{
  const double Z = 2;
  if (nu < k::NU_HEII)
    return 0;
  if (nu == k::NU_HEII)
    nu += k::TINY;
  const double eps = std::sqrt(nu / k::NU_HEII - 1);
  return (6.3e-18) / Z / Z * std::pow(k::NU_HEII / nu, 4) * std::exp(4 - (4 * std::atan(eps) / eps)) /
         (1 - std::exp(-2 * k::PI / eps));
}
double xs_HeI(double nu)
{
  if (nu < k::NU_HEI)
    return 0;
  const double x = nu / k::NU_OVER_EV / 13.61 - 0.4434;
  const double y = std::sqrt(x * x + std::pow(2.136, 2));
  return 9.492e-16 * ((x - 1) * (x - 1) + 2.039 * 2.039) * std::pow(y, (0.5 * 3.188 - 5.5)) *
         std::pow(1.0 + std::sqrt(y / 1.469), -3.188);
}

int loc_energy(float En)
{
  if (En < 1008.88)
    return (int)(std::log(En / 10.0) / 1.98026273e-2);
  return 232 + (int)(std::log(En / 1008.88) / 9.53101798e-2);
}
int loc_xhii(const HeatTables& ht, float x)
{
  int m = k::NXHII - 1;
  while (x < ht.xhii[m])
    m--;
  return m;
}

// bilinear table lookup in float (XRayHeatingFunctions.c:914-1190)
float interp_tab(const HeatTables& ht, const float (*tab)[k::NENERGY], float below, float En, float x)
{
  if (En > 0.999 * ht.energy[k::NENERGY - 1])
    En = (float)(ht.energy[k::NENERGY - 1] * 0.999);
  else if (En < ht.energy[0])
    return below;
  if (x > ht.xhii[k::NXHII - 1] * 0.999)
    x = (float)(ht.xhii[k::NXHII - 1] * 0.999);
  else if (x < ht.xhii[0])
    x = (float)(1.001 * ht.xhii[0]);
  const int n0 = loc_energy(En), n1 = n0 + 1;
  const int m0 = loc_xhii(ht, x), m1 = m0 + 1;
  const float* E = ht.energy;
  float lo = (tab[m0][n1] - tab[m0][n0]) / (E[n1] - E[n0]);
  lo *= (En - E[n0]);
  lo += tab[m0][n0];
  float hi = (tab[m1][n1] - tab[m1][n0]) / (E[n1] - E[n0]);
  hi *= (En - E[n0]);
  hi += tab[m1][n0];
  float r = (hi - lo) / (ht.xhii[m1] - ht.xhii[m0]);
  r *= (x - ht.xhii[m0]);
  r += lo;
  return r;
}

float zmax_f(float z, int n)
{
  const double num = 1 - std::pow(n + 1, -2), den = 1 - std::pow(n, -2);
  return (float)((1 + z) * num / den - 1);
}
double nu_n(int n) { return (1.0 - std::pow(n, -2.0)) / 0.75; }
double frecycle(int n)
{
  static const double t[31] = { 1,      1,      1,      0,      0.2609, 0.3078, 0.3259, 0.3353, 0.3410, 0.3448, 0.3476,
                                0.3496, 0.3512, 0.3524, 0.3535, 0.3543, 0.3550, 0.3556, 0.3561, 0.3565, 0.3569, 0.3572,
                                0.3575, 0.3578, 0.3580, 0.3582, 0.3584, 0.3586, 0.3587, 0.3589, 0.3590 };
  return (n >= 0 && n <= 30) ? t[n] : 0;
}
double spectral_emissivity(const HeatTables& ht, double nu_norm)
{
  for (int i = 1; i < k::NSPEC_MAX - 1; i++)
    if (nu_norm >= ht.spec_nu[i] && nu_norm < ht.spec_nu[i + 1])
      return ht.spec_N0[i] * std::pow(nu_norm, ht.spec_alpha[i]) / k::LYA_HZ;
  const int i = k::NSPEC_MAX - 1;
  return ht.spec_N0[i] * std::pow(nu_norm, ht.spec_alpha[i]) / k::LYA_HZ;
}

void parallel_for(int n, int nthreads, const std::function<void(int)>& fn)
{
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n)
        break;
      fn(i);
    }
  };
  const int nt = std::max(1, std::min(nthreads, n));
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++)
    pool.emplace_back(worker);
  worker();
  for (auto& t : pool)
    t.join();
}
}  // namespace

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
                       FreqTables* out)
{
  const int S = sp.S;
  const double zp = zz[snapshot];
  out->tab.assign((size_t)3 * k::NXHII * S, 0.0);
  out->sum_lyn.assign(S, 0.0);
  const double eff = p.reion_efficiency;

  // interpolate_fcoll (XRayHeatingFunctions.c:1884-1900)
  auto fcoll_at = [&](double z) {
    double v;
    if (snapshot == 0)
      v = stored_fcoll[snapshot];
    else
      v = stored_fcoll[snapshot - 1] +
          (z - zz[snapshot - 1]) * (stored_fcoll[snapshot] - stored_fcoll[snapshot - 1]) /
            (zz[snapshot] - zz[snapshot - 1]);
    return v < 0.0 ? 0.0 : v;
  };
  // tauX (XRayHeatingFunctions.c:307-375)
  auto tauX = [&](double nu, double x_e, double zpp) {
    const double nu_0 = nu / (1 + zp);
    auto integrand = [&](double zhat) {
      const double drpropdz = k::C * dtdz(p, (float)zhat);
      const double n = d.n_b0 * std::pow(1 + zhat, 3);
      const double nuhat = nu_0 * (1 + zhat);
      const double fc = fcoll_at(zhat);
      double HI = fc < 1e-20 ? 1 : 1 - (eff * fc) / (1.0 - x_e_ave);
      if (HI < 1e-4)
        HI = 1e-4;
      const double sig = d.f_h * (1 - x_e) * xs_HI(nuhat) + d.f_he * (1 - x_e) * xs_HeI(nuhat) +
                         d.f_he * x_e * xs_HeII(nuhat);
      return drpropdz * n * HI * sig;
    };
    double res, err;
    qag61(integrand, zpp, zp, 0, 0.005, 1000, &res, &err);
    return res;
  };
  // nu_tau_one (XRayHeatingFunctions.c:229-297)
  auto nu_tau_one = [&](double zpp, double x_e) {
    if (x_e > 0.9999)
      return -1.0;
    if (tauX(k::NU_HEI, x_e, zpp) < 1)
      return k::NU_HEI;
    return brent_root([&](double nu) { return tauX(nu, x_e, zpp) - 1; }, k::NU_HEI, 1e6 * k::NU_OVER_EV, 0.02, 100);
  };

  std::vector<double> zpp_mid(S), lower(S);
  for (int r = 0; r < S; r++) {
    const double prev_zpp = r == 0 ? zp : sp.zpp_edge[r - 1];
    zpp_mid[r] = (sp.zpp_edge[r] + prev_zpp) * 0.5;
  }
  const double E0 = p.nu_xray_gal_threshold, alpha = p.spec_index_xray_gal;
  parallel_for(S, nthreads, [&](int r) {
    lower[r] = std::fmax(nu_tau_one(zpp_mid[r], x_e_ave), E0 * k::NU_OVER_EV);
  });

  // integrate_over_nu (XRayHeatingFunctions.c:672-800)
  const double f_h = d.f_h, f_he = d.f_he;
  const double numax = p.nu_xray_max * k::NU_OVER_EV;
  const double hub = hubble(p, (float)zp);
  parallel_for(S * k::NXHII * 3, nthreads, [&](int job) {
    const int flag = job % 3;
    const int xi = (job / 3) % k::NXHII;
    const int r = job / (3 * k::NXHII);
    const double xe = ht.xhii[xi];
    const float xef = (float)xe;
    const double nus[3] = { k::NU_HI, k::NU_HEI, k::NU_HEII };
    Integrand fn;
    if (flag == 0) {
      fn = [&](double nu) {
        double s = interp_tab(ht, ht.fheat, 1.0f, (float)((nu - k::NU_HI) / k::NU_OVER_EV), xef) * k::PLANCK *
                   (nu - k::NU_HI) * f_h * (1 - xe) * xs_HI(nu);
        s += interp_tab(ht, ht.fheat, 1.0f, (float)((nu - k::NU_HEI) / k::NU_OVER_EV), xef) * k::PLANCK *
             (nu - k::NU_HEI) * f_he * (1 - xe) * xs_HeI(nu);
        s += interp_tab(ht, ht.fheat, 1.0f, (float)((nu - k::NU_HEII) / k::NU_OVER_EV), xef) * k::PLANCK *
             (nu - k::NU_HEII) * f_he * xe * xs_HeII(nu);
        return s * std::pow(nu / (E0 * k::NU_OVER_EV), -alpha - 1);
      };
    } else if (flag == 1) {
      fn = [&](double nu) {
        double s = 0;
        for (int q = 0; q < 3; q++) {
          const float En = (float)((nu - nus[q]) / k::NU_OVER_EV);
          const double Fi = interp_tab(ht, ht.nion_hi, 0.0f, En, xef) + interp_tab(ht, ht.nion_hei, 0.0f, En, xef) +
                            interp_tab(ht, ht.nion_heii, 0.0f, En, xef) + 1;
          if (q == 0)
            s = Fi * f_h * (1 - xe) * xs_HI(nu);
          else if (q == 1)
            s += Fi * f_he * (1 - xe) * xs_HeI(nu);
          else
            s += Fi * f_he * xe * xs_HeII(nu);
        }
        return s * std::pow(nu / (E0 * k::NU_OVER_EV), -alpha - 1);
      };
    } else {
      fn = [&](double nu) {
        double s = interp_tab(ht, ht.nlya, 0.0f, (float)((nu - k::NU_HI) / k::NU_OVER_EV), xef) * f_h * (1 - xe) *
                   xs_HI(nu);
        s += interp_tab(ht, ht.nlya, 0.0f, (float)((nu - k::NU_HEI) / k::NU_OVER_EV), xef) * f_he * (1 - xe) *
             xs_HeI(nu);
        s += interp_tab(ht, ht.nlya, 0.0f, (float)((nu - k::NU_HEII) / k::NU_OVER_EV), xef) * f_he * xe *
             xs_HeII(nu);
        return s * std::pow(nu / (E0 * k::NU_OVER_EV), -alpha - 1);
      };
    }
    double res, err;
    qag61(fn, lower[r], numax, 0, 0.01, 1000, &res, &err);
    if (flag == 2)
      res = res * k::C / (4 * k::PI) / k::LYA_HZ / hub;
    out->tab[((size_t)flag * k::NXHII + xi) * S + r] = res;
  });

  // Ly-n sums and the kink correction (ComputeTs.c:585-663)
  bool first_radii = true, first_zero = true;
  double weight = weight_in;
  const int n_pts_radii = 1000;
  for (int r = 0; r < S; r++) {
    const double prev_zpp = r == 0 ? zp : sp.zpp_edge[r - 1];
    const double prev_R = r == 0 ? 0 : sp.R[r - 1];
    const double zpp = zpp_mid[r];
    double s = 0;
    for (int n_ct = k::NSPEC_MAX; n_ct >= 2; n_ct--) {
      if (zpp > zmax_f((float)zp, n_ct))
        continue;
      const double nuprime = nu_n(n_ct) * (1 + zpp) / (1.0 + zp);
      s += frecycle(n_ct) * spectral_emissivity(ht, nuprime);
    }
    out->sum_lyn[r] = s;
    if (r > 2 && out->sum_lyn[r] == 0.0 && out->sum_lyn[r - 1] > 0. && first_radii) {
      const double tmax = (prev_zpp - (sp.R[r] - prev_R) * k::MPC / drdz(p, (float)prev_zpp) + prev_zpp) * 0.5;
      const double tmin =
        (sp.zpp_edge[r - 2] - (sp.R[r - 1] - sp.R[r - 2]) * k::MPC / drdz(p, (float)sp.zpp_edge[r - 2]) +
         sp.zpp_edge[r - 2]) *
        0.5;
      for (int ii = 0; ii < n_pts_radii; ii++) {
        const double tz = tmin + (tmax - tmin) * (float)ii / ((float)n_pts_radii - 1.);
        int counter = 0;
        for (int n_ct = k::NSPEC_MAX; n_ct >= 2; n_ct--) {
          if (tz > zmax_f((float)zp, n_ct))
            continue;
          counter++;
        }
        if (counter == 0 && first_zero) {
          first_zero = false;
          weight = (float)ii / (float)n_pts_radii;
        }
      }
      out->sum_lyn[r] = weight * out->sum_lyn[r - 1];
      first_radii = false;
    }
  }

  out->growth_zp = dicke(p, zp);
  out->dgrowth_dzp = ddicke_dz(p, zp);
  out->dt_dzp = dtdz(p, (float)zp);
  // ComputeTs.c:675-724
  double Lc;
  if (std::fabs(alpha - 1.0) < 0.000001) {
    Lc = (E0 * k::NU_OVER_EV) * std::log(p.nu_xray_soft_cut / E0);
    Lc = 1. / Lc;
  } else {
    Lc = std::pow(p.nu_xray_soft_cut * k::NU_OVER_EV, 1. - alpha) - std::pow(E0 * k::NU_OVER_EV, 1. - alpha);
    Lc = 1. / Lc;
    Lc *= std::pow(E0 * k::NU_OVER_EV, -alpha) * (1 - alpha);
  }
  Lc *= k::SEC_PER_YEAR / k::PLANCK;
  out->const_zp_prefactor = (p.lx_gal * Lc) / (E0 * k::NU_OVER_EV) * k::C * std::pow(1 + zp, alpha + 3);
}

}  // namespace mx
