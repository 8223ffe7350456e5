// Host-side tables for the GB300 scalar path.  Each function cites the
// reference routine whose behaviour it follows (paths inside the CAMB source).
#include "cosmo_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <stdexcept>
#include <thread>

namespace cg {

static inline int nint(double x) { return (int)std::lround(x); }

// ------------------------------------------------------------------------
// Ranges (forutils TRanges semantics inferred from the call sites)
// ------------------------------------------------------------------------
static const double kRangeTol = 0.1;

void Ranges::add_delta(double lo, double hi, double delta, bool islog) {
  if (!(hi > lo) || !(delta > 0)) throw std::runtime_error("Ranges::add_delta: bad range");
  int n;
  if (islog)
    n = std::max(1, (int)(std::log(hi / lo) / delta + 1.0 - kRangeTol));
  else
    n = std::max(1, (int)((hi - lo) / delta + 1.0 - kRangeTol));
  add(lo, hi, n, islog);
}

void Ranges::add(double lo, double hi, int n, bool islog) {
  if (!(hi > lo) || n < 1) throw std::runtime_error("Ranges::add: bad range");
  r.push_back({lo, hi, n, islog});
}

static double local_step(const Ranges::R& R, double x) {
  if (R.log) return x * (std::exp(std::log(R.hi / R.lo) / R.n) - 1.0);
  return (R.hi - R.lo) / R.n;
}

void Ranges::get_array(bool want_dpoints) {
  points.clear();
  dpoints.clear();
  std::vector<double> b;
  for (auto& R : r) { b.push_back(R.lo); b.push_back(R.hi); }
  std::sort(b.begin(), b.end());
  b.erase(std::unique(b.begin(), b.end()), b.end());
  for (size_t k = 0; k + 1 < b.size(); ++k) {
    double a = b[k], c = b[k + 1], mid = 0.5 * (a + c);
    const R* best = nullptr;
    double best_step = 0;
    for (auto& R : r) {
      if (R.lo <= a && R.hi >= c) {
        double s = local_step(R, mid);
        if (!best || s < best_step) { best = &R; best_step = s; }
      }
    }
    if (points.empty()) points.push_back(a);
    if (!best) { points.push_back(c); continue; }  // gap between ranges: single step
    int n;
    if (best->lo == a && best->hi == c) n = best->n;
    else if (best->log) n = std::max(1, nint(std::log(c / a) / (std::log(best->hi / best->lo) / best->n)));
    else n = std::max(1, nint((c - a) / ((best->hi - best->lo) / best->n)));
    for (int i = 1; i <= n; ++i) {
      double x;
      if (i == n) x = c;
      else if (best->log) x = a * std::exp(std::log(c / a) * i / n);
      else x = a + (c - a) * i / n;
      points.push_back(x);
    }
  }
  if (want_dpoints) {
    int n = (int)points.size();
    dpoints.resize(n);
    if (n == 1) { dpoints[0] = 0; return; }
    dpoints[0] = (points[1] - points[0]) / 2;
    for (int i = 1; i < n - 1; ++i) dpoints[i] = (points[i + 1] - points[i - 1]) / 2;
    dpoints[n - 1] = (points[n - 1] - points[n - 2]) / 2;
  }
}

int Ranges::index_of(double x) const {
  int n = (int)points.size();
  if (x <= points[0]) return 0;
  if (x >= points[n - 1]) return n - 2;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (x >= points[mid]) lo = mid; else hi = mid;
  }
  return lo;
}

// ------------------------------------------------------------------------
// cubic splines (natural unless clamped)
// ------------------------------------------------------------------------
void spline_second_derivs(const double* x, const double* y, int n, double* d2, bool clamp_start,
                          double d1_start, bool clamp_end, double d1_end) {
  std::vector<double> u(n);
  if (n < 3) { for (int i = 0; i < n; ++i) d2[i] = 0; return; }
  if (!clamp_start) { d2[0] = 0; u[0] = 0; }
  else {
    d2[0] = -0.5;
    u[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - d1_start);
  }
  for (int i = 1; i < n - 1; ++i) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * d2[i - 1] + 2.0;
    d2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double qn, un;
  if (!clamp_end) { qn = 0; un = 0; }
  else {
    qn = 0.5;
    un = (3.0 / (x[n - 1] - x[n - 2])) * (d1_end - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]));
  }
  d2[n - 1] = (un - qn * u[n - 2]) / (qn * d2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; --k) d2[k] = d2[k] * d2[k + 1] + u[k];
}

static double spline_eval(const std::vector<double>& x, const std::vector<double>& y,
                          const std::vector<double>& d2, double xv, int& klo_hint) {
  int n = (int)x.size();
  bool inc = x[n - 1] > x[0];
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if ((x[mid] > xv) == inc) hi = mid; else lo = mid;
  }
  klo_hint = lo;
  double h = x[hi] - x[lo];
  double a = (x[hi] - xv) / h, b = (xv - x[lo]) / h;
  return a * y[lo] + b * y[hi] + ((a * a * a - a) * d2[lo] + (b * b * b - b) * d2[hi]) * (h * h) / 6.0;
}

// cumulative integral of the spline from node `first`: out[first] = 0
static void spline_integral_array(const std::vector<double>& x, const std::vector<double>& y,
                                  const std::vector<double>& d2, int first, double* out) {
  int n = (int)x.size();
  out[first] = 0;
  for (int i = first; i < n - 1; ++i) {
    double h = x[i + 1] - x[i];
    out[i + 1] = out[i] + h * (y[i] + y[i + 1]) / 2 - h * h * h * (d2[i] + d2[i + 1]) / 24;
  }
}


// ------------------------------------------------------------------------
// thermal massive-neutrino background (massive_neutrinos.f90): density and
// pressure in units of one massless eigenstate, as functions of a*m/(k_B T_nu)
// ------------------------------------------------------------------------
namespace nu {
const double zeta3 = 1.2020569031595942853997, zeta5 = 1.0369277551433699263313, zeta7 = 1.0083492773819228268397;
const double fermi_dirac_const = 7.0 / 120 * K::pi * K::pi * K::pi * K::pi;
const double const2 = 5.0 / 7.0 / (K::pi * K::pi);
const double rhop_am_min = 0.42, rhop_am_max = 70.0, am_min = 0.3, am_max = 70.0;
const double rhop_fit_c = std::sqrt(rhop_am_min * rhop_am_max);
const double rhop_fit_inv_zmax = (rhop_am_max + rhop_fit_c) / (rhop_am_max - rhop_fit_c);
const double fit_c = std::sqrt(am_min * am_max);
const double fit_inv_zmax = (am_max + fit_c) / (am_max - fit_c);
const double fit_rho_scale = 3.0 * zeta3 / (2.0 * fermi_dirac_const);
const double fit_p_denom_scale = fermi_dirac_const / ((900.0 / 120.0) * zeta5);
const double rho_c[6] = {7.499710425926954249e-01, 1.188066888581748443e-01, 1.545077526625578401e-01,
                         -8.378996019212282820e-02, 2.123075360029347963e-02, -2.544964203886362908e-03};
const double p_c[7] = {9.283417043601330798e-01, 3.156134695375645838e-01, -2.435843189264263742e-01,
                       -2.509793530357270000e-02, 4.067958090718486880e-02, 2.378742143669706002e-03,
                       -1.965863329520473827e-03};
const double low_rho_c[2] = {-1.872929199948838302e-02, 1.831728681837861694e-02};
const double low_p_c[2] = {1.667044572156534468e-02, -2.277471498716537868e-02};
const double D_c[6] = {5.800497880734221123e-01, 1.801974470841860576e-01, -1.602709049602861757e-01,
                       3.167230341650149189e-02, 1.056591590995091534e-02, -3.877662402660121861e-03};

void rho_P(double am, double& rhonu, double& pnu) {
  if (am <= rhop_am_min) {
    double am2 = am * am, am4 = am2 * am2;
    rhonu = 1.0 + const2 * am2 + am4 * (low_rho_c[0] + am2 * low_rho_c[1]);
    pnu = (1.0 - const2 * am2) / 3.0 + am4 * (low_p_c[0] + am2 * low_p_c[1]);
    return;
  } else if (am >= rhop_am_max) {
    rhonu = 3 / (2 * fermi_dirac_const) * (zeta3 * am + ((15 * zeta5) / 2 - 945.0 / 16 * zeta7 / (am * am)) / am);
    pnu = 900.0 / 120.0 / fermi_dirac_const * (zeta5 - 63.0 / 4 * zeta7 / (am * am)) / am;
    return;
  }
  double z = ((am - rhop_fit_c) / (am + rhop_fit_c)) * rhop_fit_inv_zmax;
  double rfit = (((((rho_c[5] * z + rho_c[4]) * z + rho_c[3]) * z + rho_c[2]) * z + rho_c[1]) * z + rho_c[0]);
  double pfit = ((((((p_c[6] * z + p_c[5]) * z + p_c[4]) * z + p_c[3]) * z + p_c[2]) * z + p_c[1]) * z + p_c[0]);
  rhonu = (1.0 + fit_rho_scale * am) * rfit;
  pnu = pfit / (1.0 + fit_p_denom_scale * am);
}

double rho(double am) {
  double r, p;
  rho_P(am, r, p);
  return r;
}

double drho(double am, double adotoa) {
  if (am <= am_min) {
    double am2 = am * am;
    return am2 * (2 * const2 + am2 * (.4399706676e-1 * std::log(am) - .2970400378e-2 - .29331377855e-1 * am)) * adotoa;
  } else if (am >= am_max) {
    return 3 / (2 * fermi_dirac_const) * (zeta3 * am + (-(15 * zeta5) / 2 + 2835.0 / 16 * zeta7 / (am * am)) / am) *
           adotoa;
  }
  double z = ((am - fit_c) / (am + fit_c)) * fit_inv_zmax;
  double Dfit = (((((D_c[5] * z + D_c[4]) * z + D_c[3]) * z + D_c[2]) * z + D_c[1]) * z + D_c[0]);
  return am * am / (1.0 + 2.0 * am) * Dfit * adotoa;
}
}  // namespace nu

// ------------------------------------------------------------------------
// background (results.f90:332-628, equations.f90:5-24)
// ------------------------------------------------------------------------
double Cosmology::dtauda(double a) const {
  // grho_no_de (results.f90:1393-1410) + cosmological-constant dark energy
  double grhoa2 = grhok * a * a + (grhoc + grhob) * a + grhog + grhornomass;
  for (int i = 0; i < nu_eig; ++i) grhoa2 += nu::rho(a * nu_masses[i]) * grhormass[i];
  grhoa2 += grhov * a * a * a * a;
  if (grhoa2 <= 0) return 0;
  return std::sqrt(3.0 / grhoa2);
}

// Romberg integration (MathUtils.f90:648-723)
static double romberg(const std::function<double(double)>& f, double a, double b, double tol,
                      int maxit = 25, int minsteps = 0) {
  const int MAXJ = 5;
  double g[MAXJ + 2];
  double h = 0.5 * (b - a);
  double gmax = h * (f(a) + f(b));
  g[1] = gmax;
  double g0 = gmax, err = 1e20;
  int nint_ = 1, i = 0;
  for (;;) {
    ++i;
    if (i > maxit || ((i > 5 && std::fabs(err) < tol) && nint_ > minsteps)) break;
    g0 = 0;
    for (int k = 1; k <= nint_; ++k) g0 += f(a + (k + k - 1) * h);
    g0 = 0.5 * g[1] + h * g0;
    h = 0.5 * h;
    nint_ += nint_;
    int jmax = std::min(i, MAXJ);
    double fourj = 1;
    for (int j = 1; j <= jmax; ++j) {
      fourj *= 4;
      double g1 = g0 + (g0 - g[j]) / (fourj - 1);
      g[j] = g0;
      g0 = g1;
    }
    if (std::fabs(g0) > tol) err = 1 - gmax / g0; else err = gmax;
    gmax = g0;
    g[jmax + 1] = g0;
  }
  return g0;
}

double Cosmology::delta_time(double a1, double a2, double tol) const {
  // CAMBdata_DeltaTime (results.f90:647-656)
  if (tol < 0) tol = 1e-4 / 1000 / std::exp(P.AccuracyBoost * P.IntTolBoost - 1);
  return romberg([this](double a) { return dtauda(a); }, a1, a2, tol);
}

double Cosmology::ScalarPower(double k) const {
  // TInitialPowerLaw_ScalarPower (InitialPower.f90:121-144)
  double lnrat = std::log(k / P.pivot_scalar);
  return P.As * std::exp(lnrat * (P.ns - 1 + lnrat * (P.nrun / 2)));
}

// Brent's method on [a, b] (published algorithm, R. P. Brent 1971)
static double brent_zero(const std::function<double(double)>& f, double a, double b, double fa,
                         double fb, double tol, int& iflag) {
  const double eps = 2.220446049250313e-16;
  iflag = 0;
  if (fa == 0) return a;
  if (fb == 0) return b;
  if ((fa > 0) == (fb > 0)) { iflag = -1; return a; }
  double c = a, fc = fa, d = b - a, e = d;
  for (int it = 0; it < 200; ++it) {
    if (std::fabs(fc) < std::fabs(fb)) { a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
    double tol1 = 2 * eps * std::fabs(b) + 0.5 * tol;
    double xm = 0.5 * (c - b);
    if (std::fabs(xm) <= tol1 || fb == 0) return b;
    if (std::fabs(e) >= tol1 && std::fabs(fa) > std::fabs(fb)) {
      double s = fb / fa, p, q;
      if (a != c) {
        double qq = fa / fc, r = fb / fc;
        p = s * (2 * xm * qq * (qq - r) - (b - a) * (r - 1));
        q = (qq - 1) * (r - 1) * (s - 1);
      } else {
        p = 2 * xm * s;
        q = 1 - s;
      }
      if (p > 0) q = -q; else p = -p;
      if (2 * p < std::min(3 * xm * q - std::fabs(tol1 * q), std::fabs(e * q))) { e = d; d = p / q; }
      else { d = xm; e = d; }
    } else { d = xm; e = d; }
    a = b; fa = fb;
    if (std::fabs(d) > tol1) b += d; else b += (xm > 0 ? tol1 : -tol1);
    fb = f(b);
    if ((fb > 0) == (fc > 0)) { c = a; fc = fa; d = b - a; e = d; }
  }
  iflag = -2;
  return b;
}

// ------------------------------------------------------------------------
// reionization (reionization.f90:97-360, tanh model with helium)
// ------------------------------------------------------------------------
static const double Tanh_zexp = 1.5;
void Reion::set_zre(double z) {
  redshift = z;
  WindowVarMid = std::pow(1.0 + redshift, Tanh_zexp);
  WindowVarDelta = Tanh_zexp * std::pow(1.0 + redshift, Tanh_zexp - 1.0) * delta_redshift;
}
double Reion::x_e(double z, double xstart) const {
  double xod = (WindowVarMid - std::pow(1 + z, Tanh_zexp)) / WindowVarDelta;
  double tgh = xod > 100 ? 1.0 : std::tanh(xod);
  double xe = (fraction - xstart) * (tgh + 1) / 2 + xstart;
  if (z < helium_redshiftstart) {
    double xod2 = (helium_redshift - z) / helium_delta_redshift;
    double tgh2 = xod2 > 100 ? 1.0 : std::tanh(xod2);
    xe += fHe * (tgh2 + 1) / 2;
  }
  return xe;
}

// ------------------------------------------------------------------------
// RECFAST (recfast.f90: TRecfast_init 580-839, EvaluateRecfastODE 1157-1623)
// ------------------------------------------------------------------------
namespace rf {
const double zinitial = 1e4, zfinal = 0;
const double fudge_He = 0.8472367977;
const double He_rate_zmin = 1500, He_rate_zmax = 3000;
const double He_a0 = 0.07805480599148856, He_a1 = 0.899368710079757, He_a2 = -3.063896868095767;
const double He_d2 = 3.752520187028219, He_d4 = 18.126758791787946;
const double He_z0 = 1968.1134791219417, He_width = 774.0312440582285;
const double x_He_freeze = 1e-8;
const double AGauss1 = -0.1395272483, AGauss2 = 0.0729891952;
const double zGauss1 = 7.2813061282, zGauss2 = 6.7667038679;
const double wGauss1 = 0.1638966410, wGauss2 = 0.2785834127;
const double bigH = 100.0e3 / K::Mpc;
const double not4 = K::mass_ratio_He_H;
const double Lambda = 8.2245809, Lambda_He = 51.3;
const double L_H_ion = 1.096787737e7, L_H_alpha = 8.225916453e6;
const double L_He1_ion = 1.98310772e7, L_He2_ion = 4.389088863e7;
const double L_He_2s = 1.66277434e7, L_He_2p = 1.71134891e7;
const double A2P_s = 1.798287e9, A2P_t = 177.58;
const double L_He_2Pt = 1.690871466e7, L_He_2St = 1.5985597526e7, L_He2St_ion = 3.8454693845e6;
const double sigma_He_2Ps = 1.436289e-22, sigma_He_2Pt = 1.484872e-22;
const double Lalpha = 1.0 / L_H_alpha, Lalpha_He = 1.0 / L_He_2p;
const double DeltaB = K::h_P * K::c * (L_H_ion - L_H_alpha);
const double CDB = DeltaB / K::k_B;
const double DeltaB_He = K::h_P * K::c * (L_He1_ion - L_He_2s);
const double CDB_He = DeltaB_He / K::k_B;
const double CB1 = K::h_P * K::c * L_H_ion / K::k_B;
const double CB1_He1 = K::h_P * K::c * L_He1_ion / K::k_B;
const double CB1_He2 = K::h_P * K::c * L_He2_ion / K::k_B;
const double CR = K::twopi * (K::m_e / K::h_P) * (K::k_B / K::h_P);
const double CK = Lalpha * Lalpha * Lalpha / K::eightpi;
const double CK_He = Lalpha_He * Lalpha_He * Lalpha_He / K::eightpi;
const double CL = K::c * K::h_P / (K::k_B * Lalpha);
const double CL_He = K::c * K::h_P / (K::k_B / L_He_2s);
const double a_rad = 8.0 * std::pow(K::pi, 5) * std::pow(K::k_B, 4) / 15 / std::pow(K::c, 3) / std::pow(K::h_P, 3);
const double Compton_CT = K::MPC_in_sec * (8.0 / 3.0) * (K::sigma_thomson / (K::m_e * K::c)) * a_rad;
const double CT = Compton_CT / K::MPC_in_sec;
const double Bfact = K::h_P * K::c * (L_He_2p - L_He_2s) / K::k_B;
const double H_frac = 1e-3;
}  // namespace rf

struct RecfastCtx {
  const Cosmology* c;
  const Recfast* r;
};

static void escape_prob(double tau, double& p) {
  if (std::fabs(tau) < 1e-6) p = 1 - tau / 2 + tau * tau / 6;
  else p = (1 - std::exp(-tau)) / tau;
}

// ION right-hand side in redshift: y = (x_H, x_He, a*T_mat).  full_h: the full Peebles
// hydrogen equation at every x_H (the smooth system of the Rosenbrock phase), instead of
// the Saha hold above x_H = 0.99 and the Saha-rate derivative above 0.985.
static void recfast_rhs(const RecfastCtx& ctx, double z, const double* y, double* f, bool full_h = false) {
  using namespace rf;
  const Recfast& R = *ctx.r;
  double x_H = y[0], x_He = y[1];
  bool he_corr = x_He >= x_He_freeze && x_He <= 0.98;
  double x = x_H + R.fHe * x_He;
  double ion_sum = 1.0 + x + R.fHe;
  double ainv = 1.0 + z, inv_ainv = 1.0 / ainv, ainv2 = ainv * ainv, ainv3 = ainv2 * ainv;
  double aTmat = y[2], Tmat = ainv * aTmat, inv_Tmat = 1.0 / Tmat;
  double n = R.NNow * ainv3, n_He = R.fHe * R.NNow * ainv3;
  double Trad = R.Tnow * ainv, Trad3 = Trad * Trad * Trad, Trad4 = Trad3 * Trad;
  double Hz = ainv2 / ctx.c->dtauda(inv_ainv) / K::MPC_in_sec;
  double denH = Hz * ainv;
  double cr_tmat = CR * Tmat, cr_tmat_32 = cr_tmat * std::sqrt(cr_tmat);
  const double a_PPB = 4.309, b_PPB = -0.6166, c_PPB = 0.6703, d_PPB = 0.5300;
  const double a_VF = std::pow(10.0, -16.744), b_VF = 0.711;
  const double T_0 = std::pow(10.0, 0.477121), T_1 = std::pow(10.0, 5.114);
  const double a_trip = std::pow(10.0, -16.306), b_trip = 0.761;
  double theta = Tmat * 1e-4, log_theta = std::log(theta);
  double cpd = c_PPB * std::exp(d_PPB * log_theta);
  double Rdown = 1e-19 * a_PPB * std::exp(b_PPB * log_theta) / (1.0 + cpd);
  double Rup = Rdown * cr_tmat_32 * std::exp(-CDB * inv_Tmat);
  double sq_0 = std::sqrt(Tmat / T_0), sq_1 = std::sqrt(Tmat / T_1);
  double l0 = std::log(1.0 + sq_0), l1 = std::log(1.0 + sq_1);
  double Rdown_He = a_VF / sq_0 * std::exp(-((1.0 - b_VF) * l0 + (1.0 + b_VF) * l1));
  double Rup_He = 4.0 * Rdown_He * cr_tmat_32 * std::exp(-CDB_He * inv_Tmat);
  double He_Boltz = (Bfact * inv_Tmat) > 680.0 ? std::exp(680.0) : std::exp(Bfact * inv_Tmat);
  double z_scale = R.Tnow / K::COBE_CMBTemp * ainv - 1;
  double log_1pz = std::log(1.0 + z_scale);
  double g1 = (log_1pz - zGauss1) / wGauss1, g2 = (log_1pz - zGauss2) / wGauss2;
  double Kf = CK / Hz * (1.0 + AGauss1 * std::exp(-g1 * g1) + AGauss2 * std::exp(-g2 * g2));
  double Rdown_trip = a_trip / sq_0 * std::exp(-((1.0 - b_trip) * l0 + (1.0 + b_trip) * l1));
  double Rup_trip = Rdown_trip * std::exp(-K::h_P * K::c * L_He2St_ion / K::k_B * inv_Tmat) * cr_tmat_32 * (4.0 / 3.0);
  double K_He = CK_He / Hz, CfHe_t = 0, He_rate_factor = 1;
  if (he_corr && z_scale > He_rate_zmin && z_scale < He_rate_zmax) {
    double u = (z_scale - He_z0) / He_width, u2 = u * u;
    He_rate_factor = 1.0 + (He_a0 + He_a1 * u + He_a2 * u2) / (1.0 + He_d2 * u2 + He_d4 * u2 * u2);
  }
  if (he_corr) {
    double tauHe_s = A2P_s * CK_He * 3.0 * n_He * (1.0 - x_He) / Hz, pHe_s;
    escape_prob(tauHe_s, pHe_s);
    K_He = 1.0 / (A2P_s * pHe_s * 3.0 * n_He * (1.0 - x_He));
    if (x_H < 0.9999999) {
      double Doppler = 2.0 * K::k_B * Tmat / (K::m_H * not4 * K::c * K::c);
      Doppler = K::c * L_He_2p * std::sqrt(Doppler);
      double gamma_2Ps = 3.0 * A2P_s * R.fHe * (1.0 - x_He) * K::c * K::c;
      gamma_2Ps = gamma_2Ps / (std::sqrt(K::pi) * sigma_He_2Ps * K::eightpi * Doppler * (1.0 - x_H));
      gamma_2Ps = gamma_2Ps / ((K::c * L_He_2p) * (K::c * L_He_2p));
      double pgq_s = 0.36 * std::pow(gamma_2Ps, fudge_He);
      double AHcon = A2P_s / (1.0 + pgq_s);
      K_He = 1.0 / ((A2P_s * pHe_s + AHcon) * 3.0 * n_He * (1.0 - x_He));
    }
    double tauHe_t = A2P_t * n_He * (1.0 - x_He) * 3.0;
    tauHe_t = tauHe_t / (K::eightpi * Hz * L_He_2Pt * L_He_2Pt * L_He_2Pt);
    double pHe_t;
    escape_prob(tauHe_t, pHe_t);
    double CL_PSt = K::h_P * K::c * (L_He_2Pt - L_He_2St) / K::k_B;
    double EPSt = std::exp(-CL_PSt * inv_Tmat);
    if (x_H > 0.99999) {
      CfHe_t = A2P_t * pHe_t * EPSt;
      CfHe_t = CfHe_t / (Rup_trip + CfHe_t);
    } else {
      double Doppler = 2.0 * K::k_B * Tmat / (K::m_H * not4 * K::c * K::c);
      Doppler = K::c * L_He_2Pt * std::sqrt(Doppler);
      double gamma_2Pt = 3.0 * A2P_t * R.fHe * (1.0 - x_He) * K::c * K::c;
      gamma_2Pt = gamma_2Pt / (std::sqrt(K::pi) * sigma_He_2Pt * K::eightpi * Doppler * (1.0 - x_H));
      gamma_2Pt = gamma_2Pt / ((K::c * L_He_2Pt) * (K::c * L_He_2Pt));
      double pgq_t = 0.66 * std::pow(gamma_2Pt, 0.9);
      double AHcon_t = A2P_t / (1.0 + pgq_t) / 3.0;
      CfHe_t = (A2P_t * pHe_t + AHcon_t) * EPSt;
      CfHe_t = CfHe_t / (Rup_trip + CfHe_t);
    }
  }
  double timeTh = (1.0 / (CT * Trad4)) * ion_sum / x;
  double timeH = 2.0 / (3.0 * R.HO * ainv * std::sqrt(ainv));
  double RupE = Rup * std::exp(-CL * inv_Tmat);
  double A_H = x * x_H * n * Rdown - RupE * (1.0 - x_H);
  if (!full_h && x_H > 0.99) f[0] = 0;
  else if (!full_h && x_H > 0.985) f[0] = A_H / denH;
  else {
    double B_H = 1.0 + Kf * Lambda * n * (1.0 - x_H);
    double C_H = 1.0 / R.fu + Kf * Lambda * n * (1.0 - x_H) / R.fu + Kf * Rup * n * (1.0 - x_H);
    f[0] = A_H * B_H / (denH * C_H);
  }
  if (x_He < x_He_freeze) f[1] = 0;
  else {
    double EHe = std::exp(-CL_He * inv_Tmat);
    double RupHeE = Rup_He * EHe;
    double A_He = x * x_He * n * Rdown_He - RupHeE * (1.0 - x_He);
    double LHe = Lambda_He * n_He * (1.0 - x_He) * He_Boltz;
    double MHe = (Lambda_He + Rup_He) * n_He * (1.0 - x_He) * He_Boltz;
    double BHe = 1.0 + K_He * LHe, CHe = 1.0 + K_He * MHe;
    f[1] = A_He * BHe / (denH * CHe);
    if (he_corr) {
      double ETrip = std::exp(-K::h_P * K::c * L_He_2St / K::k_B * inv_Tmat);
      double RupTripE = 3.0 * Rup_trip * ETrip;
      double A_trip = x * x_He * n * Rdown_trip - (1.0 - x_He) * RupTripE;
      f[1] += A_trip * CfHe_t / denH;
    }
    f[1] *= He_rate_factor;
  }
  if (timeTh < H_frac * timeH) {
    double dHdz = (R.HO * R.HO / 2.0 / Hz) *
                  (4.0 * ainv3 / (1.0 + R.z_eq) * R.OmegaT + 3.0 * R.OmegaT * ainv2 + 2.0 * R.OmegaK * ainv);
    double eps_tc = Hz * ion_sum / (CT * Trad3 * x);
    f[2] = (R.Tnow - aTmat) * inv_ainv +
           eps_tc * ((1.0 + R.fHe) / ion_sum) * ((f[0] + R.fHe * f[1]) / x) * inv_ainv - eps_tc * dHdz / denH +
           3.0 * eps_tc / ainv2;
  } else {
    f[2] = (CT * Trad4 * x * (aTmat - R.Tnow) / (Hz * ion_sum) + aTmat) * inv_ainv;
  }
}

// Dormand-Prince 5(4) with the step control of RungeKuttaDP45.f90:94-408
// (mixed error norm, FSAL reuse across calls), for the small RECFAST system.
struct DP45Host {
  double h = 0, err = 0, hmax = 20, tol = 1e-4;
  int fails = 0;
  bool fsal_valid = false, first = true;
  double k[7][4];
};

template <class F>
static int dp45_host(F&& fcn, int n, double& x, double* y, double xend, DP45Host& s) {
  static const double a21 = 1.0 / 5, a31 = 3.0 / 40, a32 = 9.0 / 40, a41 = 44.0 / 45, a42 = -56.0 / 15,
                      a43 = 32.0 / 9, a51 = 19372.0 / 6561, a52 = -25360.0 / 2187, a53 = 64448.0 / 6561,
                      a54 = -212.0 / 729, a61 = 9017.0 / 3168, a62 = -355.0 / 33, a63 = 46732.0 / 5247,
                      a64 = 49.0 / 176, a65 = -5103.0 / 18656, b1 = 35.0 / 384, b3 = 500.0 / 1113,
                      b4 = 125.0 / 192, b5 = -2187.0 / 6784, b6 = 11.0 / 84, e1 = 71.0 / 57600,
                      e3 = -71.0 / 16695, e4 = 71.0 / 1920, e5 = -17253.0 / 339200, e6 = 22.0 / 525,
                      e7 = -1.0 / 40;
  const double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
  double w9[4], yt[4];
  bool need_f = !s.fsal_valid;
  s.fsal_valid = false;
  for (int iter = 0; iter < 1000000; ++iter) {
    if (need_f) fcn(x, y, s.k[0]);
    need_f = false;
    double ny = 0;
    for (int i = 0; i < n; ++i) ny = std::max(ny, std::fabs(y[i]));
    ny = std::min(ny, 1.0);
    double hmin = 10.0 * std::max(tiny, eps * std::max(ny / s.tol, std::fabs(x)));
    if (hmin > s.hmax) return -2;
    if (s.first) { s.h = s.hmax * std::pow(s.tol, 0.2); s.first = false; }
    else if (s.fails <= 1) {
      double t = 2.0 * s.h;
      if (s.tol < std::pow(2.0 / 0.9, 5) * s.err) t = 0.9 * std::pow(s.tol / s.err, 0.2) * s.h;
      s.h = std::max(t, 0.5 * s.h);
    } else s.h = 0.5 * s.h;
    s.h = std::min(s.h, s.hmax);
    s.h = std::max(s.h, hmin);
    double temp = std::fabs(xend - x), xt;
    if (s.h < temp && (temp > 1.2 * s.h || temp > s.hmax)) {
      s.h = std::min(s.h, 0.5 * temp);
      xt = x + std::copysign(s.h, xend - x);
    } else { s.h = temp; xt = xend; }
    double hs = xt - x;
    for (int i = 0; i < n; ++i) w9[i] = y[i] + hs * a21 * s.k[0][i];
    fcn(x + hs / 5.0, w9, s.k[1]);
    for (int i = 0; i < n; ++i) w9[i] = y[i] + hs * (a31 * s.k[0][i] + a32 * s.k[1][i]);
    fcn(x + hs * (3.0 / 10.0), w9, s.k[2]);
    for (int i = 0; i < n; ++i) w9[i] = y[i] + hs * (a41 * s.k[0][i] + a42 * s.k[1][i] + a43 * s.k[2][i]);
    fcn(x + hs * (4.0 / 5.0), w9, s.k[3]);
    for (int i = 0; i < n; ++i)
      w9[i] = y[i] + hs * (a51 * s.k[0][i] + a52 * s.k[1][i] + a53 * s.k[2][i] + a54 * s.k[3][i]);
    fcn(x + hs * (8.0 / 9.0), w9, s.k[4]);
    for (int i = 0; i < n; ++i)
      w9[i] = y[i] + hs * (a61 * s.k[0][i] + a62 * s.k[1][i] + a63 * s.k[2][i] + a64 * s.k[3][i] + a65 * s.k[4][i]);
    fcn(x + hs, w9, s.k[5]);
    for (int i = 0; i < n; ++i)
      yt[i] = y[i] + hs * (b1 * s.k[0][i] + b3 * s.k[2][i] + b4 * s.k[3][i] + b5 * s.k[4][i] + b6 * s.k[5][i]);
    fcn(x + hs, yt, s.k[6]);
    double m = 0;
    for (int i = 0; i < n; ++i) {
      double e = e1 * s.k[0][i] + e3 * s.k[2][i] + e4 * s.k[3][i] + e5 * s.k[4][i] + e6 * s.k[5][i] + e7 * s.k[6][i];
      m = std::max(m, std::fabs(e) / std::max(1.0, std::fabs(y[i])));
    }
    s.err = m * s.h;
    if (s.err <= s.tol) {
      x = xt;
      for (int i = 0; i < n; ++i) { y[i] = yt[i]; s.k[0][i] = s.k[6][i]; }
      s.fails = 0;
      if (x == xend) { s.fsal_valid = true; return 3; }
    } else {
      s.fails++;
      if (s.h <= hmin) return -3;
    }
  }
  return -1;
}

// The stiff early phase of hydrogen recombination (TRecfast_init with use_rosenbrock,
// recfast.f90:739-760): from the end of the helium Saha phase until x_H falls to 0.976 the
// full smooth H/He/T_m system is integrated with ROS2, the two-stage L-stable Rosenbrock
// method of Verwer, Spee, Blom and Hundsdorfer (1999; gamma = 1 + 1/sqrt 2), embedded
// error (k1 + k2)/(2 gamma), with the step control of RecfastRosenbrockAdvance
// (:1072-1155) and RecfastROS2Step (:1031-1070).  The Jacobian is formed by central
// differences of the right-hand side (the reference differentiates it analytically).
namespace ros2 {
const double gamma = 1.0 + 1.0 / std::sqrt(2.0);
const double a21 = 1.0 / gamma, c21 = -2.0 / gamma, m1 = 3.0 / (2.0 * gamma), m2 = 1.0 / (2.0 * gamma);
const double safety = 0.9, min_scale = 0.2, max_scale = 2.5;
const double ion_scale_floor = 1e-3;  // ionization fractions on a smaller absolute scale than a*T_m
const double tol = 3e-4, handoff_xH = 0.976;
const int max_steps = 4096;

// LU with partial pivoting of a 3x3 matrix, in place; false when singular
bool lu3(double a[3][3], int piv[3]) {
  for (int k = 0; k < 3; ++k) {
    int p = k;
    for (int i = k + 1; i < 3; ++i)
      if (std::fabs(a[i][k]) > std::fabs(a[p][k])) p = i;
    piv[k] = p;
    if (!(std::fabs(a[p][k]) > 0) || !std::isfinite(a[p][k])) return false;
    if (p != k)
      for (int j = 0; j < 3; ++j) std::swap(a[k][j], a[p][j]);
    for (int i = k + 1; i < 3; ++i) {
      a[i][k] /= a[k][k];
      for (int j = k + 1; j < 3; ++j) a[i][j] -= a[i][k] * a[k][j];
    }
  }
  return true;
}

void lu3_solve(const double a[3][3], const int piv[3], const double* b, double* x) {
  double y[3] = {b[0], b[1], b[2]};
  for (int k = 0; k < 3; ++k) {
    std::swap(y[k], y[piv[k]]);
    for (int i = k + 1; i < 3; ++i) y[i] -= a[i][k] * y[k];
  }
  for (int k = 2; k >= 0; --k) {
    double t = y[k];
    for (int j = k + 1; j < 3; ++j) t -= a[k][j] * x[j];
    x[k] = t / a[k][k];
  }
}

bool state_ok(const double* y) {
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(y[i])) return false;
  return std::min(y[0], y[1]) >= -1e-8 && y[2] > 0;
}

// f, the Jacobian d f / d y and the one-sided z derivative f_t of the full system at (z, y)
void derivs(const RecfastCtx& ctx, double z, const double* y, double h, double* f, double J[3][3], double* f_t) {
  recfast_rhs(ctx, z, y, f, true);
  for (int j = 0; j < 3; ++j) {
    const double d = 1e-7 * std::max(std::fabs(y[j]), j < 2 ? 1e-6 : 1.0);
    double yp[3] = {y[0], y[1], y[2]}, ym[3] = {y[0], y[1], y[2]}, fp[3], fm[3];
    yp[j] += d;
    ym[j] -= d;
    recfast_rhs(ctx, z, yp, fp, true);
    recfast_rhs(ctx, z, ym, fm, true);
    for (int i = 0; i < 3; ++i) J[i][j] = (fp[i] - fm[i]) / (2 * d);
  }
  // EvaluateRecfastODETimeDerivative (recfast.f90:1002-1029)
  double dz = std::min(0.05, std::max(1e-4, 1e-5 * std::max(1.0, std::fabs(z))));
  if (std::fabs(h) > 0) dz = std::max(std::min(dz, 0.5 * std::fabs(h)), 1e-8 * std::max(1.0, std::fabs(z)));
  double zp = std::max(rf::zfinal, std::min(rf::zinitial, z + std::copysign(dz, h)));
  if (zp == z) zp = std::max(rf::zfinal, std::min(rf::zinitial, z - std::copysign(dz, h)));
  if (zp != z) {
    double fz[3];
    recfast_rhs(ctx, zp, y, fz, true);
    for (int i = 0; i < 3; ++i) f_t[i] = (fz[i] - f[i]) / (zp - z);
  } else {
    f_t[0] = f_t[1] = f_t[2] = 0;
  }
}

bool step(const RecfastCtx& ctx, double z, const double* y, double h, const double* f, const double* f_t,
          const double J[3][3], double* yout, double* yerr) {
  double m[3][3];
  int piv[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m[i][j] = (i == j ? 1.0 : 0.0) - gamma * h * J[i][j];
  if (!lu3(m, piv)) return false;
  const double gh = gamma * h, gh2 = gh * gh;
  double rhs[3], k1[3], k2[3], ys[3], fs[3];
  for (int i = 0; i < 3; ++i) rhs[i] = gh * f[i] + gh2 * f_t[i];
  lu3_solve(m, piv, rhs, k1);
  for (int i = 0; i < 3; ++i) ys[i] = y[i] + a21 * k1[i];
  recfast_rhs(ctx, z + h, ys, fs, true);
  for (int i = 0; i < 3; ++i) rhs[i] = gh * fs[i] + gamma * c21 * k1[i] - gh2 * f_t[i];
  lu3_solve(m, piv, rhs, k2);
  for (int i = 0; i < 3; ++i) {
    yout[i] = y[i] + m1 * k1[i] + m2 * k2[i];
    yerr[i] = (k1[i] + k2[i]) / (2 * gamma);
    if (!std::isfinite(yerr[i])) return false;
  }
  return state_ok(yout);
}

bool advance(const RecfastCtx& ctx, double zstart, double* y, double zend, double tol) {
  if (zend == zstart) return true;
  const double dir = zend > zstart ? 1.0 : -1.0;
  double z = zstart, h = zend - zstart;
  const double min_step = std::max(std::fabs(h) * 1e-8, 1e-10);
  double f[3], f_t[3], J[3][3];
  bool need = true;
  for (int attempt = 0; attempt < max_steps; ++attempt) {
    if (dir * (zend - z) <= 0) return true;
    if (dir * (zend - (z + h)) < 0) h = zend - z;
    if (need) {  // f, J and f_t depend on (z, y) only: reused across retries
      derivs(ctx, z, y, h, f, J, f_t);
      need = false;
    }
    double yt[3], ye[3], err = 0;
    bool ok = step(ctx, z, y, h, f, f_t, J, yt, ye);
    if (ok) {
      for (int i = 0; i < 3; ++i) {
        const double sc = i < 2 ? std::max({ion_scale_floor, std::fabs(y[i]), std::fabs(yt[i])})
                                : std::max({1.0, std::fabs(y[i]), std::fabs(yt[i])});
        err = std::max(err, std::fabs(ye[i]) / sc);
      }
      if (!std::isfinite(err)) ok = false;
    }
    if (ok && err <= tol) {
      for (int i = 0; i < 3; ++i) y[i] = yt[i];
      y[0] = std::max(y[0], 0.0);
      y[1] = std::max(y[1], 0.0);
      z += h;
      need = true;
      if (dir * (zend - z) <= 0) return true;
      double fac = err == 0 ? max_scale : std::min(max_scale, std::max(min_scale, safety * std::sqrt(tol / err)));
      h = dir * std::min(std::fabs(h) * fac, std::fabs(zend - z));
    } else {
      double fac = ok ? std::min(0.9, std::max(min_scale, safety * std::sqrt(tol / std::max(err, 1e-300))))
                      : min_scale;
      h *= fac;
      if (std::fabs(h) < min_step) return false;
    }
  }
  return false;
}
}  // namespace ros2

static void regular_spline_horner(const std::vector<double>& y, const std::vector<double>& d2, double h,
                                  std::vector<double>& hc) {
  int n = (int)y.size();
  hc.assign(4 * (n - 1), 0.0);
  double h2 = h * h;
  for (int i = 0; i < n - 1; ++i) {
    hc[4 * i + 0] = y[i];
    hc[4 * i + 1] = y[i + 1] - y[i] - h2 / 6 * (2 * d2[i] + d2[i + 1]);
    hc[4 * i + 2] = h2 / 2 * d2[i];
    hc[4 * i + 3] = h2 / 6 * (d2[i + 1] - d2[i]);
  }
}

double Recfast::x_e(double a) const {
  double z = 1 / a - 1;
  if (z >= maxz) return xrec[0];
  if (z <= minz) return xrec[nz - 1];
  double zst = (rf::zinitial - z) / delta_z;
  int ihi = (int)zst;
  double az = zst - ihi;
  const double* c = &xh[4 * (ihi - 1)];
  return c[0] + az * (c[1] + az * (c[2] + az * c[3]));
}

void Recfast::xe_Tm(double a, double& xe, double& Tm) const {
  double z = 1 / a - 1;
  if (z >= maxz) { xe = xrec[0]; Tm = Tnow / a; return; }
  if (z <= minz) { xe = xrec[nz - 1]; Tm = (1 + rf::zfinal) * tmrec[nz - 1]; return; }
  double zst = (rf::zinitial - z) / delta_z;
  int ihi = (int)zst;
  double az = zst - ihi;
  const double* c = &xh[4 * (ihi - 1)];
  xe = c[0] + az * (c[1] + az * (c[2] + az * c[3]));
  const double* t = &th[4 * (ihi - 1)];
  Tm = (1 + z) * (t[0] + az * (t[1] + az * (t[2] + az * t[3])));
}

static int recfast_init(Cosmology& c, std::string& err) {
  using namespace rf;
  Recfast& R = c.recfast;
  const CambGpuParams& P = c.P;
  R.nz = std::max(2, nint(2046 * std::max(P.BackgroundTimeStepBoost, 1e-12)));
  R.delta_z = (zinitial - zfinal) / R.nz;
  R.minz = zfinal + 1e-12 * R.delta_z;
  R.maxz = zinitial - R.delta_z - 1e-12 * R.delta_z;
  R.Tnow = P.TCMB;
  double H = P.H0 / 100;
  R.OmegaT = (P.omch2 + P.ombh2) / (H * H);
  R.OmegaK = P.omk;
  R.HO = H * bigH;
  double Yp = P.YHe;
  double mu_H = 1 / (1 - Yp);
  R.fHe = Yp / (not4 * (1 - Yp));
  R.NNow = 3 * bigH * bigH * P.ombh2 / (K::eightpi * K::G * mu_H * K::m_H);
  R.z_eq = c.z_eq;
  R.fu = 1.125;
  R.xrec.assign(R.nz, 0);
  R.tmrec.assign(R.nz, 0);
  RecfastCtx ctx{&c, &R};
  auto fcn = [&](double z, const double* y, double* f) { recfast_rhs(ctx, z, y, f); };
  double y[4] = {1, 1, R.Tnow, R.Tnow};
  DP45Host s;
  s.tol = 3e-6 / P.IntTolBoost;
  s.hmax = 20;
  bool handed_off = P.recfast_no_rosenbrock != 0;  // the Rosenbrock phase has handed back to Dormand-Prince
  for (int i = 1; i <= R.nz; ++i) {
    double zstart = zinitial - (i - 1) * R.delta_z, zend = zinitial - i * R.delta_z;
    double z = zend, ainv = 1 + z, x0;
    double z_scale = R.Tnow / K::COBE_CMBTemp * ainv - 1;
    if (!handed_off && y[0] <= ros2::handoff_xH) handed_off = true;
    if (z_scale > 8000) {
      x0 = 1 + 2 * R.fHe;
      y[0] = 1; y[1] = 1; y[2] = R.Tnow;
    } else if (z_scale > 5000) {
      double rhs = std::exp(1.5 * std::log(CR * R.Tnow / ainv) - CB1_He2 / (R.Tnow * ainv)) / R.NNow;
      x0 = 0.5 * (std::sqrt((rhs - 1 - R.fHe) * (rhs - 1 - R.fHe) + 4 * (1 + 2 * R.fHe) * rhs) - (rhs - 1 - R.fHe));
      y[0] = 1; y[1] = 1; y[2] = R.Tnow;
    } else if (z_scale > 3500) {
      x0 = 1 + R.fHe;
      y[0] = 1; y[1] = 1; y[2] = R.Tnow;
    } else if (y[1] > 0.99) {
      double rhs = std::exp(1.5 * std::log(CR * R.Tnow / ainv) - CB1_He1 / (R.Tnow * ainv)) / R.NNow * 4;
      double xHe0 = 0.5 * (std::sqrt((rhs - 1) * (rhs - 1) + 4 * (1 + R.fHe) * rhs) - (rhs - 1));
      x0 = xHe0;
      y[0] = 1; y[1] = (x0 - 1) / R.fHe; y[2] = R.Tnow;
    } else if (!handed_off) {
      double ys[3] = {y[0], y[1], y[2]};
      if (!ros2::advance(ctx, zstart, y, zend, ros2::tol / P.IntTolBoost)) {
        err = "RECFAST Rosenbrock integration failed";
        return CAMBGPU_ERROR_RECOMBINATION;
      }
      if (y[0] <= ros2::handoff_xH) {
        // hand off at the interval's start: redo the crossing interval with Dormand-Prince
        y[0] = ys[0]; y[1] = ys[1]; y[2] = ys[2];
        handed_off = true;
        double zz = zstart;
        if (y[0] > 0.99) {
          double rhs = std::exp(1.5 * std::log(CR * R.Tnow / ainv) - CB1 / (R.Tnow * ainv)) / R.NNow;
          double xH0 = 0.5 * (std::sqrt(rhs * rhs + 4 * rhs) - rhs);
          int ind = dp45_host(fcn, 3, zz, y, zend, s);
          if (ind < 0) { err = "RECFAST integration failed"; return CAMBGPU_ERROR_RECOMBINATION; }
          y[0] = xH0;
          x0 = y[0] + R.fHe * y[1];
          s.fsal_valid = false;
        } else {
          int ind = dp45_host(fcn, 3, zz, y, zend, s);
          if (ind < 0) { err = "RECFAST integration failed"; return CAMBGPU_ERROR_RECOMBINATION; }
          x0 = y[0] + R.fHe * y[1];
        }
      } else {
        x0 = y[0] + R.fHe * y[1];
      }
    } else if (y[0] > 0.99) {
      double rhs = std::exp(1.5 * std::log(CR * R.Tnow / ainv) - CB1 / (R.Tnow * ainv)) / R.NNow;
      double xH0 = 0.5 * (std::sqrt(rhs * rhs + 4 * rhs) - rhs);
      s.fsal_valid = false;
      double zz = zstart;
      int ind = dp45_host(fcn, 3, zz, y, zend, s);
      if (ind < 0) { err = "RECFAST integration failed"; return CAMBGPU_ERROR_RECOMBINATION; }
      y[0] = xH0;
      x0 = y[0] + R.fHe * y[1];
      s.fsal_valid = false;
    } else {
      double zz = zstart;
      int ind = dp45_host(fcn, 3, zz, y, zend, s);
      if (ind < 0) { err = "RECFAST integration failed"; return CAMBGPU_ERROR_RECOMBINATION; }
      x0 = y[0] + R.fHe * y[1];
    }
    R.xrec[i - 1] = x0;
    R.tmrec[i - 1] = y[2];
  }
  // splines on the regular grid in z (node i at z = zinitial - i*delta_z)
  std::vector<double> zz(R.nz), d2x(R.nz), d2t(R.nz);
  for (int i = 0; i < R.nz; ++i) zz[i] = zinitial - (i + 1) * R.delta_z;
  spline_second_derivs(zz.data(), R.xrec.data(), R.nz, d2x.data());
  spline_second_derivs(zz.data(), R.tmrec.data(), R.nz, d2t.data(), false, 0, true,
                       R.tmrec[R.nz - 1] / (1 + zfinal));
  regular_spline_horner(R.xrec, d2x, R.delta_z, R.xh);
  regular_spline_horner(R.tmrec, d2t, R.delta_z, R.th);
  return 0;
}

// ------------------------------------------------------------------------
// thermal history tables (results.f90:1924-2656)
// ------------------------------------------------------------------------
static void pade_derivative(const std::vector<double>& y, std::vector<double>& dy, const std::vector<double>& g) {
  // unit_grid_pade_derivative (results.f90:2620-2642)
  int n = (int)y.size();
  std::vector<double> f(n);
  dy.assign(n, 0);
  f[0] = (-10.0 * y[0] + 15.0 * y[1] - 6.0 * y[2] + y[3]) / 6.0;
  f[n - 1] = (10.0 * y[n - 1] - 15.0 * y[n - 2] + 6.0 * y[n - 3] - y[n - 4]) / 6.0;
  for (int i = 1; i < n - 1; ++i) f[i] = g[i] * (3.0 * (y[i + 1] - y[i - 1]) - f[i - 1]);
  dy[n - 1] = f[n - 1];
  for (int i = n - 2; i >= 0; --i) dy[i] = f[i] - g[i] * dy[i + 1];
}

static double get_tau_start(const Cosmology& c, double q) {
  // GetTauStart (cmbmain.f90:706-729)
  double t = std::min(0.001 / q, 0.1);
  double mmax = 0;
  for (int i = 0; i < c.nu_eig; ++i) mmax = std::max(mmax, c.nu_masses[i]);
  if (c.nu_eig > 0 && mmax != 0) t = std::min(t, 1e-3 / mmax / c.adotrad);
  return t;
}

// MassiveNuTransferSwitchBoost / MassiveNuTransferLAccuracyBoost (equations.f90:484-510)
// high-precision matter transfer functions requested (Transfer%high_precision with WantTransfer)
static bool transfer_hp(const CambGpuParams& P) { return P.want_transfer && P.transfer_high_precision; }
static double nu_switch_boost(const Cosmology& c, double nu_mass) {
  double b = c.P.AccuracyBoost * c.P.TimeSwitchBoost;
  // AccuracyTarget > 0 and (high-precision transfers or WantCls)
  if (nu_mass > 600 && (transfer_hp(c.P) || c.P.want_cls)) b *= 2;
  return b;
}
static double nu_l_boost(const Cosmology& c, double nu_mass, double q, double tau_nonrel_phys) {
  double b = c.P.lAccuracyBoost;
  if (nu_mass > 600 && q * tau_nonrel_phys < 500) b *= transfer_hp(c.P) ? 2.15 : 2.0;
  return b;
}

static int thermo_init(Cosmology& c, double taumin, std::string& err) {
  const CambGpuParams& P = c.P;
  double background_boost = P.BackgroundTimeStepBoost * P.AccuracyBoost;
  int nthermo = nint(20000 * std::log(1.4e4 / taumin) / std::log(1.4e4 / 2e-4) * background_boost);
  c.tauminn = 0.95 * taumin;
  c.dlntau = std::log(c.tau0 / c.tauminn) / (nthermo - 1);
  c.nthermo = nthermo;
  c.dlntau_inv = 1 / c.dlntau;
  std::vector<double> g(nthermo);
  g[0] = 0;
  for (int i = 1; i < nthermo; ++i) g[i] = 1 / (4.0 - g[i - 1]);

  double grhomass = 0;
  for (int i = 0; i < c.nu_eig; ++i) grhomass += c.grhormass[i];
  double om = (c.grhob + c.grhoc) / std::sqrt(3 * (c.grhog + grhomass + c.grhornomass));
  double a0 = c.tauminn * c.adotrad * (1 + om * c.tauminn / 4);
  int ninverse = nint(background_boost * std::log(1 / a0) / std::log(1 / 2e-10) * 4000);
  int nlin = ninverse / 2;
  int nsf = ninverse + nlin;
  std::vector<double> sf(nsf), dt(nsf), times(nsf);
  double dlna = std::log(0.2 / a0) / (ninverse - 1);
  for (int i = 2; i <= ninverse - 1; ++i) sf[i] = a0 * std::exp((i - 1) * dlna);  // 0-based i -> Fortran i+1
  sf[0] = a0;
  sf[1] = a0 * std::exp(dlna / 3);
  double da_lin = 0.8 / (nlin - 2);
  for (int i = 1; i <= nlin - 2; ++i) sf[ninverse + i - 1] = 0.2 + (i - 1) * da_lin;
  sf[ninverse + nlin - 2] = 0.9 + 0.1 * sf[ninverse + nlin - 3];
  sf[ninverse + nlin - 1] = 1;
  for (int i = 0; i < nsf; ++i) dt[i] = c.dtauda(sf[i]);
  {
    std::vector<double> d2(nsf);
    spline_second_derivs(sf.data(), dt.data(), nsf, d2.data());
    spline_integral_array(sf, dt, d2, 1, times.data());
  }
  times[0] = c.tauminn;
  double t2 = 2 * (std::sqrt(1 + om * sf[1] / c.adotrad) - 1) / om;
  for (int i = 1; i < nsf; ++i) times[i] += t2;
  times[nsf - 1] = c.tau0;
  std::vector<double> d2a(nsf);
  spline_second_derivs(times.data(), sf.data(), nsf, d2a.data());

  std::vector<double> taus(nthermo), a(nthermo);
  taus[0] = c.tauminn;
  for (int i = 1; i < nthermo - 1; ++i) taus[i] = c.tauminn * std::exp(i * c.dlntau);
  taus[nthermo - 1] = c.tau0;
  int hint;
  for (int i = 1; i < nthermo; ++i) a[i] = spline_eval(times, sf, d2a, taus[i], hint);
  a[0] = a0;
  a[nthermo - 1] = 1;

  c.adot.assign(nthermo, 0);
  c.adot[0] = 1 / c.dtauda(a0);
  c.matter_verydom_tau = 0;
  double a_verydom = P.AccuracyBoost * P.TimeSwitchBoost * 5 * (c.grhog + c.grhornomass) / (c.grhoc + c.grhob);
  // reionization timesteps (TTanhReionization_get_timesteps)
  c.reion_n_steps = nint(50.0);
  double reion_z_start = c.reion.redshift + c.reion.delta_redshift * 8;
  double reion_z_complete = std::max(0.0, c.reion.redshift - c.reion.delta_redshift * 8);
  c.reion_tau_start = std::max(0.05, c.time_of_z(reion_z_start, 1e-3));
  c.reion_tau_complete = std::min(c.tau0, c.reion_tau_start + c.delta_time(1 / (1 + reion_z_start),
                                                                         1 / (1.0 + reion_z_complete), 1e-3));
  for (int i = 1; i < nthermo; ++i) {
    c.adot[i] = 1 / c.dtauda(a[i]);
    if (c.matter_verydom_tau == 0 && a[i] > a_verydom) c.matter_verydom_tau = taus[i];
  }
  c.xe.assign(nthermo, 0);
  c.tb.assign(nthermo, 0);
  c.cs2.assign(nthermo, 0);
  c.dotmu.assign(nthermo, 0);
  std::vector<double> xe_a(nthermo);
  c.recfast.xe_Tm(a0, c.xe[0], c.tb[0]);
  double barssc = K::barssc0 * (1 - 0.75 * P.YHe + (1 - P.YHe) * c.xe[0]);
  c.cs2[0] = 4.0 / 3.0 * barssc * c.tb[0];
  c.dotmu[0] = c.xe[0] * c.akthom / (a0 * a0);
  for (int i = 1; i < nthermo; ++i) c.recfast.xe_Tm(a[i], xe_a[i], c.tb[i]);
  const double thomc0 = rf::Compton_CT * std::pow(P.TCMB, 4);
  c.tight_tau = 0;
  c.actual_opt_depth = 0;
  int ncount = 0;
  double last_dotmu = 0;
  for (int i = 1; i < nthermo; ++i) {
    double tau = taus[i], ai = a[i], a2 = ai * ai, adot = c.adot[i];
    if (c.reion.on && tau > c.reion_tau_start) {
      if (ncount == 0) ncount = i;  // Fortran ncount = i-1 (1-based) -> 0-based index i-1, stored +1
      c.xe[i] = c.reion.x_e(1 / ai - 1, c.xe[ncount - 1]);
      if (P.accurate_reionization) {
        c.dotmu[i] = (xe_a[i] - c.xe[i]) * c.akthom / a2;
        if (last_dotmu != 0)
          c.actual_opt_depth -= 2.0 * (tau - taus[i - 1]) / (1.0 / c.dotmu[i] + 1.0 / last_dotmu);
        last_dotmu = c.dotmu[i];
      }
    } else c.xe[i] = xe_a[i];
    double fe = (1 - P.YHe) * xe_a[i] / (1 - 0.75 * P.YHe + (1 - P.YHe) * xe_a[i]);
    double dtbdla = -2 * c.tb[i];
    if (ai * c.tb[i] - P.TCMB < -1e-8) dtbdla -= thomc0 * fe / adot * (ai * c.tb[i] - P.TCMB) / (ai * ai * ai);
    barssc = K::barssc0 * (1 - 0.75 * P.YHe + (1 - P.YHe) * xe_a[i]);
    c.cs2[i] = barssc * c.tb[i] * (1 - dtbdla / c.tb[i] / 3);
    c.dotmu[i] = c.xe[i] * c.akthom / a2;
    if (c.tight_tau == 0 && 1 / (tau * c.dotmu[i]) > 0.005) c.tight_tau = tau;
  }
  c.dotmu_runmin.resize(nthermo);
  for (int i = 0; i < nthermo; ++i)
    c.dotmu_runmin[i] = i == 0 ? c.dotmu[0] : std::min(c.dotmu_runmin[i - 1], c.dotmu[i]);
  // optical depth integral from tau0 backwards
  std::vector<double> sdotmu(nthermo), emmu(nthermo);
  {
    std::vector<double> xr(nthermo), yr(nthermo), d2(nthermo), opts(nthermo);
    for (int i = 0; i < nthermo; ++i) { xr[i] = taus[nthermo - 1 - i]; yr[i] = c.dotmu[nthermo - 1 - i]; }
    spline_second_derivs(xr.data(), yr.data(), nthermo, d2.data());
    spline_integral_array(xr, yr, d2, 0, opts.data());
    for (int i = 0; i < nthermo; ++i) sdotmu[i] = opts[nthermo - 1 - i];
  }
  for (int j = 0; j < nthermo; ++j) emmu[j] = sdotmu[j] < -69 ? 1e-30 : std::exp(sdotmu[j]);
  double z_scale = K::COBE_CMBTemp / P.TCMB;
  double zstar_max = 2000 * z_scale;
  for (int j1 = nint(std::log(100 / c.tauminn) / c.dlntau) - 1; j1 < nthermo; ++j1) {
    if (-sdotmu[j1] - c.actual_opt_depth < 1) {
      zstar_max = 1 / a[j1 - 2] - 1;
      break;
    }
  }
  // decoupling start/end and maximum visibility
  int iv = 0, ns;
  double vfi = 0, cf1, maxvis = 0;
  if (ncount == 0) { cf1 = 1; ns = nthermo; }
  else { cf1 = std::exp(-sdotmu[ncount - 1]); ns = ncount; }
  for (int j1 = 0; j1 < ns; ++j1) {
    double vis = emmu[j1] * c.dotmu[j1], tau = taus[j1];
    vfi += vis * cf1 * c.dlntau * tau;
    if (iv == 0 && vfi > 1e-7 / P.AccuracyBoost) { c.taurst = 9.0 / 10.0 * tau; iv = 1; }
    else if (iv == 1) {
      if (vis > maxvis) { maxvis = vis; c.tau_maxvis = tau; }
      if (vfi > 0.995) { c.taurend = tau; iv = 2; break; }
    }
  }
  if (iv != 2) { err = "ThermoData Init: failed to find end of recombination"; return CAMBGPU_ERROR_REIONIZATION; }
  c.dtaurec = std::min(c.dtaurec, c.taurst / 40) / P.AccuracyBoost;
  if (c.reion.on) c.taurend = std::min(c.taurend, c.reion_tau_start);

  c.ddotmu.clear(); c.dddotmu.clear(); c.ddddotmu.clear();
  pade_derivative(c.dotmu, c.ddotmu, g);
  pade_derivative(c.ddotmu, c.dddotmu, g);
  pade_derivative(c.dddotmu, c.ddddotmu, g);
  std::vector<double> dcs2, dadot;
  pade_derivative(c.cs2, dcs2, g);
  c.emmu = emmu;
  pade_derivative(c.emmu, c.demmu, g);
  pade_derivative(c.adot, dadot, g);
  c.thermo_horner.assign((size_t)nthermo * 16, 0.0);
  std::vector<double> sfo(nthermo);
  for (int i = 0; i < nthermo; ++i) sfo[i] = a[i] / taus[i];
  double sf1 = sfo[0], dSF1 = (c.adot[0] - sf1) * c.dlntau;
  for (int j = 0; j < nthermo - 1; ++j) {
    double* h = &c.thermo_horner[(size_t)j * 16];
    h[0] = c.cs2[j];
    h[1] = dcs2[j];
    h[2] = 3 * (c.cs2[j + 1] - c.cs2[j]) - 2 * dcs2[j] - dcs2[j + 1];
    h[3] = dcs2[j] + dcs2[j + 1] + 2 * (c.cs2[j] - c.cs2[j + 1]);
    h[4] = c.dotmu[j];
    h[5] = c.ddotmu[j];
    h[6] = 3 * (c.dotmu[j + 1] - c.dotmu[j]) - 2 * c.ddotmu[j] - c.ddotmu[j + 1];
    h[7] = c.ddotmu[j] + c.ddotmu[j + 1] + 2 * (c.dotmu[j] - c.dotmu[j + 1]);
    double sf2 = sfo[j + 1], dSF2 = (c.adot[j + 1] - sf2) * c.dlntau, delta = sf2 - sf1;
    h[8] = sf1;
    h[9] = dSF1;
    h[10] = 3 * delta - 2 * dSF1 - dSF2;
    h[11] = dSF1 + dSF2 - 2 * delta;
    sf1 = sf2;
    dSF1 = dSF2;
    h[12] = c.ddotmu[j];
    h[13] = c.dddotmu[j];
    h[14] = 3 * (c.ddotmu[j + 1] - c.ddotmu[j]) - 2 * c.dddotmu[j] - c.dddotmu[j + 1];
    h[15] = c.dddotmu[j] + c.dddotmu[j + 1] + 2 * (c.ddotmu[j] - c.ddotmu[j + 1]);
  }
  // z_drag and the sound horizon there (results.f90:2489-2492), used for State%scale
  c.r_drag0 = 3.0 / 4.0 * c.grhob / c.grhog;
  auto xe_rec = [&](double z) { return c.recfast.x_e(1 / (1 + z)); };
  auto dragoptdepth = [&](double z) {
    return romberg([&](double zz) {
      double aa = 1 / (1 + zz);
      return xe_rec(zz) * c.akthom * c.dtauda(aa) / c.r_drag0 / aa;
    }, 0.0, z, 1e-5, 20, 100);
  };
  {
    double x1 = 800 * z_scale, x2 = std::max(zstar_max * 1.1, 1200 * z_scale), tol = 2e-3 / background_boost;
    double try_b = x1, try_t = x2, diff = tol * 2, last_bot = 0, last_top = 0;
    int count = 0;
    bool ok = true;
    while (diff > tol) {
      if (count > 100) { ok = false; break; }
      double avg = (try_b + try_t) / 2, D = dragoptdepth(avg);
      ++count;
      if (D < 1) { try_b = avg; last_bot = D; } else { try_t = avg; last_top = D; }
      diff = std::fabs(D - 1);
    }
    if (ok) {
      if (try_b == x1) last_bot = dragoptdepth(x1);
      if (try_t == x2) last_top = dragoptdepth(x2);
      c.z_drag = (try_t * (1 - last_bot) + try_b * (last_top - 1)) / (last_top - last_bot);
      double rs = romberg([&](double aa) {
        double Rr = 3 * c.grhob * aa / (4 * c.grhog);
        return c.dtauda(aa) / std::sqrt(3 * (1 + Rr));
      }, 1e-9, 1 / (c.z_drag + 1), 1e-6);
      const double planck2018_drag_angle = 0.010392206684501;
      c.scale = planck2018_drag_angle / (rs / c.DMt0);
    } else c.scale = 1;
  }
  return 0;
}

// ------------------------------------------------------------------------
// l sampling (results.f90:1505-1704), flat case, no log-l values
// ------------------------------------------------------------------------
static void lsamples_init(const Cosmology& c, int lmin, int max_l, std::vector<int>& out) {
  const CambGpuParams& P = c.P;
  const double near_flat_scale_tol = 0.03;
  const int lmin_log = 5000, lens_output_margin = 200, lens_convolution_gap = 50;
  std::vector<int> ls;
  double AScale = (c.scale < 1 - near_flat_scale_tol) ? c.scale / P.lSampleBoost : 1 / P.lSampleBoost;
  if (P.lSampleBoost >= 50) {
    for (int l = lmin; l <= max_l; ++l) ls.push_back(l);
    out = ls;
    return;
  }
  for (int l = lmin; l <= 10; ++l) ls.push_back(l);
  int step, bot, top;
  if (P.accurate_reionization) {
    for (int l = 11; l <= 14; ++l) ls.push_back(l);
    if (P.lSampleBoost > 1) { for (int l = 15; l <= 37; ++l) ls.push_back(l); }
    else {
      for (int l = 15; l <= 18; ++l) ls.push_back(l);
      for (int l = 19; l <= 37; l += 2) ls.push_back(l);
    }
    step = std::max(nint(5 * AScale), 2);
    bot = 40;
    top = bot + step * 10;
  } else {
    if (P.lSampleBoost > 1) { for (int l = 11; l <= 15; ++l) ls.push_back(l); }
    else { ls.push_back(12); ls.push_back(15); }
    step = std::max(nint(10 * AScale), 3);
    bot = 15 + std::max(step / 2, 2);
    top = bot + step * 7;
  }
  for (int l = bot; l <= top; l += step) ls.push_back(l);
  auto trim_to_max = [&]() {
    int lind = (int)ls.size() - 1;
    while (lind >= 0 && ls[lind] > max_l) --lind;
    ls.resize(lind + 1);
    if (ls.back() < max_l) ls.push_back(max_l);
  };
  step = std::max(nint(20 * AScale), 4);
  bot = ls.back() + step;
  top = bot + step * 2;
  for (int l = bot; l <= top; l += step) ls.push_back(l);
  if (ls.back() >= max_l) { trim_to_max(); out = ls; return; }
  step = std::max(nint(25 * AScale), 4);
  bot = ls.back() + step;
  top = bot + step;
  for (int l = bot; l <= top; l += step) ls.push_back(l);
  if (ls.back() >= max_l) { trim_to_max(); out = ls; return; }
  // use_cl_spline_template = .true. (model.f90 default) -> step 50
  step = std::max(nint(50 * AScale), 7);
  bot = ls.back() + step;
  top = std::min(lmin_log, max_l);
  for (int l = bot; l <= top; l += step) ls.push_back(l);
  if (max_l > lmin_log) {
    step = std::max(nint(100 * AScale), 50);
    double growth = 1.1;
    int l = ls.back();
    for (;;) {
      l += step;
      if (l > max_l) break;
      ls.push_back(l);
      step = nint(step * growth);
    }
    int lim = max_l - (lens_output_margin - lens_convolution_gap);
    if (ls.back() < lim) ls.push_back(lim);
    else if (ls.back() - ls[ls.size() - 2] > lens_output_margin - lens_convolution_gap) ls.back() = lim;
  }
  if (ls.back() != max_l) ls.push_back(max_l);
  out = ls;
}

// ------------------------------------------------------------------------
// per-mode setup: GetNumEqns (equations.f90:860-1070, massless neutrinos),
// GetTauStart and the tight-coupling switch of initial (equations.f90:1940-1950)
// ------------------------------------------------------------------------
static double opacity_to_time(const Cosmology& c, double opacity) {
  // Thermo_OpacityToTime (results.f90:1906-1922): the first table index j < nthermo - 1
  // with dotmu(j) <= opacity (else nthermo - 1).  The running minimum of dotmu is
  // non-increasing and first drops to <= opacity at that same index, so bisecting it
  // gives the scan's answer in O(log nthermo) per k-mode.
  int lo = 0, hi = c.nthermo - 1;
  if ((int)c.dotmu_runmin.size() != c.nthermo) {  // tables built without the running minimum
    while (lo < hi && c.dotmu[lo] > opacity) ++lo;
    return std::exp(lo * c.dlntau) * c.tauminn;
  }
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (c.dotmu_runmin[mid] <= opacity) hi = mid;
    else lo = mid + 1;
  }
  return std::exp(lo * c.dlntau) * c.tauminn;
}

static CambGpuModeSpec mode_setup(const Cosmology& c, double q, bool transfer_only = false) {
  const CambGpuParams& P = c.P;
  CambGpuModeSpec m{};
  m.q = q;
  double lab = P.lAccuracyBoost;
  int min_lmaxnr = std::max(3, nint(3 * lab));
  double max_nu_mass = 0;
  int lmaxnu = 0;
  if (c.nu_eig > 0) {
    for (int i = 0; i < c.nu_eig; ++i) max_nu_mass = std::max(max_nu_mass, c.nu_masses[i]);
    for (int i = 0; i < c.nu_eig; ++i) {
      int q_rel = 0;
      for (int j = 0; j < c.nqmax; ++j) {
        if (c.nu_q[j] > c.nu_masses[i] * c.adotrad / q) break;
        ++q_rel;
      }
      m.nq0[i] = (q_rel >= c.nqmax - 2) ? c.nqmax : q_rel;
      m.nu_l_boost[i] = nu_l_boost(c, c.nu_masses[i], q, c.nu_tau_nonrel_phys[i]);
    }
    if (transfer_hp(P)) {
      lmaxnu = nint(25 * lab);
      for (int i = 0; i < c.nu_eig; ++i) lmaxnu = std::max(lmaxnu, nint(25 * m.nu_l_boost[i]));
    } else {
      lmaxnu = std::max(3, nint(10 * lab));
      if (max_nu_mass > 700) lmaxnu = std::max(3, nint(15 * lab));
      for (int i = 0; i < c.nu_eig; ++i) {
        lmaxnu = std::max(lmaxnu, nint(10 * m.nu_l_boost[i]));
        if (c.nu_masses[i] > 700) lmaxnu = std::max(lmaxnu, nint(15 * m.nu_l_boost[i]));
      }
    }
  }
  m.lmaxnu = lmaxnu;
  int lmaxg = P.accurate_polarization ? std::max(nint(11 * lab), 3) : std::max(nint(8 * lab), 3);
  int lmaxnr = std::max(nint(14 * lab), min_lmaxnr);
  if (max_nu_mass > 700) lmaxnr = std::max(nint(32 * lab), min_lmaxnr);
  int lmaxgpol = lmaxg;
  if (!P.accurate_polarization) lmaxgpol = std::max(nint(4 * lab), 3);
  else if (P.want_cls && q > 0.15) {  // AccuracyTarget > 0 and Want_CMB
    lmaxg = std::max(lmaxg, nint(13 * lab));
    lmaxgpol = std::max(lmaxgpol, nint(14 * lab));
  }
  if (q < 0.05) {
    double scal = P.accurate_polarization ? 4 : 1;
    lmaxgpol = std::max(3, nint(std::min(8, nint(scal * 150 * q)) * lab));
    lmaxnr = std::max(min_lmaxnr, nint(std::min(8, nint(std::sqrt(scal) * 150 * q)) * lab));
    lmaxg = std::max(3, nint(std::min(8, nint(std::sqrt(scal) * 300 * q)) * lab));
    if (P.accurate_reionization) {
      lmaxg = lmaxg * 8;  // AccuracyTarget > 0
      lmaxgpol = lmaxgpol * 2;
    }
  }
  if (transfer_only) {
    lmaxgpol = std::min(lmaxgpol, nint(5 * lab));
    lmaxg = std::min(lmaxg, nint(6 * lab));
  }
  if (transfer_hp(P) && q > 0.03 && q < 0.2) {  // AccuracyTarget > 0
    lmaxg = std::max(lmaxg, nint(12 * lab));
    lmaxgpol = std::max(lmaxgpol, nint(5 * lab));
  }
  if (transfer_hp(P)) {
    // the massless-neutrino hierarchy across transfer scales (equations.f90:979-993)
    if (q >= 0.005) lmaxnr = std::max(lmaxnr, nint(4 * lab));
    if (q >= 0.010 && q < 0.05)
      lmaxnr = std::max(std::max(lmaxnr, nint((8.0 + 6.0 * (q - 0.010) / 0.040) * lab)), min_lmaxnr);
    else if (q >= 0.05 && q < 0.12)
      lmaxnr = std::max(std::max(lmaxnr, nint((14.0 + 31.0 * (q - 0.05) / 0.07) * lab)), min_lmaxnr);
    else if (q >= 0.12)
      lmaxnr = std::max(nint(45 * lab), min_lmaxnr);
    if (q > 0.04 && q < 0.5) lmaxg = std::max(lmaxg, nint(10 * lab));
  }
  if (lmaxnr < lmaxnu) lmaxnr = lmaxnu;
  m.lmaxg = lmaxg;
  m.lmaxgpol = lmaxgpol;
  m.lmaxnr = lmaxnr;
  m.taustart = get_tau_start(c, q);
  // MassiveNuApproxTime (initial, equations.f90:2091-2102)
  for (int i = 0; i < c.nu_eig; ++i) {
    double sb = nu_switch_boost(c, c.nu_masses[i]);
    m.nu_approx_time[i] = c.nu_tau_massive[i];
    double a_massive = 20000 * q / c.nu_masses[i] * sb * m.nu_l_boost[i];
    if (a_massive >= 0.99) m.nu_approx_time[i] = c.tau0 + 1;
    else if (a_massive > 17.0 / c.nu_masses[i] * sb)
      m.nu_approx_time[i] = std::max(m.nu_approx_time[i], c.delta_time(0, a_massive, 0.01));
  }
  // tight-coupling switch time
  double epsw = 100 / c.tau0, ep0 = 1e-2, ep;
  if (q > epsw) ep = (q > epsw * 5) ? ep0 * 5 / P.AccuracyBoost * 0.65 : ep0;
  else ep = ep0;
  ep = ep * 2;  // second_order_tightcoupling
  m.tight_switch_tau = std::min(c.tight_tau, opacity_to_time(c, q / ep));
  return m;
}

// ------------------------------------------------------------------------
// build everything for one cosmology
// ------------------------------------------------------------------------
int build_cosmology(const CambGpuParams& p, Cosmology& c, std::string& err) {
  c.P = p;
  const CambGpuParams& P = c.P;
  if (std::fabs(P.omk) > 5e-7) { err = "only flat models are supported"; return CAMBGPU_ERROR_UNSUPPORTED_PARAMS; }
  if (!(P.H0 > 0 && P.ombh2 > 0 && P.omch2 >= 0 && P.YHe > 0 && P.YHe < 1 && P.TCMB > 0)) {
    err = "invalid cosmological parameters";
    return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
  }
  if (P.max_l < 10 || P.max_l > 8000) { err = "max_l out of range"; return CAMBGPU_ERROR_UNSUPPORTED_PARAMS; }
  // CAMB_GetResults: P%Max_eta_k = max(min(Max_l,3000)*2.5, Max_eta_k)
  c.maximum_l = P.max_l;
  c.maximum_qeta = std::max(std::min(P.max_l, 3000) * 2.5, P.max_eta_k);
  // SetParams (results.f90:466-520)
  double c_si = K::c;
  c.grhocrit = 3 * P.H0 * P.H0 / (c_si * c_si) * 1000 * 1000;
  c.grhog = K::kappa / (c_si * c_si) * 4 * K::sigma_boltz / (c_si * c_si * c_si) * std::pow(P.TCMB, 4) * K::Mpc * K::Mpc;
  c.grhor = 7.0 / 8 * std::pow(4.0 / 11, 4.0 / 3) * c.grhog;
  // neutrinos: CAMBparams_SetNeutrinoMasses, degenerate hierarchy (model.f90:260-405), then
  // the massive-neutrino part of SetParams (results.f90:405-433, 497-525)
  double h2 = (P.H0 / 100) * (P.H0 / 100);
  double nu_massless_degeneracy = P.nnu;
  c.nu_eig = 0;
  c.omnuh2 = 0;
  if (P.mnu > 0) {
    const double default_nnu = 3.044;
    const double eV = 1.602176634e-19, hbar = K::h_P / K::twopi;
    const double kB_T = K::k_B * K::COBE_CMBTemp / hbar / K::c;
    const double inv_neutrino_mass_fac = nu::zeta3 * 3.0 / 2 / (K::pi * K::pi) * 4.0 / 11 *
                                         (kB_T * kB_T * kB_T * K::kappa / 3 /
                                          ((100 * 1000 / K::Mpc) * (100 * 1000 / K::Mpc)) / (K::c * K::c / eV));
    const double neutrino_mass_fac = 1 / inv_neutrino_mass_fac;
    int nmass = std::max(1, P.num_massive_neutrinos);
    double neff_massive_standard = nmass * default_nnu / 3;
    if (P.nnu > neff_massive_standard) nu_massless_degeneracy = P.nnu - neff_massive_standard;
    else {
      nu_massless_degeneracy = 0;
      neff_massive_standard = P.nnu;
    }
    c.nu_eig = 1;
    c.nu_degeneracy[0] = neff_massive_standard;
    double mass = P.mnu / nmass;
    double T_nu = K::k_B * P.TCMB / eV * std::pow(4.0 / 11, 1.0 / 3);
    double rhonu = nu::rho(mass / (T_nu * std::pow(neff_massive_standard / nmass, 0.25)));
    c.omnuh2 = neff_massive_standard * T_nu * std::pow(P.TCMB / K::COBE_CMBTemp, 3) * rhonu /
               (neutrino_mass_fac * nu::fit_rho_scale);
  }
  c.grhornomass = c.grhor * nu_massless_degeneracy;
  for (int i = 0; i < c.nu_eig; ++i) c.grhormass[i] = c.grhor * c.nu_degeneracy[i];
  c.grhoc = c.grhocrit * P.omch2 / h2;
  c.grhob = c.grhocrit * P.ombh2 / h2;
  c.grhok = 0;
  c.Omega_de = 1 - (P.omch2 + P.ombh2 + c.omnuh2) / h2 - P.omk - (c.grhornomass + c.grhog) / c.grhocrit;
  c.grhov = c.grhocrit * c.Omega_de;
  double grhomass = 0;
  for (int i = 0; i < c.nu_eig; ++i) grhomass += c.grhormass[i];
  c.adotrad = std::sqrt((c.grhog + c.grhornomass + grhomass) / 3);
  if (c.nu_eig > 0) {
    // nu_masses = m c^2/(k_B T_nu0) from the density (find_nu_mass_for_rho, massive_neutrinos.f90:271-322)
    for (int i = 0; i < c.nu_eig; ++i) {
      double rho = c.omnuh2 / h2 * 1.0 * c.grhocrit / c.grhormass[i];
      double m;
      if (rho <= 1) m = 0;
      else if (rho <= 1.005) {
        double delta = rho - 1;
        double y = delta / nu::const2 - nu::low_rho_c[0] * delta * delta / (nu::const2 * nu::const2 * nu::const2);
        m = std::sqrt(std::max(0.0, y));
      } else {
        m = nu::fermi_dirac_const / (1.5 * nu::zeta3) * rho;
        if (m > 4) {
          double B = 15.0 * nu::zeta5 / (2.0 * nu::zeta3);
          m = m - B / m;
          double rn = nu::rho(m), rnd = nu::drho(m, 1.0);
          m = m - m * (rn - rho) / rnd;
        } else {
          int iflag = 0;
          double fa = nu::rho(0.0) - rho, fb = nu::rho(m) - rho;
          m = brent_zero([&](double x) { return nu::rho(x) - rho; }, 0.0, m, fa, fb, 0.01, iflag);
          if (iflag) { err = "find_nu_mass_for_rho failed"; return CAMBGPU_ERROR_UNSUPPORTED_PARAMS; }
        }
      }
      c.nu_masses[i] = std::max(m, 1e-3);
    }
    // TNuPerturbations_init (massive_neutrinos.f90:122-171)
    double acc = P.AccuracyBoost;
    double max_nu_mass = c.nu_masses[0];
    if (max_nu_mass > 4300) acc = std::max(acc, 2.001);
    else if (max_nu_mass > 600) acc = std::max(acc, 1.001);
    if (acc > 3) c.nqmax = nint(acc * 10);
    else if (acc > 2) c.nqmax = 5;
    else if (acc > 1) c.nqmax = 4;
    else c.nqmax = 3;
    if (c.nqmax == 3) {
      c.nu_q = {0.913201, 3.37517, 7.79184};
      c.nu_int_kernel = {0.0687359, 3.31435, 2.29911};
    } else if (c.nqmax == 4) {
      c.nu_q = {0.5802007037903776, 2.2150938570691223, 4.948032138986023, 9.65253759848097};
      c.nu_int_kernel = {0.0082119845039711, 1.1143258498419168, 3.6819104154615907, 0.8777790167504481};
    } else if (c.nqmax == 5) {
      c.nu_q = {0.4620995950854295, 1.7331898360630928, 3.7956972681313816, 7.2113928588584990,
                13.2665914595911080};
      c.nu_int_kernel = {0.0026946402277849193, 0.46041071394952310, 2.9207114780286405, 2.1821643017186352,
                         0.11621584305889110};
    } else {
      c.nu_q.assign(c.nqmax, 0);
      c.nu_int_kernel.assign(c.nqmax, 0);
      double dq = (12 + c.nqmax / 5) / (double)c.nqmax;
      for (int i = 0; i < c.nqmax; ++i) {
        double qq = (i + 0.5) * dq, dlfdlq = -qq / (1.0 + std::exp(-qq));
        c.nu_q[i] = qq;
        c.nu_int_kernel[i] = dq * qq * qq * qq / (std::exp(qq) + 1.0) * (-0.25 * dlfdlq);
      }
    }
    for (auto& w : c.nu_int_kernel) w /= nu::fermi_dirac_const;
  }
  c.Nnow = P.ombh2 / h2 * (1 - P.YHe) * c.grhocrit * c_si * c_si / K::kappa / K::m_H / (K::Mpc * K::Mpc);
  c.akthom = K::sigma_thomson * c.Nnow * K::Mpc;
  c.fHe = P.YHe / (K::mass_ratio_He_H * (1 - P.YHe));
  c.z_eq = (c.grhob + c.grhoc) / (c.grhog + c.grhornomass + grhomass) - 1;
  c.tau0 = c.time_of_z(0);
  c.DMt0 = c.tau0;
  // GaugeInterface_Init (equations.f90:512-583): times at which the momentum bins and the
  // eigenstates become non-relativistic
  if (c.nu_eig > 0) {
    auto dtm = [&](double a1, double a2, double tol) {  // DeltaTimeMaxed
      if (a1 > 1) return 0.0;
      if (a2 > 1) return c.delta_time(a1, 1.01, tol);
      return c.delta_time(a1, a2, tol);
    };
    c.nu_tau_notmassless.assign((size_t)c.nu_eig * c.nqmax, 0.0);
    for (int i = 0; i < c.nu_eig; ++i) {
      double nu_mass = std::max(0.1, c.nu_masses[i]);
      double a_mass = 1e-1 / nu_mass / P.lAccuracyBoost;
      double time = c.delta_time(0, c.nu_q[0] * a_mass);
      c.nu_tau_notmassless[(size_t)i * c.nqmax] = time;
      for (int j = 1; j < c.nqmax; ++j) {
        time += dtm(c.nu_q[j - 1] * a_mass, c.nu_q[j] * a_mass, 0.01);
        c.nu_tau_notmassless[(size_t)i * c.nqmax + j] = time;
      }
      double a_nonrel = 2.5 / nu_mass;
      c.nu_tau_nonrel_phys[i] = dtm(0, a_nonrel, -1);
      a_nonrel = a_nonrel * nu_switch_boost(c, nu_mass);
      c.nu_tau_nonrel[i] = dtm(0, a_nonrel, -1);
      double a_massive = 17.0 / nu_mass * nu_switch_boost(c, nu_mass);
      c.nu_tau_massive[i] = c.nu_tau_nonrel[i] + dtm(a_nonrel, a_massive, -1);
    }
  }
  // reionization (TBaseTauWithHeReionization_Init, zreFromOptDepth)
  Reion& R = c.reion;
  R.fHe = c.fHe;
  R.delta_redshift = P.reion_delta_redshift;
  R.on = P.reion_use_optical_depth ? P.optical_depth >= 0.001 : P.reion_redshift > 0;
  if (R.on && !P.reion_use_optical_depth) {
    R.fraction = 1 + c.fHe;
    R.set_zre(P.reion_redshift);
  } else if (R.on) {
    R.fraction = 1 + c.fHe;
    auto reion_tau = [&](double zre) {
      R.set_zre(zre);
      double zstart = zre + R.delta_redshift * 8;
      return romberg([&](double z) { return R.x_e(z) * c.akthom * c.dtauda(1 / (1 + z)); }, 0.0, zstart,
                     1e-5 / P.AccuracyBoost) - P.optical_depth;
    };
    double zb = 0, zt = 50;
    double fb = reion_tau(zb), ft = reion_tau(zt);
    int iflag = 0;
    double z = brent_zero(reion_tau, zb, zt, fb, ft, 1e-3, iflag);
    if (iflag != 0) { err = "reionization did not converge to optical depth"; return CAMBGPU_ERROR_REIONIZATION; }
    R.set_zre(z);
  }
  // InitVars (cmbmain.f90:785-862)
  double initAccuracyBoost = P.AccuracyBoost * P.TimeStepBoost;
  c.qmax = c.maximum_qeta / c.tau0;
  c.qmin = 0.1 / c.tau0 / initAccuracyBoost;
  c.dtaurec = 4 / c.qmax / initAccuracyBoost;
  c.max_etak_scalar = initAccuracyBoost * std::max(1700.0, c.maximum_qeta) / 20;
  if (c.maximum_qeta < 3500 && P.AccuracyBoost < 2) c.max_etak_scalar *= 1.5;
  const bool transfer_only = P.want_transfer && !P.want_cls;
  if (P.want_transfer) {
    if (!(P.transfer_kmax > 0) || P.num_transfer_redshifts < 1 || P.num_transfer_redshifts > 256) {
      err = "transfer kmax and 1-256 redshifts required";
      return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
    }
    for (int i = 1; i < P.num_transfer_redshifts; ++i)
      if (!(P.transfer_redshifts[i] < P.transfer_redshifts[i - 1])) {
        err = "transfer redshifts must be strictly decreasing";
        return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
      }
  }
  // maxq: qmax with the CMB, Transfer%kmax without; the transfer grid runs 5% past kmax
  double maxq = transfer_only ? P.transfer_kmax : c.qmax;
  if (P.want_transfer) maxq = std::max(maxq, P.transfer_kmax * 1.05);
  double taumin = get_tau_start(c, maxq);
  int rc = recfast_init(c, err);
  if (rc) return rc;
  rc = thermo_init(c, taumin, err);
  if (rc) return rc;
  // The logarithmic part of the source k grid ends at min(dkn1/dlnk0, q_switch),
  // (CMB only)
  // which exceeds qmax when max_eta_k is small (lmax below ~220): its modes would start
  // before the thermal tables (the reference stops with 'thermo out of bounds' there).
  // Extend the tables back to the start time of the largest grid wavenumber.
  {
    double SAB = P.AccuracyBoost * P.SourcekAccuracyBoost;
    double dlnk0 = (c.reion.on && P.accurate_polarization) ? 2.0 / 10 / SAB : 5.0 / 10 / SAB;
    if (P.accurate_reionization) dlnk0 /= 2;
    if (c.reion.on && P.accurate_polarization && P.accurate_reionization) dlnk0 = std::min(dlnk0, 0.075);
    double qlog_end = std::min(0.6 / c.taurst / SAB / dlnk0, 2 * 6.3 / c.taurst);
    if (!transfer_only && qlog_end > c.qmax * 1.0001) {
      double dtaurec0 = 4 / c.qmax / initAccuracyBoost;
      c.dtaurec = dtaurec0;
      rc = thermo_init(c, get_tau_start(c, 1.2 * qlog_end), err);
      if (rc) return rc;
    }
  }
  // SetTimeSteps (results.f90:2658-2779)
  {
    double TimeSampleBoost = P.AccuracyBoost * P.TimeStepBoost;
    c.timesteps = Ranges();
    c.timesteps.add_delta(c.taurst, c.taurend, c.dtaurec);
    double dtau0 = c.tau0 / 500.0 / TimeSampleBoost;
    c.timesteps.add_delta(c.taurend, c.tau0, dtau0);
    if (c.reion.on) c.timesteps.add(c.reion_tau_start, c.reion_tau_complete, (int)(c.reion_n_steps * TimeSampleBoost));
    c.timesteps.get_array(true);
  }
  // SetkValuesForSources (cmbmain.f90:864-936)
  {
    double SAB = P.AccuracyBoost * P.SourcekAccuracyBoost;
    double dlnk0;
    if (c.reion.on && P.accurate_polarization) dlnk0 = 2.0 / 10 / SAB;
    else dlnk0 = 5.0 / 10 / SAB;
    if (P.accurate_reionization) dlnk0 /= 2;
    if (c.reion.on && P.accurate_polarization && P.accurate_reionization) dlnk0 = std::min(dlnk0, 0.075);
    // highPrecisionTransferSources: a run that wants high-precision transfer functions with
    // the CMB reuses this grid for them, at least 20 points per e-fold (k_per_logint = 0)
    if (P.want_cls && transfer_hp(P)) dlnk0 = std::min(dlnk0, 1.0 / 20);
    double dkn1 = 0.6 / c.taurst / SAB;
    double dkn2 = 0.9 / c.taurst / SAB / 1.2;
    double q_switch = 2 * 6.3 / c.taurst;
    double qmax_log = std::min(dkn1 / dlnk0, q_switch);
    double q_cmb = 2 * 3000 / c.DMt0 * SAB;
    if (c.maximum_l > 5000 && P.accurate_polarization) q_cmb *= 1.4;
    q_cmb = std::max(q_switch * 2, q_cmb);
    double dksmooth = q_cmb / 2 / (SAB * SAB);
    dksmooth /= 6;
    c.evolve_q = Ranges();
    c.evolve_q.add_delta(c.qmin, qmax_log, dlnk0, true);
    if (c.qmax > qmax_log && q_switch > qmax_log) c.evolve_q.add_delta(qmax_log, std::min(c.qmax, q_switch), dkn1);
    if (c.qmax > q_switch) {
      c.evolve_q.add_delta(q_switch, std::min(q_cmb, c.qmax), dkn2);
      if (c.qmax > q_cmb) {
        dksmooth = std::log(1 + dksmooth / q_cmb);
        c.evolve_q.add_delta(q_cmb, c.qmax, dksmooth, true);
      }
    }
    c.evolve_q.get_array(false);
  }
  c.nsrc = P.do_lensing ? 3 : 2;
  lsamples_init(c, 2, c.maximum_l, c.ls);
  // SetkValuesForInt (cmbmain.f90:1267-1349), flat
  {
    double max_bessels_etak = c.maximum_qeta;
    double qmax_int = std::min(c.qmax, max_bessels_etak / c.tau0);
    double ISB = P.AccuracyBoost * P.IntkAccuracyBoost;
    double LowQIntBoost = ISB;
    if (P.accurate_polarization && P.accurate_reionization) LowQIntBoost *= 1.8;
    int lognum = nint(10 * LowQIntBoost);
    double dlnk1 = 1.0 / lognum;
    int no = nint(600 * ISB);
    double dk0 = 1.8 / c.DMt0 / LowQIntBoost;
    double dk = 3.0 / c.DMt0 / ISB / 1.6;
    double k_max_log = lognum * dk0, k_max_0 = no * dk0;
    double dk2 = 0.04 / ISB;
    c.q_int = Ranges();
    c.q_int.add_delta(c.qmin, k_max_log, dlnk1, true);
    c.q_int.add_delta(k_max_log, std::min(qmax_int, k_max_0), dk0);
    if (qmax_int > k_max_0) {
      double max_k_dk = std::max(3000, 2 * c.maximum_l) / c.tau0;
      c.q_int.add_delta(k_max_0, std::min(qmax_int, max_k_dk), dk);
      if (qmax_int > max_k_dk) c.q_int.add_delta(max_k_dk, qmax_int, dk2);
    }
    c.q_int.get_array(true);
  }
  c.tol1 = 1e-4 / std::exp(P.AccuracyBoost * P.IntTolBoost - 1);
  // CalcScalarSources and GetTransfer alike: high-precision transfers tighten the
  // tolerance of every mode, the CMB source modes of a run with transfers included
  // (cmbmain.f90:1018-1021, 1180-1181)
  if (transfer_hp(P)) c.tol1 /= 100;
  c.modes.clear();
  c.tr_q.clear();
  c.tr_modes.clear();
  if (P.want_transfer) {
    // transfer times: cumulative DeltaTime over the decreasing redshifts (TimeOfzArr,
    // results.f90:683-711)
    c.transfer_times.assign(P.num_transfer_redshifts, 0.0);
    for (int i = 0; i < P.num_transfer_redshifts; ++i) {
      double t = i == 0 ? c.delta_time(0, 1 / (1 + P.transfer_redshifts[0]))
                        : c.delta_time(1 / (1 + P.transfer_redshifts[i - 1]), 1 / (1 + P.transfer_redshifts[i]));
      c.transfer_times[i] = i == 0 ? t : c.transfer_times[i - 1] + t;
    }
    // InitTransfer optimized spacing, no CMB (cmbmain.f90:573-645); k_per_logint = 0,
    // TransferkBoost = 1
    double boost = P.AccuracyBoost * (transfer_hp(P) ? 1.5 : 1.0);
    double kmax = P.transfer_kmax;
    double q_switch_lowk1 = 0.7 / c.taurst, dlog_lowk1 = 2 * boost;
    double q_switch_lowk = 8 / c.taurst, dlog_lowk = 8 * boost * 2.5;
    double q_switch_osc = std::min(kmax, 30 / c.taurst), d_osc = 200 * boost * 1.8;
    double dlog_osc = 17 * boost;
    double q_switch_highk = std::min(kmax, 90 / c.taurst);
    double dlog_highk = 3 * boost;
    const double amin = 5e-5;
    std::vector<double>& qt = c.q_trans;
    qt.clear();
    int nq = (int)(std::log(q_switch_lowk1 / amin) * dlog_lowk1) + 1;
    for (int i = 1; i <= nq; ++i) qt.push_back(amin * std::exp((i - 1) / dlog_lowk1));
    double last = qt.back();
    nq = (int)(std::log(q_switch_lowk / last) * dlog_lowk) + 1;
    for (int i = 1; i <= nq; ++i) qt.push_back(last * std::exp(i / dlog_lowk));
    last = qt.back();
    if (q_switch_osc > q_switch_lowk) {
      nq = (int)((q_switch_osc - last) * d_osc) + 1;
      for (int i = 1; i <= nq; ++i) qt.push_back(last + i / d_osc);
      last = qt.back();
    }
    if (kmax > last) {
      nq = (int)(std::log(q_switch_highk / last) * dlog_osc) + 1;
      for (int i = 1; i <= nq; ++i) qt.push_back(last * std::exp(i / dlog_osc));
      last = qt.back();
    }
    if (kmax > last) {
      nq = (int)(std::log(kmax / last) * dlog_highk) + 1;
      dlog_highk = nq / std::log(kmax * 1.05 / last);
      for (int i = 1; i <= nq; ++i) qt.push_back(last * std::exp(i / dlog_highk));
    }
  }
  if (transfer_only) {
    for (double q : c.q_trans) c.modes.push_back(mode_setup(c, q, true));
  } else {
    for (double q : c.evolve_q.points) c.modes.push_back(mode_setup(c, q));
    if (P.want_transfer) {
      // InitTransfer with WantCls (cmbmain.f90:681-699): the source modes carry the
      // transfer outputs up to the source grid's last point, the transfer grid's points
      // beyond it (TransferOut, cmbmain.f90:1136-1165) are transfer-only modes
      const double top = c.evolve_q.points.back() + 1e-4;
      c.tr_q = c.evolve_q.points;
      c.tr_modes = c.modes;
      for (double q : c.q_trans)
        if (q > top) {
          c.tr_q.push_back(q);
          c.tr_modes.push_back(mode_setup(c, q, true));
        }
    }
  }
  return 0;
}

// ------------------------------------------------------------------------
// flat Bessel table (bessels.f90:140-228): exact j_l on the x grid, then a
// cubic spline per l in Horner form (natural start, clamped derivative at end)
// ------------------------------------------------------------------------
// j_l(x) for l = 0..lmax: upward recurrence below the turning point l ~ x,
// Miller's downward recurrence above it, normalised on the upward values.
static void sph_bessel_all(int lmax, double x, double* out) {
  if (x == 0) {
    out[0] = 1;
    for (int l = 1; l <= lmax; ++l) out[l] = 0;
    return;
  }
  double j0 = std::sin(x) / x;
  int lup = std::min(lmax, (int)x);
  std::vector<double> up;
  if (x >= 1) {
    up.resize(lup + 1);
    up[0] = j0;
    if (lup >= 1) up[1] = std::sin(x) / (x * x) - std::cos(x) / x;
    for (int l = 1; l < lup; ++l) up[l + 1] = (2 * l + 1) / x * up[l] - up[l - 1];
    for (int l = 0; l <= lup; ++l) out[l] = up[l];
    if (lup == lmax) return;
  } else lup = 0;
  // downward recurrence from above the larger of lmax and x
  double top = std::max((double)lmax, x);
  int N = (int)(top + 20 + 18 * std::cbrt(top));
  double jp1 = 0, jc = 1e-300;
  std::vector<double> dn(lmax + 1, 0.0);
  for (int l = N; l >= 1; --l) {
    double jm1 = (2 * l + 1) / x * jc - jp1;
    if (l - 1 <= lmax) dn[l - 1] = jm1;
    if (l <= lmax) dn[l] = jc;
    jp1 = jc;
    jc = jm1;
    if (std::fabs(jc) > 1e250) {
      jc *= 1e-250;
      jp1 *= 1e-250;
      for (int k = l - 1; k <= lmax; ++k) dn[k] *= 1e-250;
    }
  }
  double scale;
  if (x < 1) scale = j0 / dn[0];
  else {
    int lr = (lup >= 1 && std::fabs(up[lup - 1]) > std::fabs(up[lup])) ? lup - 1 : lup;
    scale = up[lr] / dn[lr];
  }
  for (int l = lup + (x >= 1 ? 1 : 0); l <= lmax; ++l) out[l] = dn[l] * scale;
  if (x < 1) out[0] = j0;
}

static std::mutex g_bessel_mutex;
static std::vector<std::shared_ptr<BesselTable>> g_bessel_cache;

std::shared_ptr<const BesselTable> get_bessel_table(const std::vector<int>& ls, double max_bessels_etak,
                                                    double bessel_boost, double accuracy_boost) {
  double requested_xmax = (double)((int)max_bessels_etak + 1);
  double acc = bessel_boost * accuracy_boost;
  std::lock_guard<std::mutex> lock(g_bessel_mutex);
  for (auto& t : g_bessel_cache)
    if (t->ls == ls && t->xmax >= requested_xmax && std::fabs(t->boost - bessel_boost) < 1e-2 &&
        std::fabs(t->acc - acc) < 1e-2)
      return t;
  auto tab = std::make_shared<BesselTable>();
  tab->ls = ls;
  tab->xmax = requested_xmax;
  tab->acc = acc;
  tab->boost = bessel_boost;
  Ranges br;
  // bessels.f90:170-178; ranges are clipped at x_max for small max_eta_k
  const double edges[6] = {0.0, 1.0, 5.0, 25.0, 150.0, 1e300};
  const double steps[5] = {0.01 / bessel_boost, 0.1 / bessel_boost, 0.2 / bessel_boost, 0.5 / acc, 0.7 / acc};
  for (int r = 0; r < 5 && edges[r] < requested_xmax; ++r)
    br.add_delta(edges[r], std::min(edges[r + 1], requested_xmax), steps[r]);
  br.get_array(false);
  tab->x = br.points;
  int num_xx = (int)tab->x.size(), nl = (int)ls.size();
  int lmax = ls.back();
  std::vector<double> vals((size_t)num_xx * nl);
  unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        std::vector<double> all(lmax + 1);
        for (int i = (int)t; i < num_xx; i += (int)nth) {
          sph_bessel_all(lmax, tab->x[i], all.data());
          for (int j = 0; j < nl; ++j) vals[(size_t)j * num_xx + i] = all[ls[j]];
        }
      });
    for (auto& t : th) t.join();
  }
  static const double cut[25] = {0.000000, 0.000000, 0.063316, 0.208916, 0.448187, 0.769530, 1.158338,
                                 1.601506, 2.088363, 2.610505, 3.161369, 3.735827, 4.329841, 4.940211,
                                 5.564374, 6.200262, 6.846189, 7.500771, 8.162861, 8.831502, 9.505890,
                                 10.185346, 10.869292, 11.557230, 12.248737};
  tab->horner.assign((size_t)nl * (num_xx - 1) * 4, 0.0);
  {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        std::vector<double> y(num_xx), d2(num_xx);
        for (int j = (int)t; j < nl; j += (int)nth) {
          int l = ls[j];
          double xlim = std::max(l - 4.2 * std::cbrt((double)l) - 1, cut[std::min(25, l) - 1]);
          int min_ix = std::max(1, br.index_of(xlim) + 1 - 1);  // Fortran 1-based IndexOf(xlim)-1
          for (int i = 0; i < num_xx; ++i) y[i] = (i + 1 >= min_ix) ? vals[(size_t)j * num_xx + i] : 0.0;
          for (int i = 0; i < std::max(min_ix - 1, 1); ++i) y[i] = 0;
          double xe = tab->x[num_xx - 1], jl = y[num_xx - 1];
          std::vector<double> tmp(l + 2);
          sph_bessel_all(l + 1, xe, tmp.data());
          double djl = (l == 0) ? -tmp[1] : tmp[l - 1] - (l + 1) * jl / xe;
          spline_second_derivs(tab->x.data(), y.data(), num_xx, d2.data(), false, 0, true, djl);
          double* H = &tab->horner[(size_t)j * (num_xx - 1) * 4];
          for (int i = std::max(1, min_ix - 1) - 1; i < num_xx - 1; ++i) {
            double h = tab->x[i + 1] - tab->x[i], h2o6 = h * h / 6;
            double y0 = y[i], y1 = y[i + 1], c1 = y1, c2 = y0 - y1 - h2o6 * (d2[i] + 2 * d2[i + 1]);
            double c3 = 3 * h2o6 * d2[i + 1], c4 = y0 - y1 - c2 - c3;
            H[4 * i + 0] = c1;
            H[4 * i + 1] = c2;
            H[4 * i + 2] = c3;
            H[4 * i + 3] = c4;
          }
        }
      });
    for (auto& t : th) t.join();
  }
  g_bessel_cache.push_back(tab);
  if (g_bessel_cache.size() > 4) g_bessel_cache.erase(g_bessel_cache.begin());
  return tab;
}

int build_shared_grid(const std::vector<const Cosmology*>& cs, SharedGrid& g, std::string& err) {
  if (cs.empty()) {
    err = "shared grid: empty batch";
    return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
  }
  // k and q grids of the member with the median tau0
  std::vector<int> order(cs.size());
  for (size_t i = 0; i < cs.size(); ++i) order[i] = (int)i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return cs[a]->tau0 < cs[b]->tau0; });
  g.grid_member = order[cs.size() / 2];
  const Cosmology& m = *cs[g.grid_member];
  g.evolve_q = m.evolve_q.points;
  g.q_int = m.q_int.points;
  g.dq_int = m.q_int.dpoints;
  // chi grid: from chi = 0 (tau0) out to the largest chi of any member's native time
  // steps, each step the finest native spacing of any member at that chi
  double chi_end = 0;
  for (const Cosmology* c : cs) chi_end = std::max(chi_end, c->tau0 - c->timesteps.points.front());
  auto native_step = [](const Cosmology& c, double chi) {
    const std::vector<double>& t = c.timesteps.points;
    const double tau = c.tau0 - chi;
    if (tau < t.front() || tau > t.back()) return 1e300;
    size_t i = std::upper_bound(t.begin(), t.end(), tau) - t.begin();
    if (i == 0) i = 1;
    if (i >= t.size()) i = t.size() - 1;
    return t[i] - t[i - 1];
  };
  auto min_step = [&](double chi) {
    double h = 1e300;
    for (const Cosmology* c : cs) h = std::min(h, native_step(*c, chi));
    return h;
  };
  std::vector<double> up{0.0};
  while (up.back() < chi_end && up.size() < 1000000) {
    double h = min_step(up.back());
    if (!(h < 1e299)) break;
    h = std::min(h, min_step(up.back() + h));  // do not step over the start of a finer region
    up.push_back(std::min(up.back() + h, chi_end));
  }
  if (up.size() < 4) {
    err = "shared grid: degenerate time steps";
    return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
  }
  const size_t n = up.size();
  g.chi.assign(up.rbegin(), up.rend());  // decreasing chi
  g.dchi.assign(n, 0.0);
  g.dchi[0] = (g.chi[0] - g.chi[1]) / 2;
  for (size_t i = 1; i + 1 < n; ++i) g.dchi[i] = (g.chi[i - 1] - g.chi[i + 1]) / 2;
  g.dchi[n - 1] = (g.chi[n - 2] - g.chi[n - 1]) / 2;
  return 0;
}

int apply_shared_grid(Cosmology& c, const SharedGrid& g) {
  const double tau_floor = 0.5 * c.timesteps.points.front();
  int first = 0;
  while (first < (int)g.chi.size() && c.tau0 - g.chi[first] < tau_floor) ++first;
  c.timesteps.points.clear();
  c.timesteps.dpoints.clear();
  for (size_t i = first; i < g.chi.size(); ++i) {
    c.timesteps.points.push_back(c.tau0 - g.chi[i]);
    c.timesteps.dpoints.push_back(g.dchi[i]);
  }
  c.timesteps.points.back() = c.tau0;
  c.evolve_q.points = g.evolve_q;
  c.evolve_q.dpoints.clear();
  c.modes.clear();
  for (double q : c.evolve_q.points) c.modes.push_back(mode_setup(c, q));
  c.q_int.points = g.q_int;
  c.q_int.dpoints = g.dq_int;
  return first;
}

void fill_view(const Cosmology& c, const BesselTable& b, CambGpuTables& v) {
  std::memset(&v, 0, sizeof(v));
  v.grhog = c.grhog; v.grhor = c.grhor; v.grhornomass = c.grhornomass; v.grhoc = c.grhoc;
  v.grhob = c.grhob; v.grhov = c.grhov; v.grhok = c.grhok; v.adotrad = c.adotrad; v.tau0 = c.tau0;
  v.DMt0 = c.DMt0; v.taurst = c.taurst; v.taurend = c.taurend; v.tau_maxvis = c.tau_maxvis;
  v.matter_verydom_tau = c.matter_verydom_tau; v.akthom = c.akthom; v.fHe = c.fHe;
  v.nu_eig = c.nu_eig; v.nqmax = c.nqmax;
  for (int i = 0; i < 3; ++i) {
    v.nu_masses[i] = c.nu_masses[i]; v.grhormass[i] = c.grhormass[i]; v.nu_tau_nonrel[i] = c.nu_tau_nonrel[i];
  }
  v.nu_q = c.nu_q.empty() ? nullptr : c.nu_q.data();
  v.nu_int_kernel = c.nu_int_kernel.empty() ? nullptr : c.nu_int_kernel.data();
  v.nu_tau_notmassless = c.nu_tau_notmassless.empty() ? nullptr : c.nu_tau_notmassless.data();
  v.nthermo = c.nthermo; v.tauminn = c.tauminn; v.dlntau = c.dlntau; v.dlntau_inv = c.dlntau_inv;
  v.tight_tau = c.tight_tau;
  v.thermo_horner = c.thermo_horner.data();
  v.dotmu = c.dotmu.data(); v.ddotmu = c.ddotmu.data(); v.cs2 = c.cs2.data(); v.dddotmu = c.dddotmu.data(); v.ddddotmu = c.ddddotmu.data();
  v.emmu = c.emmu.data(); v.demmu = c.demmu.data();
  v.ntau = c.timesteps.npoints(); v.tau_points = c.timesteps.points.data();
  v.tau_dpoints = c.timesteps.dpoints.data();
  const bool transfer_only = c.P.want_transfer && !c.P.want_cls;
  if (transfer_only) {
    v.nk = (int)c.q_trans.size(); v.q_evolve = c.q_trans.data(); v.modes = c.modes.data();
  } else {
    v.nk = c.evolve_q.npoints(); v.q_evolve = c.evolve_q.points.data(); v.modes = c.modes.data();
  }
  v.transfer_only = transfer_only ? 1 : 0;
  v.num_transfer_times = transfer_only ? (int)c.transfer_times.size() : 0;
  v.transfer_times = transfer_only ? c.transfer_times.data() : nullptr;
  // with transfer functions wanted too, the source modes keep evolving (and storing their
  // sources) at late times until the last transfer time (CalcScalarSources,
  // cmbmain.f90:1032-1035)
  v.src_keep_tau = (!transfer_only && c.P.want_transfer) ? c.transfer_times.back() : -1.0;
  v.hubble_h = c.P.H0 / 100;
  v.want_cls = c.P.want_cls;
  v.transfer_high_precision = transfer_hp(c.P) ? 1 : 0;
  // latePhotSwitchBoost >= 2 for high-precision transfers (AccuracyTarget > 0)
  v.late_phot_switch_boost_min = transfer_hp(c.P) ? 2.0 : 0.0;
  v.nq = c.q_int.npoints(); v.q_int = c.q_int.points.data(); v.dq_int = c.q_int.dpoints.data();
  v.nl = (int)c.ls.size(); v.ls = c.ls.data();
  v.num_xx = (int)b.x.size();
  v.bess_x = b.x.empty() ? nullptr : b.x.data();
  v.bessel_horner = b.horner.empty() ? nullptr : b.horner.data();
  v.nsrc = c.nsrc; v.want_late_time = c.P.do_lensing ? 1 : 0;
  v.max_etak_scalar = c.max_etak_scalar; v.tol1 = c.tol1; v.max_bessels_etak = c.maximum_qeta;
  v.AccuracyBoost = c.P.AccuracyBoost; v.IntTolBoost = c.P.IntTolBoost;
  v.TimeSwitchBoost = c.P.TimeSwitchBoost; v.BessIntBoost = c.P.BessIntBoost; v.LimberBoost = c.P.LimberBoost;
  v.lAccuracyBoost = c.P.lAccuracyBoost; v.accurate_polarization = c.P.accurate_polarization;
  v.accurate_reionization = c.P.accurate_reionization;
  v.As = c.P.As; v.ns = c.P.ns; v.nrun = c.P.nrun; v.pivot_scalar = c.P.pivot_scalar; v.Alens = c.P.Alens;
  v.max_l = c.P.max_l;
  v.do_lensing = c.P.do_lensing;
  // lSamples%template_l_scale: the drag-angle scale when it differs from 1 by more than
  // template_shift_scale_tol (results.f90:49, 1517-1520)
  v.cl_template_scale = std::fabs(c.scale - 1.0) > 0.01 ? c.scale : 1.0;
  v.lens_accuracy_boost = c.P.AccuracyBoost * (c.P.LensingBoost > 0 ? c.P.LensingBoost : 1.0);
}

void fill_transfer_view(const Cosmology& c, CambGpuTables& v) {
  static const BesselTable empty;
  fill_view(c, empty, v);
  v.nk = (int)c.tr_q.size();
  v.q_evolve = c.tr_q.data();
  v.modes = c.tr_modes.data();
  v.transfer_only = 1;  // the device's transfer-function path, WantCls still set (want_cls)
  v.num_transfer_times = (int)c.transfer_times.size();
  v.transfer_times = c.transfer_times.data();
  v.src_keep_tau = -1.0;
  v.transfer_source_modes = c.evolve_q.npoints();
}


}  // namespace cg
