// Host-side tables for one cosmology: background, recombination, reionization,
// thermal-history tables, the source/integration grids, the l sampling and the
// flat Bessel table.  These are the inputs the GPU hot path consumes; the
// reference builds them on the host too (results.f90 SetParams / Thermo_Init,
// recfast.f90, reionization.f90, cmbmain.f90 InitVars and grid setup,
// bessels.f90 GenerateBessels).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../../include/cambgpu.h"

namespace cg {

// ---- physical constants (constants.f90:17-60) ----
namespace K {
constexpr double pi = 3.1415926535897932384626433832795;
constexpr double twopi = 2 * pi, fourpi = 4 * pi, eightpi = 8 * pi;
constexpr double c = 2.99792458e8;
constexpr double h_P = 6.62607015e-34;
constexpr double G = 6.67430e-11;
constexpr double sigma_thomson = 6.6524587321e-29;
constexpr double sigma_boltz = 5.670374419e-8;
constexpr double k_B = 1.380649e-23;
constexpr double m_p = 1.67262192369e-27;
constexpr double m_e = 9.1093837015e-31;
constexpr double m_H = 1.673575e-27;
constexpr double m_He4 = 6.646479073e-27;
constexpr double mass_ratio_He_H = m_He4 / m_H;
constexpr double Mpc = 3.085677581e22;
constexpr double MPC_in_sec = Mpc / c;
constexpr double barssc0 = k_B / m_p / (c * c);
constexpr double kappa = 8.0 * pi * G;
constexpr double COBE_CMBTemp = 2.7255;
}  // namespace K

// forutils-style ranges of points (RangeUtils TRanges) as used at the call sites
// cmbmain.f90:918-933, 1284-1345, results.f90:2669-2741, bessels.f90:168-180.
// The forutils source is not available; semantics inferred from the call sites:
//  - Add_delta(a,b,d,log): n = max(1, int((b-a)/d + 1 - RangeTol)) equal steps
//    (in log space if log), RangeTol = 0.1;
//  - overlapping ranges are merged so that the finer local spacing wins;
//  - dpoints(i) = (points(i+1)-points(i-1))/2 with half intervals at the ends.
struct Ranges {
  struct R { double lo, hi; int n; bool log; };
  std::vector<R> r;
  std::vector<double> points, dpoints;
  void add_delta(double lo, double hi, double delta, bool islog = false);
  void add(double lo, double hi, int n, bool islog = false);
  void get_array(bool want_dpoints = true);
  int npoints() const { return (int)points.size(); }
  // 0-based index i with points[i] <= x < points[i+1] (clamped to [0, n-2]).
  int index_of(double x) const;
};

// natural/clamped cubic spline helpers
void spline_second_derivs(const double* x, const double* y, int n, double* d2,
                          bool clamp_start = false, double d1_start = 0,
                          bool clamp_end = false, double d1_end = 0);

struct Recfast {
  int nz = 2046;
  double delta_z = 0, minz = 0, maxz = 0, Tnow = 0, NNow = 0, fHe = 0, HO = 0, z_eq = 0;
  double OmegaT = 0, OmegaK = 0, fu = 1.125;
  std::vector<double> xrec, tmrec, xh, th;  // xh/th: [nz-1][4] Horner coefficients
  double x_e(double a) const;
  void xe_Tm(double a, double& xe, double& Tm) const;
};

struct Reion {
  bool on = true;
  double redshift = 10, optical_depth = 0.06, delta_redshift = 0.5, fraction = -1;
  double helium_redshift = 3.5, helium_delta_redshift = 0.4, helium_redshiftstart = 5.5;
  double fHe = 0, WindowVarMid = 0, WindowVarDelta = 0;
  void set_zre(double z);
  double x_e(double z, double xstart = 0) const;
};

struct Cosmology {
  CambGpuParams P;
  // background (CAMBdata)
  double grhocrit, grhog, grhor, grhornomass, grhoc, grhob, grhov, grhok, adotrad;
  // massive neutrinos (MassiveNu / GaugeInterface_Init)
  int nu_eig = 0, nqmax = 0;
  double omnuh2 = 0, nu_masses[3] = {0, 0, 0}, grhormass[3] = {0, 0, 0}, nu_degeneracy[3] = {0, 0, 0};
  double nu_tau_nonrel[3] = {0, 0, 0}, nu_tau_nonrel_phys[3] = {0, 0, 0}, nu_tau_massive[3] = {0, 0, 0};
  std::vector<double> nu_q, nu_int_kernel, nu_tau_notmassless;  // notmassless [eig][nqmax]
  double Nnow, akthom, fHe, z_eq, Omega_de, tau0, DMt0, scale = 1;
  // InitVars
  double qmax, qmin, dtaurec, max_etak_scalar, maximum_qeta;
  int maximum_l;
  // thermal history (TThermoData)
  int nthermo;
  double tauminn, dlntau, dlntau_inv, tight_tau, matter_verydom_tau, actual_opt_depth;
  double taurst, taurend, tau_maxvis, reion_tau_start, reion_tau_complete;
  int reion_n_steps;
  double z_drag, r_drag0;
  std::vector<double> thermo_horner;  // [nthermo][16]
  std::vector<double> dotmu, ddotmu, dddotmu, ddddotmu, emmu, demmu, cs2, xe, tb, adot;
  std::vector<double> dotmu_runmin;  // running minimum of dotmu (non-increasing), for opacity_to_time
  Recfast recfast;
  Reion reion;
  // grids
  Ranges timesteps, evolve_q, q_int;
  std::vector<int> ls;
  std::vector<CambGpuModeSpec> modes;       // per k mode: the source grid, or q_trans without the CMB
  std::vector<double> q_trans, transfer_times;  // transfer k grid and times (transfer functions only)
  // a run that wants the CMB and transfer functions (InitTransfer with WantCls,
  // cmbmain.f90:681-699): the source grid followed by the transfer grid's points above it,
  // with the source modes' own set-up and the others' transfer-only set-up
  std::vector<double> tr_q;
  std::vector<CambGpuModeSpec> tr_modes;
  int nsrc;
  double tol1;

  double dtauda(double a) const;
  double delta_time(double a1, double a2, double tol = -1) const;
  double time_of_z(double z, double tol = -1) const { return delta_time(0, 1 / (z + 1), tol); }
  double ScalarPower(double k) const;
};

// Shared flat Bessel table keyed on (l sampling, x_max, BesselBoost*AccuracyBoost).
struct BesselTable {
  std::vector<int> ls;
  double xmax = 0, acc = 0, boost = 0;
  std::vector<double> x;       // [num_xx]
  std::vector<double> horner;  // [nl][num_xx-1][4]
};

int build_cosmology(const CambGpuParams& p, Cosmology& c, std::string& err);

// Grids shared by a batch of cosmologies (the split-BF16 tensor-core projection needs one
// Bessel matrix j_l(q chi_n) dchi_n per integration q for every member): one comoving-
// distance grid chi_n = tau0 - tau_n (node 0 the largest chi, i.e. the earliest time), one
// source k grid and one integration q grid.  The chi grid follows, at every chi, the finest
// native time spacing (SetTimeSteps) of any member there, so that each member's
// recombination and reionization stay as resolved as on its own grid.
struct SharedGrid {
  std::vector<double> chi, dchi;  // [nchi], decreasing chi; dchi the quadrature weights
  std::vector<double> evolve_q, q_int, dq_int;
  int grid_member = 0;  // the member whose k and q grids are shared
};
int build_shared_grid(const std::vector<const Cosmology*>& cs, SharedGrid& g, std::string& err);
// Replaces a member's time steps (its chi nodes with tau >= taurst / 2), source k grid
// (with its own mode set-up at each k) and integration q grid by the shared ones; returns
// the index of the member's first chi node.
int apply_shared_grid(Cosmology& c, const SharedGrid& g);
std::shared_ptr<const BesselTable> get_bessel_table(const std::vector<int>& ls, double xmax,
                                                    double bessel_boost, double accuracy_boost);
void fill_view(const Cosmology& c, const BesselTable& b, CambGpuTables& v);
// the transfer-function half of a run that wants the CMB too (view of tr_q / tr_modes)
void fill_transfer_view(const Cosmology& c, CambGpuTables& v);

}  // namespace cg
