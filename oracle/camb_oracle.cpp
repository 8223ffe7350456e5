// ORACLE -- test infrastructure only.
//
// CPU restatement of the reference CAMB scalar flat hot path, used by tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker of the
// CUDA library.  Nothing in the product links or calls this file.
//
// It restates, following the reference Fortran line by line in scalar form
// (1-based arrays, same control flow):
//   RungeKuttaDP45            fortran/RungeKuttaDP45.f90:94-408
//   GaugeInterface_ScalEv      fortran/equations.f90:212-234
//   GaugeInterface_EvolveScal  fortran/equations.f90:261-460
//   SetupScalarArrayIndices / CopyScalarVariableArray  equations.f90:585-791
//   GetNumEqns                 equations.f90:860-1070 (massless neutrinos)
//   initial                    equations.f90:1891-2112 (adiabatic mode)
//   derivs + output sources    equations.f90:2273-2949, 1739-1755
//   Thermo_values, IonizationFunctionsAtTime, OpacityToTime  results.f90:1826-1922, 3069-3108
//   CalcScalarSources / DoSourcek / GetTauStart  cmbmain.f90:706-753, 998-1074
//   InitSourceInterpolation / InterpolateSources  cmbmain.f90:1249-1265, 1351-1480
//   DoSourceIntegration / DoFlatIntegration        cmbmain.f90:1491-1569, 1639-1862
//   CalcScalCls                                     cmbmain.f90:3179-3343
// Inputs are the host tables in CambGpuTables (include/cambgpu.h).  The reference
// itself cannot be built here (no Fortran compiler; its forutils submodule is
// empty), so the oracle is pinned by the reference's in-repo known answers
// (tests/golden) rather than by running the reference.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../include/cambgpu.h"

namespace {

inline int nint(double x) { return (int)std::lround(x); }

const int max_l_evolve = 256;
const double ep0 = 1.0e-2;

const int max_nu = 3;
const int lmaxnu_high_ktau = 4;

struct EvolutionVars {
  double q, q2, k_buf, k2_buf;
  int lmaxg, lmaxnr, lmaxgpol, MaxlNeeded;
  int g_ix, r_ix, polind, nvar, ScalEqsToPropagate;
  bool TightCoupling, high_ktau_neutrino_approx, no_nu_multpoles, no_phot_multpoles;
  double TightSwitchoffTime, pig, pigdot, poltruncfac;
  // massive neutrinos (EvolutionVars, equations.f90:66-151)
  int lmaxnu, nq[max_nu], lmaxnu_tau[max_nu], nu_ix[max_nu], nu_pert_ix, lmaxnu_pert;
  bool has_nu_relativistic, MassiveNuApprox[max_nu], nu_nonrelativistic[max_nu];
  double MassiveNuApproxTime[max_nu], G11[max_nu], G30[max_nu], nu_l_boost[max_nu];
  double denlk[max_l_evolve + 1], denlk2[max_l_evolve + 1], polfack[max_l_evolve + 1];
  double* OutputSources;  // non-null inside output()
  double* OutputTransfer;  // non-null inside outtransf(): 13 transfer variables
};

struct RKSettings {
  double max_step_size = 0;
  bool reuse_first_derivative = false;
  double weighted_norm_y = 0, computed_min_step_size = 0, current_step_size = 0, computed_scale = 0;
  double computed_max_step_size = 0, trial_x = 0, trial_step = 0, estimated_error = 0, previous_xend = 0;
  bool xend_reached = false, first_derivative_valid = false;
  int successful_steps = 0, successive_failures = 0;
  long function_evaluations = 0;
};

struct Ctx {
  const CambGpuTables* T;
  double polfac[max_l_evolve + 1], denl[max_l_evolve + 1];
  double epsw;
};

// ---- massive neutrino background in units of one massless eigenstate
// (massive_neutrinos.f90: rho_P 186-216, drho 325-347) ----
namespace nufit {
const double zeta3 = 1.2020569031595942853997, zeta5 = 1.0369277551433699263313, zeta7 = 1.0083492773819228268397;
const double pi = 3.1415926535897932384626433832795;
const double fdc = 7.0 / 120 * pi * pi * pi * pi;
const double const2 = 5.0 / 7.0 / (pi * pi);
const double rc[6] = {7.499710425926954249e-01, 1.188066888581748443e-01, 1.545077526625578401e-01,
                      -8.378996019212282820e-02, 2.123075360029347963e-02, -2.544964203886362908e-03};
const double pc[7] = {9.283417043601330798e-01, 3.156134695375645838e-01, -2.435843189264263742e-01,
                      -2.509793530357270000e-02, 4.067958090718486880e-02, 2.378742143669706002e-03,
                      -1.965863329520473827e-03};
const double lrc[2] = {-1.872929199948838302e-02, 1.831728681837861694e-02};
const double lpc[2] = {1.667044572156534468e-02, -2.277471498716537868e-02};
const double dc[6] = {5.800497880734221123e-01, 1.801974470841860576e-01, -1.602709049602861757e-01,
                      3.167230341650149189e-02, 1.056591590995091534e-02, -3.877662402660121861e-03};
void rho_P(double am, double& rhonu, double& pnu) {
  const double amin = 0.42, amax = 70.0;
  if (am <= amin) {
    double am2 = am * am, am4 = am2 * am2;
    rhonu = 1.0 + const2 * am2 + am4 * (lrc[0] + am2 * lrc[1]);
    pnu = (1.0 - const2 * am2) / 3.0 + am4 * (lpc[0] + am2 * lpc[1]);
    return;
  }
  if (am >= amax) {
    rhonu = 3 / (2 * fdc) * (zeta3 * am + ((15 * zeta5) / 2 - 945.0 / 16 * zeta7 / (am * am)) / am);
    pnu = 900.0 / 120.0 / fdc * (zeta5 - 63.0 / 4 * zeta7 / (am * am)) / am;
    return;
  }
  double fc = std::sqrt(amin * amax), izm = (amax + fc) / (amax - fc);
  double z = ((am - fc) / (am + fc)) * izm;
  double rfit = (((((rc[5] * z + rc[4]) * z + rc[3]) * z + rc[2]) * z + rc[1]) * z + rc[0]);
  double pfit = ((((((pc[6] * z + pc[5]) * z + pc[4]) * z + pc[3]) * z + pc[2]) * z + pc[1]) * z + pc[0]);
  rhonu = (1.0 + 3.0 * zeta3 / (2.0 * fdc) * am) * rfit;
  pnu = pfit / (1.0 + fdc / ((900.0 / 120.0) * zeta5) * am);
}
double drho(double am, double adotoa) {
  const double amin = 0.3, amax = 70.0;
  if (am <= amin) {
    double am2 = am * am;
    return am2 * (2 * const2 + am2 * (.4399706676e-1 * std::log(am) - .2970400378e-2 - .29331377855e-1 * am)) * adotoa;
  }
  if (am >= amax) return 3 / (2 * fdc) * (zeta3 * am + (-(15 * zeta5) / 2 + 2835.0 / 16 * zeta7 / (am * am)) / am) * adotoa;
  double fc = std::sqrt(amin * amax), izm = (amax + fc) / (amax - fc);
  double z = ((am - fc) / (am + fc)) * izm;
  double D = (((((dc[5] * z + dc[4]) * z + dc[3]) * z + dc[2]) * z + dc[1]) * z + dc[0]);
  return am * am / (1.0 + 2.0 * am) * D * adotoa;
}
}  // namespace nufit

// ---- thermal history lookups (results.f90:1826-1880, 3069-3108) ----
void thermo_values(const Ctx& C, double tau, double& a, double& cs2b, double& opacity, double* dopacity) {
  const CambGpuTables* T = C.T;
  double d = std::log(tau / T->tauminn) * T->dlntau_inv + 1.0;
  int i = (int)d;
  d = d - i;
  if (i >= T->nthermo) {
    cs2b = T->cs2[T->nthermo - 1];
    opacity = T->dotmu[T->nthermo - 1];
    a = 1;
    if (dopacity) *dopacity = T->ddotmu[T->nthermo - 1] / (tau * T->dlntau);
  } else {
    const double* h = &T->thermo_horner[(size_t)(i - 1) * 16];
    cs2b = h[0] + d * (h[1] + d * (h[2] + d * h[3]));
    opacity = h[4] + d * (h[5] + d * (h[6] + d * h[7]));
    a = (h[8] + d * (h[9] + d * (h[10] + d * h[11]))) * tau;
    if (dopacity) *dopacity = (h[12] + d * (h[13] + d * (h[14] + d * h[15]))) / (tau * T->dlntau);
  }
}

void ionization_functions(const Ctx& C, double tau, double& a, double& opac, double& dopac, double& ddopac,
                          double& vis, double& dvis, double& ddvis, double& expmmu) {
  const CambGpuTables* T = C.T;
  double cs2;
  thermo_values(C, tau, a, cs2, opac, &dopac);
  double d = std::log(tau / T->tauminn) * T->dlntau_inv + 1.0;
  int i = (int)d;
  d = d - i;
  if (i < T->nthermo) {
    const double *f3 = T->dddotmu, *f4 = T->ddddotmu, *em = T->emmu, *dem = T->demmu;
    int j = i - 1;  // 0-based
    ddopac = (f3[j] + d * (f4[j] + d * (3.0 * (f3[j + 1] - f3[j]) - 2.0 * f4[j] - f4[j + 1] +
                                        d * (f4[j] + f4[j + 1] + 2.0 * (f3[j] - f3[j + 1])))) -
              (T->dlntau * T->dlntau) * tau * dopac) /
             ((tau * T->dlntau) * (tau * T->dlntau));
    expmmu = em[j] + d * (dem[j] + d * (3.0 * (em[j + 1] - em[j]) - 2.0 * dem[j] - dem[j + 1] +
                                        d * (dem[j] + dem[j + 1] + 2.0 * (em[j] - em[j + 1]))));
  } else {
    int j = T->nthermo - 1;
    ddopac = (T->dddotmu[j] - (T->dlntau * T->dlntau) * tau * dopac) / ((tau * T->dlntau) * (tau * T->dlntau));
    expmmu = T->emmu[j];
  }
  vis = opac * expmmu;
  dvis = expmmu * (opac * opac + dopac);
  ddvis = expmmu * (opac * opac * opac + 3 * opac * dopac + ddopac);
}

double opacity_to_time(const Ctx& C, double opacity) {
  int j = 1;
  while (j < C.T->nthermo && C.T->dotmu[j - 1] > opacity) ++j;
  return std::exp((j - 1) * C.T->dlntau) * C.T->tauminn;
}

// ---- GetNumEqns (massless neutrinos) ----
void get_num_eqns(const Ctx& C, EvolutionVars& EV, const CambGpuModeSpec& ms) {
  const CambGpuTables* T = C.T;
  double lab = T->lAccuracyBoost;
  int min_lmaxnr = std::max(3, nint(3 * lab));
  double max_nu_mass = 0;
  EV.lmaxnu = 0;
  if (T->nu_eig > 0) {
    for (int i = 0; i < T->nu_eig; ++i) max_nu_mass = std::max(max_nu_mass, T->nu_masses[i]);
    for (int i = 0; i < T->nu_eig; ++i) {
      int q_rel = 0;
      for (int j = 1; j <= T->nqmax; ++j) {
        if (T->nu_q[j - 1] > T->nu_masses[i] * T->adotrad / EV.q) break;
        q_rel++;
      }
      EV.nq[i] = (q_rel >= T->nqmax - 2) ? T->nqmax : q_rel;
      EV.nu_nonrelativistic[i] = false;
      EV.nu_l_boost[i] = ms.nu_l_boost[i];  // MassiveNuTransferLAccuracyBoost, a host input
    }
    if (T->transfer_high_precision) {
      EV.lmaxnu = nint(25 * lab);
      for (int i = 0; i < T->nu_eig; ++i) EV.lmaxnu = std::max(EV.lmaxnu, nint(25 * EV.nu_l_boost[i]));
    } else {
      EV.lmaxnu = std::max(3, nint(10 * lab));
      if (max_nu_mass > 700) EV.lmaxnu = std::max(3, nint(15 * lab));
      for (int i = 0; i < T->nu_eig; ++i) {
        EV.lmaxnu = std::max(EV.lmaxnu, nint(10 * EV.nu_l_boost[i]));
        if (T->nu_masses[i] > 700) EV.lmaxnu = std::max(EV.lmaxnu, nint(15 * EV.nu_l_boost[i]));
      }
    }
  }
  EV.high_ktau_neutrino_approx = false;
  for (int i = 0; i < max_nu; ++i) EV.MassiveNuApprox[i] = false;
  EV.TightCoupling = true;
  EV.no_phot_multpoles = false;
  EV.no_nu_multpoles = false;
  if (T->accurate_polarization) EV.lmaxg = std::max(nint(11 * lab), 3);
  else EV.lmaxg = std::max(nint(8 * lab), 3);
  EV.lmaxnr = std::max(nint(14 * lab), min_lmaxnr);
  if (max_nu_mass > 700) EV.lmaxnr = std::max(nint(32 * lab), min_lmaxnr);
  EV.lmaxgpol = EV.lmaxg;
  if (!T->accurate_polarization) EV.lmaxgpol = std::max(nint(4 * lab), 3);
  else if (T->want_cls && EV.q > 0.15) {  // AccuracyTarget > 0 and Want_CMB
    EV.lmaxg = std::max(EV.lmaxg, nint(13 * lab));
    EV.lmaxgpol = std::max(EV.lmaxgpol, nint(14 * lab));
  }
  if (EV.q < 0.05) {
    double scal = T->accurate_polarization ? 4 : 1;
    EV.lmaxgpol = std::max(3, nint(std::min(8, nint(scal * 150 * EV.q)) * lab));
    EV.lmaxnr = std::max(min_lmaxnr, nint(std::min(8, nint(std::sqrt(scal) * 150 * EV.q)) * lab));
    EV.lmaxg = std::max(3, nint(std::min(8, nint(std::sqrt(scal) * 300 * EV.q)) * lab));
    if (T->accurate_reionization) {
      EV.lmaxg = EV.lmaxg * 8;
      EV.lmaxgpol = EV.lmaxgpol * 2;
    }
  }
  if (T->transfer_only) {  // EV%TransferOnly (equations.f90:968-971)
    EV.lmaxgpol = std::min(EV.lmaxgpol, nint(5 * lab));
    EV.lmaxg = std::min(EV.lmaxg, nint(6 * lab));
  }
  if (T->transfer_high_precision && EV.q > 0.03 && EV.q < 0.2) {  // equations.f90:974-978
    EV.lmaxg = std::max(EV.lmaxg, nint(12 * lab));
    EV.lmaxgpol = std::max(EV.lmaxgpol, nint(5 * lab));
  }
  if (T->transfer_high_precision) {  // equations.f90:979-996
    if (EV.q >= 0.005) EV.lmaxnr = std::max(EV.lmaxnr, nint(4 * lab));
    if (EV.q >= 0.010 && EV.q < 0.05) {
      double t = (8.0 + 6.0 * (EV.q - 0.010) / 0.040) * lab;
      EV.lmaxnr = std::max(std::max(EV.lmaxnr, nint(t)), min_lmaxnr);
    } else if (EV.q >= 0.05 && EV.q < 0.12) {
      double t = (14.0 + 31.0 * (EV.q - 0.05) / 0.07) * lab;
      EV.lmaxnr = std::max(std::max(EV.lmaxnr, nint(t)), min_lmaxnr);
    } else if (EV.q >= 0.12) {
      EV.lmaxnr = std::max(nint(45 * lab), min_lmaxnr);
    }
    if (EV.q > 0.04 && EV.q < 0.5) EV.lmaxg = std::max(EV.lmaxg, nint(10 * lab));
  }
  if (EV.lmaxnr < EV.lmaxnu) EV.lmaxnr = EV.lmaxnu;
  EV.poltruncfac = (double)EV.lmaxgpol / std::max(1, EV.lmaxgpol - 2);
  EV.MaxlNeeded = std::max(std::max(EV.lmaxg, EV.lmaxnu), std::max(EV.lmaxnr, EV.lmaxgpol));
}

thread_local const Ctx* C_ = nullptr;  // the context of the mode being evolved

void setup_indices(EvolutionVars& EV, bool want_maxeq = false) {
  int neq = 4;
  if (!EV.no_phot_multpoles) {
    EV.g_ix = 5;
    if (EV.TightCoupling) neq += 2;
    else {
      neq += EV.lmaxg + 1;
      EV.polind = neq - 1;
      neq += EV.lmaxgpol - 1;
    }
  }
  if (!EV.no_nu_multpoles) {
    EV.r_ix = neq + 1;
    if (EV.high_ktau_neutrino_approx) neq += 3;
    else neq += EV.lmaxnr + 1;
  }
  int maxeq = 4 + (EV.lmaxg + 1) + (EV.lmaxnr + 1) + EV.lmaxgpol - 1;
  EV.has_nu_relativistic = false;
  if (C_->T->nu_eig > 0) {
    const CambGpuTables* T = C_->T;
    for (int i = 0; i < T->nu_eig; ++i) EV.has_nu_relativistic |= EV.nq[i] != T->nqmax;
    if (EV.has_nu_relativistic) {
      EV.lmaxnu_pert = EV.lmaxnu;
      EV.nu_pert_ix = neq + 1;
      neq += EV.lmaxnu_pert + 1;
      maxeq += EV.lmaxnu_pert + 1;
    } else EV.lmaxnu_pert = 0;
    for (int i = 0; i < T->nu_eig; ++i) {
      double b = EV.nu_l_boost[i];
      if (EV.high_ktau_neutrino_approx) EV.lmaxnu_tau[i] = (int)(lmaxnu_high_ktau * b);
      else {
        EV.lmaxnu_tau[i] = std::max(std::min(nint(0.8 * EV.q * T->nu_tau_nonrel[i] * b), EV.lmaxnu), 3);
        if (EV.nu_nonrelativistic[i]) EV.lmaxnu_tau[i] = std::min(EV.lmaxnu_tau[i], nint(4 * b));
      }
      EV.lmaxnu_tau[i] = std::min(EV.lmaxnu, EV.lmaxnu_tau[i]);
      EV.nu_ix[i] = neq + 1;
      if (EV.MassiveNuApprox[i]) neq += 4;
      else neq += EV.nq[i] * (EV.lmaxnu_tau[i] + 1);
      maxeq += T->nqmax * (EV.lmaxnu + 1);
    }
  }
  EV.ScalEqsToPropagate = neq;
  if (want_maxeq) EV.nvar = maxeq;
}

void copy_vars(const double* y, double* yout, const EvolutionVars& EV, const EvolutionVars& EVo) {
  for (int i = 1; i <= EVo.nvar; ++i) yout[i] = 0;
  for (int i = 1; i <= 4; ++i) yout[i] = y[i];
  if (!EV.no_phot_multpoles && !EVo.no_phot_multpoles) {
    int lmax = (EV.TightCoupling || EVo.TightCoupling) ? 1 : std::min(EV.lmaxg, EVo.lmaxg);
    for (int l = 0; l <= lmax; ++l) yout[EVo.g_ix + l] = y[EV.g_ix + l];
    if (!EV.TightCoupling && !EVo.TightCoupling) {
      lmax = std::min(EV.lmaxgpol, EVo.lmaxgpol);
      for (int l = 2; l <= lmax; ++l) yout[EVo.polind + l] = y[EV.polind + l];
    }
  }
  if (!EV.no_nu_multpoles && !EVo.no_nu_multpoles) {
    int lmax = (EV.high_ktau_neutrino_approx || EVo.high_ktau_neutrino_approx) ? 2 : std::min(EV.lmaxnr, EVo.lmaxnr);
    for (int l = 0; l <= lmax; ++l) yout[EVo.r_ix + l] = y[EV.r_ix + l];
  }
  const CambGpuTables* T = C_->T;
  if (T->nu_eig > 0) {
    for (int i = 0; i < T->nu_eig; ++i) {
      int off = EV.nu_ix[i], off2 = EVo.nu_ix[i];
      if (EV.MassiveNuApprox[i] && EVo.MassiveNuApprox[i]) {
        for (int j = 0; j < 4; ++j) yout[off2 + j] = y[off + j];
      } else if (!EV.MassiveNuApprox[i] && !EVo.MassiveNuApprox[i]) {
        int lmax = std::min(EV.lmaxnu_tau[i], EVo.lmaxnu_tau[i]);
        int nq = std::min(EV.nq[i], EVo.nq[i]);
        for (int iq = 1; iq <= nq; ++iq) {
          int ind = off + (iq - 1) * (EV.lmaxnu_tau[i] + 1), ind2 = off2 + (iq - 1) * (EVo.lmaxnu_tau[i] + 1);
          for (int l = 0; l <= lmax; ++l) yout[ind2 + l] = y[ind + l];
        }
        for (int iq = nq + 1; iq <= EVo.nq[i]; ++iq) {
          int lm = std::min(EVo.lmaxnu_tau[i], EV.lmaxnr);
          int ind2 = off2 + (iq - 1) * (EVo.lmaxnu_tau[i] + 1);
          for (int l = 0; l <= lm; ++l) yout[ind2 + l] = y[EV.r_ix + l];
          double qq = T->nu_q[iq - 1];
          double pert_scale = (T->nu_masses[i] / qq) * (T->nu_masses[i] / qq) / 2;
          lm = std::min(lm, EV.lmaxnu_pert);
          for (int l = 0; l <= lm; ++l) yout[ind2 + l] = yout[ind2 + l] + y[EV.nu_pert_ix + l] * pert_scale;
        }
      }
    }
    if (EVo.has_nu_relativistic && EV.has_nu_relativistic) {
      int lmax = std::min(EVo.lmaxnu_pert, EV.lmaxnu_pert);
      for (int l = 0; l <= lmax; ++l) yout[EVo.nu_pert_ix + l] = y[EV.nu_pert_ix + l];
    }
  }
}

// Nu_Integrate_L01 / L012 / Nu_pinudot / Nu_Intvsq (equations.f90:1178-1356)
void nu_integrate_l012(const EvolutionVars& EV, const double* y, double a, int i, double& drhonu, double& fnu,
                       double& dpnu, double& pinu, bool want_l2) {
  const CambGpuTables* T = C_->T;
  drhonu = fnu = dpnu = pinu = 0;
  double am = a * T->nu_masses[i];
  int ind = EV.nu_ix[i];
  for (int iq = 1; iq <= EV.nq[i]; ++iq) {
    double aq = am / T->nu_q[iq - 1];
    double w = T->nu_int_kernel[iq - 1];
    if (want_l2) {
      double v = 1.0 / std::sqrt(1.0 + aq * aq);
      drhonu += w * y[ind] / v;
      fnu += w * y[ind + 1];
      dpnu += w * y[ind] * v;
      pinu += w * y[ind + 2] * v;
    } else {
      drhonu += w * y[ind] * std::sqrt(1.0 + aq * aq);
      fnu += w * y[ind + 1];
    }
    ind += EV.lmaxnu_tau[i] + 1;
  }
  ind = EV.nu_pert_ix;
  for (int iq = EV.nq[i] + 1; iq <= T->nqmax; ++iq) {
    double qq = T->nu_q[iq - 1], aq = am / qq, w = T->nu_int_kernel[iq - 1];
    double pert_scale = (T->nu_masses[i] / qq) * (T->nu_masses[i] / qq) / 2;
    double tmp = w * (y[EV.r_ix] + pert_scale * y[ind]);
    if (want_l2) {
      double v = 1.0 / std::sqrt(1.0 + aq * aq);
      drhonu += tmp / v;
      fnu += w * (y[EV.r_ix + 1] + pert_scale * y[ind + 1]);
      dpnu += tmp * v;
      pinu += w * (y[EV.r_ix + 2] + pert_scale * y[ind + 2]) * v;
    } else {
      drhonu += tmp * std::sqrt(1.0 + aq * aq);
      fnu += w * (y[EV.r_ix + 1] + pert_scale * y[ind + 1]);
    }
  }
  if (want_l2) dpnu = dpnu / 3;
}

double nu_pinudot(const EvolutionVars& EV, const double* y, const double* ydot, double a, double adotoa, int i) {
  const CambGpuTables* T = C_->T;
  double pinudot = 0;
  int ind = EV.nu_ix[i] + 2;
  double am = a * T->nu_masses[i];
  for (int iq = 1; iq <= EV.nq[i]; ++iq) {
    double qq = T->nu_q[iq - 1], aq = am / qq, aqdot = aq * adotoa;
    double v = 1.0 / std::sqrt(1.0 + aq * aq);
    double vdot = -aq * aqdot / std::pow(1.0 + aq * aq, 1.5);
    pinudot += T->nu_int_kernel[iq - 1] * (ydot[ind] * v + y[ind] * vdot);
    ind += EV.lmaxnu_tau[i] + 1;
  }
  ind = EV.nu_pert_ix + 2;
  for (int iq = EV.nq[i] + 1; iq <= T->nqmax; ++iq) {
    double qq = T->nu_q[iq - 1], aq = am / qq, aqdot = aq * adotoa;
    double pert_scale = (T->nu_masses[i] / qq) * (T->nu_masses[i] / qq) / 2;
    double v = 1.0 / std::sqrt(1.0 + aq * aq);
    double vdot = -aq * aqdot / std::pow(1.0 + aq * aq, 1.5);
    double psi2dot = ydot[EV.r_ix + 2] + pert_scale * ydot[ind];
    double psi2 = y[EV.r_ix + 2] + pert_scale * y[ind];
    pinudot += T->nu_int_kernel[iq - 1] * (psi2dot * v + psi2 * vdot);
  }
  return pinudot;
}

void nu_intvsq(const EvolutionVars& EV, const double* y, double a, int i, double& G11, double& G30) {
  const CambGpuTables* T = C_->T;
  double am = a * T->nu_masses[i];
  int ind = EV.nu_ix[i];
  G11 = G30 = 0;
  for (int iq = 1; iq <= EV.nq[i]; ++iq) {
    double aq = am / T->nu_q[iq - 1];
    double v = 1.0 / std::sqrt(1.0 + aq * aq);
    G11 += T->nu_int_kernel[iq - 1] * y[ind + 1] * v * v;
    if (EV.lmaxnu_tau[i] > 2) G30 += T->nu_int_kernel[iq - 1] * y[ind + 3] * v * v;
    ind += EV.lmaxnu_tau[i] + 1;
  }
}

// ---- derivs (equations.f90:2273-2949), flat, Lambda, massless neutrinos ----
void derivs(const Ctx& C, EvolutionVars& EV, int n, double tau, const double* ay, double* ayprime) {
  const CambGpuTables* T = C.T;
  double k = EV.k_buf, k2 = EV.k2_buf;
  double a, cs2, opacity, dopacity = 0;
  if (EV.TightCoupling) thermo_values(C, tau, a, cs2, opacity, &dopacity);
  else thermo_values(C, tau, a, cs2, opacity, nullptr);
  double a2 = a * a;
  double etak = ay[1], clxc = ay[2], clxb = ay[3], vb = ay[4];
  double grhob_t = T->grhob / a, grhoc_t = T->grhoc / a, grhor_t = T->grhornomass / a2, grhog_t = T->grhog / a2;
  double grhov_t = T->grhov * a2, w_dark_energy_t = -1;
  double dgrho_matter = grhob_t * clxb + grhoc_t * clxc;
  double dgq = grhob_t * vb;
  double gpres_nu = 0, grhonu_t = 0, wnu_arr[max_nu] = {0, 0, 0};
  for (int i = 0; i < T->nu_eig; ++i) {  // MassiveNuVars (equations.f90:1358-1401)
    double grhormass_t = T->grhormass[i] / (a * a), rhonu, pnu, clxnu, qnu;
    nufit::rho_P(a * T->nu_masses[i], rhonu, pnu);
    if (EV.MassiveNuApprox[i]) {
      clxnu = ay[EV.nu_ix[i]];
      qnu = ay[EV.nu_ix[i] + 2];
    } else {
      double dp, pn;
      nu_integrate_l012(EV, ay, a, i, clxnu, qnu, dp, pn, false);
      qnu = qnu / rhonu;
      clxnu = clxnu / rhonu;
    }
    double g_t = grhormass_t * rhonu, gp_t = grhormass_t * pnu;
    grhonu_t += g_t;
    gpres_nu += gp_t;
    dgrho_matter += g_t * clxnu;
    dgq += g_t * qnu;
    wnu_arr[i] = pnu / rhonu;
  }
  double grho_matter = grhonu_t + grhob_t + grhoc_t;
  double grho = grho_matter + grhor_t + grhog_t + grhov_t;
  double gpres_noDE = gpres_nu + (grhor_t + grhog_t) / 3;
  double adotoa = std::sqrt(grho / 3);
  double cothxor = 1.0 / tau;
  double dgrho = dgrho_matter;
  double z, dz = 0, clxr, qr, pir, clxg, qg, pig;
  if (EV.no_nu_multpoles) {
    z = (0.5 * dgrho / k + etak) / adotoa;
    dz = -adotoa * z - 0.5 * dgrho / k;
    clxr = -4 * dz / k;
    qr = -4.0 / 3 * z;
    pir = 0;
  } else {
    clxr = ay[EV.r_ix];
    qr = ay[EV.r_ix + 1];
    pir = ay[EV.r_ix + 2];
  }
  pig = 0;
  if (EV.no_phot_multpoles) {
    if (!EV.no_nu_multpoles) {
      z = (0.5 * dgrho / k + etak) / adotoa;
      dz = -adotoa * z - 0.5 * dgrho / k;
      clxg = -4 * dz / k - 4 / k * opacity * (vb + z);
      qg = -4.0 / 3 * z;
    } else {
      clxg = clxr - 4 / k * opacity * (vb + z);
      qg = qr;
    }
  } else {
    clxg = ay[EV.g_ix];
    qg = ay[EV.g_ix + 1];
    if (!EV.TightCoupling) pig = ay[EV.g_ix + 2];
  }
  dgrho = dgrho + grhog_t * clxg + grhor_t * clxr;
  dgq = dgq + grhog_t * qg + grhor_t * qr;
  double photbar = grhog_t / grhob_t;
  double pb43 = 4.0 / 3 * photbar;
  z = (0.5 * dgrho / k + etak) / adotoa;
  double sigma = (z + 1.5 * dgq / k2);
  ayprime[1] = 0.5 * dgq;
  double clxcdot = -k * z;
  ayprime[2] = clxcdot;
  double clxbdot = -k * (z + vb);
  ayprime[3] = clxbdot;
  double clxgdot = -k * (4.0 / 3.0 * z + qg);
  double delta_p_b = cs2 * clxb;
  double vbdot, gpres, pigdot = 0, qgdot = 0, sigmadot, slip, adotdota, dgs;
  if (EV.TightCoupling) {
    gpres = gpres_noDE + w_dark_energy_t * grhov_t;
    adotdota = (adotoa * adotoa - gpres) / 2;
    pig = 32.0 / 45 / opacity * k * (sigma + vb);
    slip = -(2 * adotoa / (1 + pb43) + dopacity / opacity) * (vb - 3.0 / 4 * qg) +
           (-adotdota * vb - k / 2 * adotoa * clxg + k * (cs2 * clxbdot - clxgdot / 4)) / (opacity * (1 + pb43));
    dgs = grhog_t * pig + grhor_t * pir;
    sigmadot = -2 * adotoa * sigma - dgs / k + etak;
    qgdot = k * (clxg / 4.0 - pig / 2.0) + opacity * slip;
    pig = 32.0 / 45 / opacity * k * (sigma + 3.0 * qg / 4.0) * (1 + (dopacity * 11.0 / 6.0 / (opacity * opacity))) +
          (32.0 / 45.0 / (opacity * opacity)) * k * (sigmadot + 3.0 * qgdot / 4.0) * (-11.0 / 6.0);
    pigdot = -(32.0 / 45.0) * (dopacity / (opacity * opacity)) * k * (sigma + 3.0 * qg / 4.0) *
                 (1 + dopacity * 11.0 / 6.0 / (opacity * opacity)) +
             (32.0 / 45.0 / opacity) * k * (sigmadot + 3.0 * qgdot / 4.0) *
                 (1 + (11.0 / 6.0) * (dopacity / (opacity * opacity)));
    EV.pigdot = pigdot;
    vbdot = (-adotoa * vb + cs2 * k * clxb + k / 4 * pb43 * (clxg - 2 * pig)) / (1 + pb43);
    vbdot = vbdot + pb43 / (1 + pb43) * slip;
    EV.pig = pig;
  } else {
    vbdot = -adotoa * vb + k * delta_p_b - photbar * opacity * (4.0 / 3 * vb - qg);
  }
  ayprime[4] = vbdot;
  double polter = 0;
  if (!EV.no_phot_multpoles) {
    ayprime[EV.g_ix] = clxgdot;
    qgdot = 4.0 / 3 * (-vbdot - adotoa * vb + delta_p_b * k) / pb43 + EV.denlk[1] * clxg - EV.denlk2[1] * pig;
    ayprime[EV.g_ix + 1] = qgdot;
    if (!EV.TightCoupling) {
      double E2 = ay[EV.polind + 2];
      polter = pig / 10 + 9.0 / 15 * E2;
      int ix = EV.g_ix + 2;
      pigdot = EV.denlk[2] * qg - EV.denlk2[2] * ay[ix + 1] - opacity * (pig - polter) + 8.0 / 15.0 * k * sigma;
      ayprime[ix] = pigdot;
      for (int l = 3; l <= EV.lmaxg - 1; ++l) {
        ++ix;
        ayprime[ix] = (EV.denlk[l] * ay[ix - 1] - EV.denlk2[l] * ay[ix + 1]) - opacity * ay[ix];
      }
      ++ix;
      ayprime[ix] = k * ay[ix - 1] - (EV.lmaxg + 1) * cothxor * ay[ix] - opacity * ay[ix];
      ix = EV.polind + 2;
      ayprime[ix] = -opacity * (ay[ix] - polter) - k / 3.0 * ay[ix + 1];
      for (int l = 3; l <= EV.lmaxgpol - 1; ++l) {
        ++ix;
        ayprime[ix] = -opacity * ay[ix] + (EV.denlk[l] * ay[ix - 1] - EV.polfack[l] * ay[ix + 1]);
      }
      ++ix;
      ayprime[ix] = -opacity * ay[ix] + k * EV.poltruncfac * ay[ix - 1] - (EV.lmaxgpol + 3) * cothxor * ay[ix];
    }
  }
  double clxrdot = 0, qrdot = 0, pirdot = 0;
  if (!EV.no_nu_multpoles) {
    clxrdot = -k * (4.0 / 3.0 * z + qr);
    ayprime[EV.r_ix] = clxrdot;
    qrdot = EV.denlk[1] * clxr - EV.denlk2[1] * pir;
    ayprime[EV.r_ix + 1] = qrdot;
    if (EV.high_ktau_neutrino_approx) {
      pirdot = -3 * pir * cothxor - clxrdot;
      ayprime[EV.r_ix + 2] = pirdot;
    } else {
      int ix = EV.r_ix + 2;
      pirdot = EV.denlk[2] * qr - EV.denlk2[2] * ay[ix + 1] + 8.0 / 15.0 * k * sigma;
      ayprime[ix] = pirdot;
      for (int l = 3; l <= EV.lmaxnr - 1; ++l) {
        ++ix;
        ayprime[ix] = (EV.denlk[l] * ay[ix - 1] - EV.denlk2[l] * ay[ix + 1]);
      }
      ++ix;
      ayprime[ix] = k * ay[ix - 1] - (EV.lmaxnr + 1) * cothxor * ay[ix];
    }
  }
  // massive neutrino equations of motion (equations.f90:2710-2773)
  for (int i = 0; i < T->nu_eig; ++i) {
    if (EV.MassiveNuApprox[i]) {
      double G11_t = EV.G11[i] / a / a2, G30_t = EV.G30[i] / a / a2;
      int off = EV.nu_ix[i];
      double w = wnu_arr[i];
      ayprime[off] = -k * z * (w + 1) + 3 * adotoa * (w * ay[off] - ay[off + 1]) - k * ay[off + 2];
      ayprime[off + 1] = (3 * w - 2) * adotoa * ay[off + 1] - 5.0 / 3 * k * z * w - k / 3 * G11_t;
      ayprime[off + 2] = (3 * w - 1) * adotoa * ay[off + 2] - k * (2.0 / 3 * ay[off + 3] - ay[off + 1]);
      ayprime[off + 3] = (3 * w - 2) * adotoa * ay[off + 3] + 2 * w * k * sigma - k / 5 * (3 * G30_t - 2 * G11_t);
    } else {
      int ind = EV.nu_ix[i];
      for (int iq = 1; iq <= EV.nq[i]; ++iq) {
        double qq = T->nu_q[iq - 1], aq = a * T->nu_masses[i] / qq;
        double v = 1.0 / std::sqrt(1.0 + aq * aq);
        ayprime[ind] = -k * (4.0 / 3.0 * z + v * ay[ind + 1]);
        ind++;
        ayprime[ind] = v * (EV.denlk[1] * ay[ind - 1] - EV.denlk2[1] * ay[ind + 1]);
        ind++;
        if (EV.lmaxnu_tau[i] == 2) {
          ayprime[ind] = -ayprime[ind - 2] - 3 * cothxor * ay[ind];
        } else {
          ayprime[ind] = v * (EV.denlk[2] * ay[ind - 1] - EV.denlk2[2] * ay[ind + 1]) + k * 8.0 / 15.0 * sigma;
          for (int l = 3; l <= EV.lmaxnu_tau[i] - 1; ++l) {
            ind++;
            ayprime[ind] = v * (EV.denlk[l] * ay[ind - 1] - EV.denlk2[l] * ay[ind + 1]);
          }
          ind++;
          ayprime[ind] = k * v * ay[ind - 1] - (EV.lmaxnu_tau[i] + 1) * cothxor * ay[ind];
        }
        ind++;
      }
    }
  }
  if (EV.has_nu_relativistic) {
    int ind = EV.nu_pert_ix;
    ayprime[ind] = +k * a2 * qr - k * ay[ind + 1];
    int ind2 = EV.r_ix;
    for (int l = 1; l <= EV.lmaxnu_pert - 1; ++l) {
      ind++;
      ind2++;
      ayprime[ind] = -a2 * (EV.denlk[l] * ay[ind2 - 1] - EV.denlk2[l] * ay[ind2 + 1]) +
                     (EV.denlk[l] * ay[ind - 1] - EV.denlk2[l] * ay[ind + 1]);
    }
    ind++;
    ind2++;
    ayprime[ind] = k * (ay[ind - 1] - a2 * ay[ind2 - 1]) - (EV.lmaxnu_pert + 1) * cothxor * ay[ind];
  }
  if (!EV.OutputSources && !EV.OutputTransfer) return;
  // ---- source and transfer output (equations.f90:2775-2912) ----
  double E[4] = {0, 0, 0, 0}, Edot[4] = {0, 0, 0, 0}, octg, octgdot;
  if (!(EV.TightCoupling || EV.no_phot_multpoles)) {
    E[2] = ay[EV.polind + 2];
    E[3] = ay[EV.polind + 3];
    Edot[2] = ayprime[EV.polind + 2];
    Edot[3] = ayprime[EV.polind + 3];
  }
  if (EV.no_nu_multpoles) {
    pirdot = 0;
    qrdot = -4 * dz / 3;
  }
  if (EV.no_phot_multpoles) {
    pigdot = 0;
    octg = 0;
    octgdot = 0;
    qgdot = -4 * dz / 3;
  } else {
    if (EV.TightCoupling) {
      octg = (3.0 / 7.0) * pig * (EV.k_buf / opacity);
      E[2] = pig / 4 + pigdot * (1.0 / opacity) * (-5.0 / 8.0);
      E[3] = (3.0 / 7.0) * (EV.k_buf / opacity) * E[2];
      Edot[2] = (pigdot / 4.0) * (1 + (5.0 / 2.0) * (dopacity / (opacity * opacity)));
      octgdot = 0;
    } else {
      octg = ay[EV.g_ix + 3];
      octgdot = ayprime[EV.g_ix + 3];
    }
  }
  (void)octg;
  double dgpi = grhor_t * pir + grhog_t * pig;
  double dgpi_diff = 0;
  double pidot_sum = grhog_t * pigdot + grhor_t * pirdot;
  double grhonu_out = 0, dgrhonu_out = 0;
  for (int i = 0; i < T->nu_eig; ++i) {  // MassiveNuVarsOut (equations.f90:1113-1176)
    double grhormass_t = T->grhormass[i] / (a * a), rhonu, pnu, clxnu, qnu, pinu, pinudot;
    nufit::rho_P(a * T->nu_masses[i], rhonu, pnu);
    if (EV.MassiveNuApprox[i]) {
      clxnu = ay[EV.nu_ix[i]];
      qnu = ay[EV.nu_ix[i] + 2];
      pinu = ay[EV.nu_ix[i] + 3];
      pinudot = ayprime[EV.nu_ix[i] + 3];
    } else {
      double dpnu;
      nu_integrate_l012(EV, ay, a, i, clxnu, qnu, dpnu, pinu, true);
      qnu = qnu / rhonu;
      clxnu = clxnu / rhonu;
      pinu = pinu / rhonu;
      double rhonudot = nufit::drho(a * T->nu_masses[i], adotoa);
      pinudot = nu_pinudot(EV, ay, ayprime, a, adotoa, i);
      pinudot = pinudot / rhonu - rhonudot / rhonu * pinu;
    }
    (void)qnu;
    double g_t = grhormass_t * rhonu, gp_t = grhormass_t * pnu;
    grhonu_out += g_t;
    dgrhonu_out += g_t * clxnu;
    dgpi += g_t * pinu;
    dgpi_diff += pinu * (3 * gp_t - g_t);
    pidot_sum += g_t * pinudot;
  }
  gpres = gpres_noDE + w_dark_energy_t * grhov_t;
  double diff_rhopi = pidot_sum - (4 * dgpi + dgpi_diff) * adotoa;
  double phi = -((dgrho + 3 * dgq * adotoa / k) + dgpi) / (2 * k2);
  if (EV.OutputTransfer) {  // equations.f90:2832-2845
    double* O = EV.OutputTransfer;
    O[0] = k / T->hubble_h;
    O[1] = clxc;
    O[2] = clxb;
    O[3] = clxg;
    O[4] = clxr;
    O[5] = T->nu_eig > 0 ? dgrhonu_out / grhonu_out : 0.0;  // clxnu_all
    O[6] = dgrho_matter / grho_matter;
    O[7] = (grhob_t * clxb + grhoc_t * clxc) / (grhob_t + grhoc_t);
    O[8] = dgrho / grho_matter;
    O[9] = k2 * phi;
    O[10] = -k * sigma / adotoa;
    O[11] = -k * (vb + sigma) / adotoa;
    O[12] = vb;
  }
  if (!EV.OutputSources) return;
  double ddopacity, visibility, dvisibility, ddvisibility, exptau;
  ionization_functions(C, tau, a, opacity, dopacity, ddopacity, visibility, dvisibility, ddvisibility, exptau);
  double tau0 = T->tau0;
  double phidot = (1.0 / 2.0) * (adotoa * (-dgpi - 2 * k2 * phi) + dgq * k - diff_rhopi + k * sigma * (gpres + grho)) / k2;
  sigmadot = -adotoa * sigma - 1.0 / 2.0 * dgpi / k + k * phi;
  polter = pig / 10 + 9.0 / 15 * E[2];
  double polterdot = (1.0 / 10.0) * pigdot + (3.0 / 5.0) * Edot[2];
  double polterddot = -2.0 / 25.0 * adotoa * dgq / k - 4.0 / 75.0 * adotoa * k * sigma - 4.0 / 75.0 * dgpi -
                      2.0 / 75.0 * dgrho - 3.0 / 50.0 * k * octgdot + (1.0 / 25.0) * k * qgdot -
                      1.0 / 5.0 * k * Edot[3] + (-1.0 / 10.0 * pig + (7.0 / 10.0) * polter - 3.0 / 5.0 * E[2]) * dopacity +
                      (-1.0 / 10.0 * pigdot + (7.0 / 10.0) * polterdot - 3.0 / 5.0 * Edot[2]) * opacity;
  double ISW = 2 * phidot * exptau;
  double monopole_source = (-etak / k + 2 * phi + clxg / 4) * visibility;
  double doppler = ((sigma + vb) * dvisibility + (sigmadot + vbdot) * visibility) / k;
  double quadrupole_source = (5.0 / 8.0) *
                             (3 * polter * ddvisibility + 6 * polterdot * dvisibility + (k * k * polter + 3 * polterddot) * visibility) /
                             (k * k);
  double* S = EV.OutputSources;
  S[0] = ISW + doppler + monopole_source + quadrupole_source;
  double ang_dist = tau0 - tau;
  S[1] = 0;
  if (tau < tau0) S[1] = visibility * polter * (15.0 / 8.0) / (ang_dist * ang_dist * k2);
  if (T->nsrc > 2) {
    S[2] = 0;
    if (tau > T->tau_maxvis && tau0 - tau > 0.1)
      S[2] = -2 * phi * (tau - T->tau_maxvis) / ((tau0 - T->tau_maxvis) * ang_dist);
  }
}

// ---- RungeKuttaDP45 (RungeKuttaDP45.f90:94-408), mixed error control ----
void runge_kutta_dp45(const Ctx& C, EvolutionVars& EV, int n, double& x, double* y, double xend, double tol,
                      int& ind, RKSettings& s, std::vector<double>* w) {
  const double one_fifth = 1.0 / 5.0, default_max_step_size = 20.0;
  const double a21 = 1.0 / 5.0, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0, a41 = 44.0 / 45.0, a42 = -56.0 / 15.0,
               a43 = 32.0 / 9.0, a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0,
               a54 = -212.0 / 729.0, a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0,
               a64 = 49.0 / 176.0, a65 = -5103.0 / 18656.0, b1 = 35.0 / 384.0, b3 = 500.0 / 1113.0,
               b4 = 125.0 / 192.0, b5 = -2187.0 / 6784.0, b6 = 11.0 / 84.0, e1 = 71.0 / 57600.0,
               e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0, e6 = 22.0 / 525.0,
               e7 = -1.0 / 40.0;
  const double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
  double* W[10];
  for (int j = 1; j <= 9; ++j) W[j] = w[j].data();
  if (ind == 1) {
    bool reuse = s.reuse_first_derivative;
    s = RKSettings();
    s.reuse_first_derivative = reuse;
    s.previous_xend = x;
  } else if (ind == 3) {
    s.xend_reached = false;
  }
  if (ind == 1) {
    s.xend_reached = false;
    s.first_derivative_valid = false;
    s.successful_steps = 0;
    s.successive_failures = 0;
    s.function_evaluations = 0;
  }
  for (;;) {
    if (s.function_evaluations > 50000000L) { ind = -1; return; }
    if (ind != 6) {
      if (s.reuse_first_derivative && s.first_derivative_valid) s.first_derivative_valid = false;
      else {
        derivs(C, EV, n, x, y, W[1]);
        s.function_evaluations++;
      }
    }
    double temp = 0;
    for (int i = 1; i <= n; ++i) temp = std::max(temp, std::fabs(y[i]));
    s.weighted_norm_y = std::min(temp, 1.0);
    s.computed_min_step_size = 10.0 * std::max(tiny, eps * std::max(s.weighted_norm_y / tol, std::fabs(x)));
    s.computed_scale = 1;
    s.computed_max_step_size = s.max_step_size != 0 ? std::fabs(s.max_step_size) : default_max_step_size;
    if (s.computed_min_step_size > s.computed_max_step_size) { ind = -2; return; }
    if (ind <= 2) s.current_step_size = s.computed_max_step_size * std::pow(tol, one_fifth);
    else if (s.successive_failures <= 1) {
      temp = 2.0 * s.current_step_size;
      if (tol < std::pow(2.0 / 0.9, 5) * s.estimated_error)
        temp = 0.9 * std::pow(tol / s.estimated_error, one_fifth) * s.current_step_size;
      s.current_step_size = std::max(temp, 0.5 * s.current_step_size);
    } else s.current_step_size = 0.5 * s.current_step_size;
    s.current_step_size = std::min(s.current_step_size, s.computed_max_step_size);
    s.current_step_size = std::max(s.current_step_size, s.computed_min_step_size);
    temp = std::fabs(xend - x);
    if (s.current_step_size < temp && (temp > 1.2 * s.current_step_size || temp > s.computed_max_step_size)) {
      s.current_step_size = std::min(s.current_step_size, 0.5 * temp);
      s.trial_x = x + std::copysign(s.current_step_size, xend - x);
    } else {
      s.current_step_size = temp;
      s.trial_x = xend;
    }
    double h = s.trial_x - x;
    s.trial_step = h;
    for (int i = 1; i <= n; ++i) W[9][i] = y[i] + h * a21 * W[1][i];
    derivs(C, EV, n, x + h / 5.0, W[9], W[2]);
    for (int i = 1; i <= n; ++i) W[9][i] = y[i] + h * (a31 * W[1][i] + a32 * W[2][i]);
    derivs(C, EV, n, x + h * (3.0 / 10.0), W[9], W[3]);
    for (int i = 1; i <= n; ++i) W[9][i] = y[i] + h * (a41 * W[1][i] + a42 * W[2][i] + a43 * W[3][i]);
    derivs(C, EV, n, x + h * (4.0 / 5.0), W[9], W[4]);
    for (int i = 1; i <= n; ++i)
      W[9][i] = y[i] + h * (a51 * W[1][i] + a52 * W[2][i] + a53 * W[3][i] + a54 * W[4][i]);
    derivs(C, EV, n, x + h * (8.0 / 9.0), W[9], W[5]);
    for (int i = 1; i <= n; ++i)
      W[9][i] = y[i] + h * (a61 * W[1][i] + a62 * W[2][i] + a63 * W[3][i] + a64 * W[4][i] + a65 * W[5][i]);
    derivs(C, EV, n, x + h, W[9], W[6]);
    for (int i = 1; i <= n; ++i)
      W[9][i] = y[i] + h * (b1 * W[1][i] + b3 * W[3][i] + b4 * W[4][i] + b5 * W[5][i] + b6 * W[6][i]);
    derivs(C, EV, n, x + h, W[9], W[7]);
    s.function_evaluations += 6;
    temp = 0;
    for (int i = 1; i <= n; ++i) {
      W[2][i] = e1 * W[1][i] + e3 * W[3][i] + e4 * W[4][i] + e5 * W[5][i] + e6 * W[6][i] + e7 * W[7][i];
      temp = std::max(temp, std::fabs(W[2][i]) / std::max(1.0, std::fabs(y[i])));
    }
    s.estimated_error = temp * s.current_step_size * s.computed_scale;
    ind = 5;
    if (s.estimated_error > tol) ind = 6;
    if (ind == 5) {
      x = s.trial_x;
      for (int i = 1; i <= n; ++i) y[i] = W[9][i];
      s.successful_steps++;
      s.successive_failures = 0;
      if (x == xend) {
        ind = 3;
        s.previous_xend = xend;
        s.xend_reached = true;
        if (s.reuse_first_derivative) {
          for (int i = 1; i <= n; ++i) W[1][i] = W[7][i];
          s.first_derivative_valid = true;
        }
        return;
      }
      for (int i = 1; i <= n; ++i) W[1][i] = W[7][i];
      ind = 6;
    } else {
      s.successive_failures++;
      if (s.current_step_size <= s.computed_min_step_size) { ind = -3; return; }
    }
  }
}

struct ModeStats { long evals = 0; int status = 0; };

// next_nu_nq (equations.f90:242-258)
int next_nu_nq(const CambGpuTables* T, int nq) {
  if (nq == 0) return 1;
  int qq = (int)T->nu_q[nq - 1];
  return qq >= 10 ? T->nqmax : nq + 1;
}

// SwitchToMassiveNuApprox (equations.f90:1072-1111)
void switch_to_massive_nu_approx(EvolutionVars& EV, double a, std::vector<double>& y, int i) {
  const CambGpuTables* T = C_->T;
  double a2 = a * a;
  EvolutionVars EVout = EV;
  EVout.MassiveNuApprox[i] = true;
  setup_indices(EVout);
  std::vector<double> yout(EV.nvar + 2, 0.0);
  copy_vars(y.data(), yout.data(), EV, EVout);
  double rhonu, pnu;
  nufit::rho_P(a * T->nu_masses[i], rhonu, pnu);
  double clxnu, qnu, dpnu, pinu;
  nu_integrate_l012(EV, y.data(), a, i, clxnu, qnu, dpnu, pinu, true);
  dpnu = dpnu / rhonu;
  qnu = qnu / rhonu;
  clxnu = clxnu / rhonu;
  pinu = pinu / rhonu;
  yout[EVout.nu_ix[i]] = clxnu;
  yout[EVout.nu_ix[i] + 1] = dpnu;
  yout[EVout.nu_ix[i] + 2] = qnu;
  yout[EVout.nu_ix[i] + 3] = pinu;
  nu_intvsq(EV, y.data(), a, i, EVout.G11[i], EVout.G30[i]);
  EVout.G11[i] = EVout.G11[i] * a2 * a / rhonu;
  EVout.G30[i] = EVout.G30[i] * a2 * a / rhonu;
  EV = EVout;
  y = yout;
}

bool scal_ev(const Ctx& C, EvolutionVars& EV, double* y, double& tau, double tauend, double tol1, int& ind,
             RKSettings& s, std::vector<double>* w, ModeStats& st) {
  if (EV.q < 2e-3 && tau <= C.T->taurend && C.T->want_cls) s.max_step_size = 2.0;
  else s.max_step_size = 20.0 / C.T->IntTolBoost;
  s.reuse_first_derivative = true;
  long before = s.function_evaluations;
  runge_kutta_dp45(C, EV, EV.ScalEqsToPropagate, tau, y, tauend, tol1, ind, s, w);
  st.evals += s.function_evaluations >= before ? s.function_evaluations - before : s.function_evaluations;
  if (ind < 0) { st.status = CAMBGPU_ERROR_EVOLUTION; return false; }
  return true;
}

// GaugeInterface_EvolveScal (equations.f90:261-460) as a loop over switches
bool evolve_scal(const Ctx& C, EvolutionVars& EV, double& tau, std::vector<double>& y, double tauend, double tol1,
                 int& ind, RKSettings& s, std::vector<double>* w, ModeStats& st) {
  const CambGpuTables* T = C.T;
  for (;;) {
    double noSwitch = T->tau0 + 1;
    double smallTime = std::min(tau, 1 / EV.k_buf) / 100;
    double switchBoost = T->AccuracyBoost * T->TimeSwitchBoost;
    double tau_switch_ktau = noSwitch, tau_switch_no_nu_multpoles = noSwitch, tau_switch_no_phot_multpoles = noSwitch;
    double tau_switch_nu_massless = noSwitch, tau_switch_nu_nonrel = noSwitch, tau_switch_nu_massive = noSwitch;
    if (!EV.high_ktau_neutrino_approx && !EV.no_nu_multpoles)
      tau_switch_ktau = std::max(20, EV.lmaxnr - 4) / EV.k_buf;
    for (int i = 0; i < T->nu_eig; ++i) {
      if (EV.nq[i] != T->nqmax)
        tau_switch_nu_massless =
            std::min(tau_switch_nu_massless, T->nu_tau_notmassless[(size_t)i * T->nqmax + next_nu_nq(T, EV.nq[i]) - 1]);
      else if (!EV.nu_nonrelativistic[i]) tau_switch_nu_nonrel = std::min(T->nu_tau_nonrel[i], tau_switch_nu_nonrel);
      else if (!EV.MassiveNuApprox[i]) tau_switch_nu_massive = std::min(tau_switch_nu_massive, EV.MassiveNuApproxTime[i]);
    }
    // DoLateRadTruncation
    if (!EV.no_nu_multpoles)
      tau_switch_no_nu_multpoles = std::max(15 / EV.k_buf * switchBoost, std::min(T->taurend, T->matter_verydom_tau));
    if (!EV.no_phot_multpoles) {
      double latePhotSwitchBoost = switchBoost;
      // high-precision transfers keep the photon hierarchy longer (equations.f90:317-320)
      if (T->transfer_high_precision) latePhotSwitchBoost = std::max(latePhotSwitchBoost, 2.0);
      if (!T->want_cls || EV.k_buf > 0.03 * latePhotSwitchBoost)
        tau_switch_no_phot_multpoles = std::max(15 / EV.k_buf, T->taurend) * latePhotSwitchBoost;
    }
    double next_switch = std::min(std::min(std::min(tau_switch_ktau, tau_switch_nu_massless), EV.TightSwitchoffTime),
                                  std::min(std::min(tau_switch_nu_massive, tau_switch_no_nu_multpoles),
                                           std::min(std::min(tau_switch_no_phot_multpoles, tau_switch_nu_nonrel), noSwitch)));
    if (next_switch < tauend) {
      if (next_switch > tau + smallTime) {
        if (!scal_ev(C, EV, y.data(), tau, next_switch, tol1, ind, s, w, st)) return false;
      }
      EvolutionVars EVout = EV;
      std::vector<double> yout(EV.nvar + 2, 0.0);
      if (next_switch == EV.TightSwitchoffTime) {
        EVout.TightCoupling = false;
        EVout.TightSwitchoffTime = noSwitch;
        setup_indices(EVout);
        copy_vars(y.data(), yout.data(), EV, EVout);
        EV = EVout;
        y = yout;
        ind = 1;
        y[EV.g_ix + 2] = EV.pig;
        double a, cs2, opacity, dopacity;
        thermo_values(C, tau, a, cs2, opacity, &dopacity);
        double kb = EV.k_buf;
        y[EV.g_ix + 3] = (3.0 / 7.0) * y[EV.g_ix + 2] * (kb / opacity) * (1.0 + dopacity / (opacity * opacity)) +
                         (3.0 / 7.0) * EV.pigdot * (kb / (opacity * opacity)) * (-1.0);
        y[EV.polind + 2] = EV.pig / 4 + EV.pigdot * (1.0 / opacity) * (-5.0 / 8.0 - (25.0 / 16.0) * dopacity / (opacity * opacity)) +
                           EV.pig * (kb / opacity) * (kb / opacity) * (-5.0 / 56.0);
        y[EV.polind + 3] = (3.0 / 7.0) * (kb / opacity) * y[EV.polind + 2] * (1.0 + dopacity / (opacity * opacity)) +
                           (3.0 / 7.0) * (kb / (opacity * opacity)) *
                               ((EV.pigdot / 4.0) * (1.0 + (5.0 / 2.0) * dopacity / (opacity * opacity))) * (-1.0);
      } else if (next_switch == tau_switch_ktau) {
        EVout.high_ktau_neutrino_approx = true;
        for (int i = 0; i < T->nu_eig; ++i) EVout.nq[i] = T->nqmax;
        setup_indices(EVout);
        copy_vars(y.data(), yout.data(), EV, EVout);
        y = yout;
        EV = EVout;
      } else if (next_switch == tau_switch_nu_massless) {
        for (int i = 0; i < T->nu_eig; ++i) {
          if (EV.nq[i] != T->nqmax &&
              next_switch == T->nu_tau_notmassless[(size_t)i * T->nqmax + next_nu_nq(T, EV.nq[i]) - 1]) {
            EVout.nq[i] = next_nu_nq(T, EV.nq[i]);
            setup_indices(EVout);
            copy_vars(y.data(), yout.data(), EV, EVout);
            EV = EVout;
            y = yout;
            break;
          }
        }
      } else if (next_switch == tau_switch_nu_nonrel) {
        for (int i = 0; i < T->nu_eig; ++i) {
          if (!EV.nu_nonrelativistic[i] && next_switch == T->nu_tau_nonrel[i]) {
            EVout.nu_nonrelativistic[i] = true;
            setup_indices(EVout);
            copy_vars(y.data(), yout.data(), EV, EVout);
            EV = EVout;
            y = yout;
            break;
          }
        }
      } else if (next_switch == tau_switch_nu_massive) {
        double a, cs2, opacity;
        thermo_values(C, tau, a, cs2, opacity, nullptr);
        for (int i = 0; i < T->nu_eig; ++i) {
          if (!EV.MassiveNuApprox[i] && next_switch == EV.MassiveNuApproxTime[i]) {
            switch_to_massive_nu_approx(EV, a, y, i);
            break;
          }
        }
      } else if (next_switch == tau_switch_no_nu_multpoles) {
        ind = 1;
        EVout.no_nu_multpoles = true;
        for (int i = 0; i < T->nu_eig; ++i) EVout.nq[i] = T->nqmax;
        setup_indices(EVout);
        copy_vars(y.data(), yout.data(), EV, EVout);
        y = yout;
        EV = EVout;
      } else if (next_switch == tau_switch_no_phot_multpoles) {
        ind = 1;
        EVout.no_phot_multpoles = true;
        setup_indices(EVout);
        copy_vars(y.data(), yout.data(), EV, EVout);
        y = yout;
        EV = EVout;
      }
      s.first_derivative_valid = false;
      continue;
    }
    return scal_ev(C, EV, y.data(), tau, tauend, tol1, ind, s, w, st);
  }
}

// initial (equations.f90:1891-2112), adiabatic, flat, massless neutrinos
void initial(const Ctx& C, EvolutionVars& EV, std::vector<double>& y, double tau) {
  const CambGpuTables* T = C.T;
  EV.k_buf = EV.q;
  EV.k2_buf = EV.q2;
  double k = EV.k_buf;
  for (int j = 1; j <= EV.MaxlNeeded; ++j) {
    EV.denlk[j] = C.denl[j] * k * j;
    EV.denlk2[j] = C.denl[j] * k * 1.0 * (j + 1);
    EV.polfack[j] = C.polfac[j] * k * 1.0 * C.denl[j];
  }
  double ep;
  if (EV.k_buf > C.epsw) ep = (EV.k_buf > C.epsw * 5) ? ep0 * 5 / T->AccuracyBoost * 0.65 : ep0;
  else ep = ep0;
  ep = ep * 2;
  EV.TightSwitchoffTime = std::min(T->tight_tau, opacity_to_time(C, EV.k_buf / ep));
  std::fill(y.begin(), y.end(), 0.0);
  double x = k * tau, x2 = x * x, x3 = x2 * x;
  double rhomass = 0;
  for (int i = 0; i < T->nu_eig; ++i) rhomass += T->grhormass[i];
  double grhonu = rhomass + T->grhornomass;
  double om = (T->grhob + T->grhoc) / std::sqrt(3 * (T->grhog + grhonu));
  double omtau = om * tau;
  double Rv = grhonu / (grhonu + T->grhog);
  double Rp15 = 4 * Rv + 15;
  double iv_clxg = -1.0 / 3 * x2 * (1 - omtau / 5);
  double iv_clxr = iv_clxg, iv_clxb = 0.75 * iv_clxg, iv_clxc = iv_clxb;
  double iv_qg = iv_clxg * x / 9.0;
  double iv_qr = -(4 * Rv + 23) / Rp15 * x3 / 27;
  double iv_vb = 0.75 * iv_qg;
  double iv_pir = 4.0 / 3 * x2 / Rp15 * (1 + omtau / 4 * (4 * Rv - 5) / (2 * Rv + 15));
  double iv_aj3r = 4 / 21.0 / Rp15 * x3;
  double iv_eta = -2 * (1 - x2 / 12 * (-10.0 / Rp15 + 1));
  // adiabatic: initvec = -initv(1, :)
  y[1] = -(-iv_eta) * k / 2;
  y[2] = -iv_clxc;
  y[3] = -iv_clxb;
  y[4] = -iv_vb;
  y[EV.g_ix] = -iv_clxg;
  y[EV.g_ix + 1] = -iv_qg;
  y[EV.r_ix] = -iv_clxr;
  y[EV.r_ix + 1] = -iv_qr;
  y[EV.r_ix + 2] = -iv_pir;
  if (EV.lmaxnr > 2) y[EV.r_ix + 3] = -iv_aj3r;
  for (int i = 0; i < T->nu_eig; ++i) {
    int ind = EV.nu_ix[i];
    for (int iq = 1; iq <= EV.nq[i]; ++iq) {
      for (int j = 0; j < 3; ++j) y[ind + j] = y[EV.r_ix + j];
      if (EV.lmaxnu_tau[i] > 2) y[ind + 3] = -iv_aj3r;
      ind += EV.lmaxnu_tau[i] + 1;
    }
  }
}

// CalcScalarSources (cmbmain.f90:998-1074)
// GetTauStart (cmbmain.f90:706-729)
double tau_start(const CambGpuTables* T, double q) {
  double t = std::min(0.001 / q, 0.1);
  double mmax = 0;
  for (int i = 0; i < T->nu_eig; ++i) mmax = std::max(mmax, T->nu_masses[i]);
  if (T->nu_eig > 0 && mmax != 0) t = std::min(t, 1e-3 / mmax / T->adotrad);
  return t;
}

void calc_scalar_sources(const Ctx& C, int q_ix, double* LinearSrc, ModeStats& st) {
  const CambGpuTables* T = C.T;
  C_ = &C;
  EvolutionVars EV{};
  EV.q = T->q_evolve[q_ix];
  EV.q2 = EV.q * EV.q;
  EV.OutputSources = nullptr;
  double taustart = tau_start(T, EV.q);
  const CambGpuModeSpec& ms = T->modes[q_ix];
  get_num_eqns(C, EV, ms);
  setup_indices(EV, true);
  for (int i = 0; i < T->nu_eig; ++i) EV.MassiveNuApproxTime[i] = ms.nu_approx_time[i];
  std::vector<double> w[10];
  for (int j = 1; j <= 9; ++j) w[j].assign(EV.nvar + 2, 0.0);
  std::vector<double> y(EV.nvar + 2, 0.0);
  initial(C, EV, y, taustart);
  double tau = taustart;
  int ind = 1;
  RKSettings s;
  double tol1 = T->tol1;
  int nsrc = T->nsrc, nk = T->nk;
  double sources[8];
  for (int j = 2; j <= T->ntau; ++j) {
    double tauend = T->tau_points[j - 1];
    if (EV.q * tauend > T->max_etak_scalar && tauend > T->taurend && !T->want_late_time && tau > T->src_keep_tau) {
      for (int s_ = 0; s_ < nsrc; ++s_) LinearSrc[((size_t)(j - 1) * nsrc + s_) * nk + q_ix] = 0;
    } else {
      if (!evolve_scal(C, EV, tau, y, tauend, tol1, ind, s, w, st)) return;
      std::vector<double> yprime(EV.nvar + 2, 0.0);
      EV.OutputSources = sources;
      derivs(C, EV, EV.ScalEqsToPropagate, tau, y.data(), yprime.data());
      EV.OutputSources = nullptr;
      for (int s_ = 0; s_ < nsrc; ++s_) LinearSrc[((size_t)(j - 1) * nsrc + s_) * nk + q_ix] = sources[s_];
    }
  }
}

// outtransf (equations.f90:2256-2271) at the current state: the 13 transfer variables in
// single precision, the entries after k/h divided by k^2 after the float store
static void store_transfer(const Ctx& C, EvolutionVars& EV, double tau, std::vector<double>& y, float* o) {
  double O[13];
  std::vector<double> yprime(EV.nvar + 2, 0.0);
  EV.OutputTransfer = O;
  derivs(C, EV, EV.ScalEqsToPropagate, tau, y.data(), yprime.data());
  EV.OutputTransfer = nullptr;
  o[0] = (float)O[0];
  for (int v = 1; v < 13; ++v) {
    float f = (float)O[v];
    o[v] = (float)(f / EV.k2_buf);
  }
}

// CalcScalarSources with WantTransfer (cmbmain.f90:998-1074), the reference's form of a run
// that wants the CMB and transfer functions: the source mode also stops at every transfer
// time (before the second source time, or inside the source interval that contains it) and
// stores the transfer variables there as TransferData(:, q_ix, itf) of the transfer half
// `Ttr` (its first nk entries are the source grid); it keeps evolving at late times until
// the last transfer time.
void calc_sources_and_transfers(const Ctx& C, const CambGpuTables* Ttr, int q_ix, double* LinearSrc, float* tr,
                                ModeStats& st) {
  const CambGpuTables* T = C.T;
  C_ = &C;
  EvolutionVars EV{};
  EV.q = T->q_evolve[q_ix];
  EV.q2 = EV.q * EV.q;
  EV.OutputSources = nullptr;
  EV.OutputTransfer = nullptr;
  double taustart = tau_start(T, EV.q);
  const CambGpuModeSpec& ms = T->modes[q_ix];
  get_num_eqns(C, EV, ms);
  setup_indices(EV, true);
  for (int i = 0; i < T->nu_eig; ++i) EV.MassiveNuApproxTime[i] = ms.nu_approx_time[i];
  std::vector<double> w[10];
  for (int j = 1; j <= 9; ++j) w[j].assign(EV.nvar + 2, 0.0);
  std::vector<double> y(EV.nvar + 2, 0.0);
  initial(C, EV, y, taustart);
  double tau = taustart;
  int ind = 1;
  RKSettings s;
  const double tol1 = T->tol1;
  const int nsrc = T->nsrc, nk = T->nk, ntau = T->ntau;
  const int ntr = Ttr->num_transfer_times, trk = Ttr->nk;
  const double* TT = Ttr->transfer_times;
  auto out_tr = [&](int itf) { store_transfer(C, EV, tau, y, tr + ((size_t)itf * trk + q_ix) * 13); };
  int itf = 0;
  while (itf < ntr && T->tau_points[1] > TT[itf]) {
    if (!evolve_scal(C, EV, tau, y, TT[itf], tol1, ind, s, w, st)) return;
    out_tr(itf);
    ++itf;
  }
  double sources[8];
  for (int j = 2; j <= ntau; ++j) {  // the reference's 1-based time index
    const double tauend = T->tau_points[j - 1];
    if (EV.q * tauend > T->max_etak_scalar && tauend > T->taurend && !T->want_late_time && tau > TT[ntr - 1]) {
      for (int s_ = 0; s_ < nsrc; ++s_) LinearSrc[((size_t)(j - 1) * nsrc + s_) * nk + q_ix] = 0;
      continue;
    }
    if (!evolve_scal(C, EV, tau, y, tauend, tol1, ind, s, w, st)) return;
    std::vector<double> yprime(EV.nvar + 2, 0.0);
    EV.OutputSources = sources;
    derivs(C, EV, EV.ScalEqsToPropagate, tau, y.data(), yprime.data());
    EV.OutputSources = nullptr;
    for (int s_ = 0; s_ < nsrc; ++s_) LinearSrc[((size_t)(j - 1) * nsrc + s_) * nk + q_ix] = sources[s_];
    bool again = true;  // the reference's `goto 101`
    while (again && itf < ntr) {
      again = false;
      if (j < ntau && tauend < TT[itf] && T->tau_points[j] > TT[itf])
        if (!evolve_scal(C, EV, tau, y, TT[itf], tol1, ind, s, w, st)) return;
      if (std::fabs(tau - TT[itf]) < 1e-5 || j == ntau) {
        out_tr(itf);
        ++itf;
        if (j < ntau && itf < ntr && T->tau_points[j] > TT[itf]) again = true;
      }
    }
  }
}

// GetTransfer (cmbmain.f90:1167-1188) + outtransf (equations.f90:2256-2271): the mode is
// evolved to every transfer time and the 13 transfer variables are stored in single
// precision as MatterTransferData%TransferData(:, q_ix, itf), the entries after k/h
// divided by k^2 after the float store.
void calc_transfer(const Ctx& C, int q_ix, float* out, ModeStats& st) {
  const CambGpuTables* T = C.T;
  C_ = &C;
  EvolutionVars EV{};
  EV.q = T->q_evolve[q_ix];
  EV.q2 = EV.q * EV.q;
  EV.OutputSources = nullptr;
  EV.OutputTransfer = nullptr;
  const CambGpuModeSpec& ms = T->modes[q_ix];
  get_num_eqns(C, EV, ms);
  setup_indices(EV, true);
  for (int i = 0; i < T->nu_eig; ++i) EV.MassiveNuApproxTime[i] = ms.nu_approx_time[i];
  std::vector<double> w[10];
  for (int j = 1; j <= 9; ++j) w[j].assign(EV.nvar + 2, 0.0);
  std::vector<double> y(EV.nvar + 2, 0.0);
  double tau = tau_start(T, EV.q);
  initial(C, EV, y, tau);
  int ind = 1;
  RKSettings s;
  for (int itf = 0; itf < T->num_transfer_times; ++itf) {
    if (!evolve_scal(C, EV, tau, y, T->transfer_times[itf], T->tol1, ind, s, w, st)) return;
    double O[13];
    std::vector<double> yprime(EV.nvar + 2, 0.0);
    EV.OutputTransfer = O;
    derivs(C, EV, EV.ScalEqsToPropagate, tau, y.data(), yprime.data());
    EV.OutputTransfer = nullptr;
    float* o = out + ((size_t)itf * T->nk + q_ix) * 13;
    o[0] = (float)O[0];
    for (int v = 1; v < 13; ++v) {
      float f = (float)O[v];
      o[v] = (float)(f / EV.k2_buf);
    }
  }
}

void init_ctx(Ctx& C, const CambGpuTables* T) {
  C.T = T;
  for (int j = 2; j <= max_l_evolve; ++j) C.polfac[j] = (double)((j + 3) * (j - 1)) / (j + 1);
  C.polfac[1] = 0;
  for (int j = 1; j <= max_l_evolve; ++j) C.denl[j] = 1.0 / (2 * j + 1);
  C.epsw = 100 / T->tau0;
}

// natural cubic spline second derivatives (as forutils cubic_spline_second_derivs)
void spline_d2(const double* x, const double* y, int n, double* d2) {
  std::vector<double> u(n);
  d2[0] = 0;
  u[0] = 0;
  for (int i = 1; i < n - 1; ++i) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * d2[i - 1] + 2.0;
    d2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  d2[n - 1] = 0;
  for (int k = n - 2; k >= 0; --k) d2[k] = d2[k] * d2[k + 1] + u[k];
}

int index_of(const double* pts, int n, double x) {  // 1-based index with pts(i) <= x < pts(i+1)
  if (x < pts[0]) return 0;
  if (x >= pts[n - 1]) return n;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (x >= pts[mid]) lo = mid; else hi = mid;
  }
  return lo + 1;
}

}  // namespace

extern "C" {

// Mode setup as restated from GetNumEqns/initial, for cross-checking the product's
// per-mode specs: out = [lmaxg, lmaxgpol, lmaxnr], tight_switch_tau.
int oracle_mode_setup(const CambGpuTables* T, double q, int* lmax3, double* tight_switch) {
  Ctx C;
  init_ctx(C, T);
  C_ = &C;
  EvolutionVars EV{};
  EV.q = q;
  EV.q2 = q * q;
  int q_ix = 0;
  for (int i = 0; i < T->nk; ++i)
    if (T->q_evolve[i] == q) q_ix = i;
  get_num_eqns(C, EV, T->modes[q_ix]);
  setup_indices(EV, true);
  std::vector<double> y(EV.nvar + 2);
  initial(C, EV, y, tau_start(T, q));
  lmax3[0] = EV.lmaxg;
  lmax3[1] = EV.lmaxgpol;
  lmax3[2] = EV.lmaxnr;
  *tight_switch = EV.TightSwitchoffTime;
  return 0;
}

// TransferOut (cmbmain.f90:1136-1165) -- OpenMP over the transfer k, descending.
// out: [num_transfer_times][nk][13] floats.
int oracle_evolve_transfer(const CambGpuTables* T, float* out, int nthreads, long* evals) {
  Ctx C;
  init_ctx(C, T);
  int nk = T->nk, status = 0;
  // the transfer half of a run with the CMB has source modes that also stop at the source
  // times: oracle_evolve_combined restates that run
  if (!T->transfer_only || T->transfer_source_modes > 0) return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
  for (int i = nk - 1; i >= 0; --i) {
    ModeStats st;
    calc_transfer(C, i, out, st);
    if (evals) evals[i] = st.evals;
    if (st.status) {
#pragma omp critical
      status = st.status;
    }
  }
  return status;
}

// A run that wants the CMB and transfer functions, as the reference computes it: the
// source modes of `Tcmb` by CalcScalarSources with the transfer stops, the transfer
// half's modes above the source grid by TransferOut (cmbmain.f90:182-221).
// LinearSrc: [ntau][nsrc][Tcmb->nk]; tr: [num_transfer_times][Ttr->nk][13].
int oracle_evolve_combined(const CambGpuTables* Tcmb, const CambGpuTables* Ttr, double* LinearSrc, float* tr,
                           int nthreads) {
  if (Tcmb->transfer_only || !Ttr->transfer_only || Ttr->num_transfer_times < 1 || Ttr->nk < Tcmb->nk)
    return CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
  Ctx C, Ct;
  init_ctx(C, Tcmb);
  init_ctx(Ct, Ttr);
  int status = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const int nsrc_k = Tcmb->nk, ntot = Ttr->nk;
#pragma omp parallel for schedule(dynamic)
  for (int i = ntot - 1; i >= 0; --i) {
    ModeStats st;
    if (i < nsrc_k) calc_sources_and_transfers(C, Ttr, i, LinearSrc, tr, st);
    else calc_transfer(Ct, i, tr, st);
    if (st.status) {
#pragma omp critical
      status = st.status;
    }
  }
  return status;
}

// Transfer_Get_sigmas (results.f90:4115-4182) at R = 8 Mpc/h with delta = total matter
// (Transfer_tot) and v = Newtonian CDM velocity, for every transfer time.
void oracle_sigma8(const CambGpuTables* T, const float* tr, double* sigma8, double* sigma2_vdelta_8) {
  const double pi = 3.1415926535897932384626433832795;
  (void)pi;
  int nz = T->num_transfer_times, nk = T->nk;
  double h = T->hubble_h;
  for (int z = 0; z < nz; ++z) {
    double lnko = 0, dsig8o = 0, sig8 = 0, dsigvo = 0, sigv = 0;
    for (int ik = 0; ik < nk; ++ik) {
      double kh = tr[((size_t)0 * nk + ik) * 13 + 0];
      if (kh == 0) continue;
      double k = kh * h;
      double delta = tr[((size_t)z * nk + ik) * 13 + 6];
      double dsig8 = delta * delta;
      double dsigv = delta * tr[((size_t)z * nk + ik) * 13 + 10];
      double x = kh * 8.0, win;
      if (x < 1e-2) win = 1.0 - x * x / 10;
      else win = 3 * (std::sin(x) - x * std::cos(x)) / (x * x * x);
      double lnk = std::log(k), dlnk;
      if (ik == 0) dlnk = 0.5;
      else dlnk = lnk - lnko;
      double lnrat = std::log(k / T->pivot_scalar);
      double pk = T->As * std::exp(lnrat * (T->ns - 1 + lnrat * (T->nrun / 2)));
      double powers = (win * k * k) * (win * k * k) * pk;
      dsig8 = powers * dsig8;
      sig8 += (dsig8 + dsig8o) * dlnk / 2;
      dsig8o = dsig8;
      dsigv = powers * dsigv;
      sigv += (dsigv + dsigvo) * dlnk / 2;
      dsigvo = dsigv;
      lnko = lnk;
    }
    sigma8[z] = std::sqrt(sig8);
    sigma2_vdelta_8[z] = sigv;
  }
}

// cmbmain.f90:205-209 -- OpenMP over k, dynamic schedule, k descending.
// evals (optional, [nk]) receives the derivative evaluations per mode.
int oracle_evolve_scalar_sources(const CambGpuTables* T, double* LinearSrc, int nthreads, long* evals, int k_lo,
                                 int k_hi) {
  Ctx C;
  init_ctx(C, T);
  if (k_hi <= 0 || k_hi > T->nk) k_hi = T->nk;
  if (k_lo < 0) k_lo = 0;
  int err = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
  for (int q_ix = k_hi - 1; q_ix >= k_lo; --q_ix) {
    ModeStats st;
    calc_scalar_sources(C, q_ix, LinearSrc, st);
    if (evals) evals[q_ix] = st.evals;
    if (st.status) {
#pragma omp critical
      err = st.status;
    }
  }
  return err;
}

// cmbmain.f90:1249-1265 (spline in k), 287-291 and 1351-1862 (flat LOS)
int oracle_los_flat(const CambGpuTables* T, const double* LinearSrc, double* Delta, int nthreads) {
  int nk = T->nk, ntau = T->ntau, nsrc = T->nsrc, nl = T->nl, nq = T->nq;
  std::vector<double> dd((size_t)ntau * nsrc * nk);
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ntau; ++i)
    for (int j = 0; j < nsrc; ++j)
      spline_d2(T->q_evolve, &LinearSrc[((size_t)i * nsrc + j) * nk], nk, &dd[((size_t)i * nsrc + j) * nk]);
  const double max_etak = T->want_late_time ? 0 : T->max_etak_scalar;
  const bool ignore_etak = T->want_late_time != 0;
  std::memset(Delta, 0, sizeof(double) * (size_t)nq * nl * nsrc);
#pragma omp parallel for schedule(static, 4)
  for (int q_ix = 0; q_ix < nq; ++q_ix) {
    double q = T->q_int[q_ix];
    std::vector<double> Src((size_t)(ntau + 1) * nsrc, 0.0);  // Source_q(i, s) 1-based i
    // InterpolateSources
    int klo;
    if (q <= T->q_evolve[0]) klo = 1;
    else if (q >= T->q_evolve[nk - 1]) klo = nk - 1;
    else {
      int lo = 1, hi = nk;
      while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (q >= T->q_evolve[mid - 1]) lo = mid; else hi = mid;
      }
      klo = lo;
    }
    int khi = klo + 1;
    double ho = T->q_evolve[khi - 1] - T->q_evolve[klo - 1];
    double a0 = (T->q_evolve[khi - 1] - q) / ho, b0 = (q - T->q_evolve[klo - 1]) / ho;
    double ho2o6 = ho * ho / 6.0, a03 = a0 * a0 * a0 - a0, b03 = b0 * b0 * b0 - b0;
    int step = 2;
    for (int i = 2; i <= ntau; ++i) {
      double tau = T->tau_points[i - 1];
      double xf = q * (T->tau0 - tau);
      if ((ignore_etak || q * tau < max_etak) && xf > 1e-8) {
        step = i;
        for (int j = 0; j < nsrc; ++j) {
          size_t b = ((size_t)(i - 1) * nsrc + j) * nk;
          Src[(size_t)i * nsrc + j] = a0 * LinearSrc[b + klo - 1] + b0 * LinearSrc[b + khi - 1] +
                                      (a03 * dd[b + klo - 1] + b03 * dd[b + khi - 1]) * ho2o6;
        }
      } else break;
    }
    int SourceSteps = step;
    // DoSourceIntegration, flat: llmax
    int llmax = nint(q * T->DMt0);
    if (llmax < 15) llmax = 17;
    else llmax = nint(q * (T->tau0 + 6 * 3.14159265358979323846 / q));
    // DoFlatIntegration
    std::vector<double> left_weight(SourceSteps + 1);
    std::vector<int> bes_index(SourceSteps + 1);
    for (int j = 1; j <= SourceSteps; ++j) {
      double xx = std::fabs(q * (T->tau0 - T->tau_points[j - 1]));
      int bi = index_of(T->bess_x, T->num_xx, xx);
      if (bi < 1) bi = 1;
      if (bi > T->num_xx - 1) bi = T->num_xx - 1;
      bes_index[j] = bi;
      double x_hi = T->bess_x[bi], dx = x_hi - T->bess_x[bi - 1];
      left_weight[j] = (x_hi - xx) / dx;
    }
    double BessIntBoost = T->AccuracyBoost * T->BessIntBoost;
    for (int j = 1; j <= nl; ++j) {
      int l = T->ls[j - 1];
      if (l > llmax) break;
      double xlim = std::max(0.0, l - 4.2 * std::cbrt((double)l));
      double xlmax1 = 80 * l * BessIntBoost;
      double tmin = T->tau0 - xlmax1 / q;
      tmin = std::max(T->tau_points[1], tmin);
      double tmax = T->tau0 - xlim / q;
      if (tmax < T->tau_points[1]) break;
      double sums[3] = {0, 0, 0};
      const double* H = &T->bessel_horner[(size_t)(j - 1) * (T->num_xx - 1) * 4];
      int nstart = index_of(T->tau_points, ntau, tmin), nend = std::min(SourceSteps, index_of(T->tau_points, ntau, tmax));
      bool DoInt = true;
      if (nsrc > 2) {
        double qmax_int = std::max(850, l) * 3 * BessIntBoost / T->tau0 * 1.2;
        DoInt = q < qmax_int;
      }
      if (DoInt) {
        for (int n = nstart; n <= nend; ++n) {
          double a2 = left_weight[n];
          const double* c = &H[(size_t)(bes_index[n] - 1) * 4];
          double J_l = c[0] + a2 * (c[1] + a2 * (c[2] + a2 * c[3]));
          J_l = J_l * T->tau_dpoints[n - 1];
          for (int s_ = 0; s_ < nsrc; ++s_) sums[s_] += Src[(size_t)n * nsrc + s_] * J_l;
        }
      }
      if (nsrc > 2 && (!DoInt || l > 400 * std::sqrt(T->AccuracyBoost * T->LimberBoost))) {
        double xf = T->tau0 - (l + 0.5) / q;
        if (xf < T->tau_points[ntau - 1] && xf > T->tau_points[0]) {
          int n = index_of(T->tau_points, ntau, xf);
          double f = (xf - T->tau_points[n - 1]) / (T->tau_points[n] - T->tau_points[n - 1]);
          sums[2] = (Src[(size_t)n * nsrc + 2] * (1 - f) + f * Src[(size_t)(n + 1) * nsrc + 2]) *
                    std::sqrt(3.14159265358979323846 / 2 / (l + 0.5)) / q;
        } else sums[2] = 0;
      }
      for (int s_ = 0; s_ < nsrc; ++s_) Delta[((size_t)q_ix * nl + (j - 1)) * nsrc + s_] += sums[s_];
    }
  }
  return 0;
}

// CalcScalCls (cmbmain.f90:3179-3343), flat
int oracle_calc_scal_cls(const CambGpuTables* T, const double* Delta, double* iCl) {
  int nq = T->nq, nl = T->nl, nsrc = T->nsrc;
  std::vector<double> dlnks(nq), pows(nq);
  for (int q_ix = 0; q_ix < nq; ++q_ix) {
    double k = T->q_int[q_ix];
    dlnks[q_ix] = T->dq_int[q_ix] / k;
    double lnrat = std::log(k / T->pivot_scalar);
    pows[q_ix] = T->As * std::exp(lnrat * (T->ns - 1 + lnrat * (T->nrun / 2)));
  }
  const double fourpi = 4 * 3.14159265358979323846, twopi = 2 * 3.14159265358979323846;
  for (int j = 0; j < nl; ++j) {
    double ell = T->ls[j];
    double c[6] = {0, 0, 0, 0, 0, 0};
    for (int q_ix = 0; q_ix < nq; ++q_ix) {
      const double* D = &Delta[((size_t)q_ix * nl + j) * nsrc];
      double dlnk = dlnks[q_ix], ap = pows[q_ix];
      c[0] += ap * D[0] * D[0] * dlnk;
      c[1] += ap * D[1] * D[1] * dlnk;
      c[2] += ap * D[0] * D[1] * dlnk;
      if (nsrc > 2) {
        c[3] += ap * D[2] * D[2] * dlnk;
        c[4] += ap * D[2] * D[0] * dlnk;
        c[5] += ap * D[2] * D[1] * dlnk;
      }
    }
    double ctnorm = (ell * ell - 1) * (ell + 2) * ell;
    double dbletmp = (ell * (ell + 1)) / twopi * fourpi;
    double* o = &iCl[(size_t)j * 6];
    o[0] = c[0] * dbletmp;
    o[1] = c[1] * dbletmp * ctnorm;
    o[2] = c[2] * dbletmp * std::sqrt(ctnorm);
    o[3] = o[4] = o[5] = 0;
    if (nsrc > 2) {
      o[3] = T->Alens * c[3] * fourpi * ell * ell * ell * ell;
      o[4] = std::sqrt(T->Alens) * c[4] * fourpi * ell * ell * ell;
      o[5] = std::sqrt(T->Alens) * c[5] * fourpi * ell * ell * ell * std::sqrt(ctnorm);
    }
  }
  return 0;
}

}  // extern "C"
