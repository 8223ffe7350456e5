// Per-k-mode Einstein-Boltzmann integrator for sm_103a (FP64): device code shared by the
// translation units that instantiate its kernels (ode_*.cu), so that they compile in parallel.
//
//
// One "team" of T lanes integrates one k-mode (T = 32 is one warp per mode).
// The mode's state vector uses a fixed per-mode layout
//     [etak, clxc, clxb, vb | T_0..T_lmaxg | E_0..E_lmaxgpol | N_0..N_lmaxnr]
// (photon temperature, photon E polarization, massless neutrinos) spread over
// the team's lanes entry-major: flat index i lives in lane i % T, register
// entry i / T.  The approximation switches of the reference only change which
// entries are active (tight coupling, k*tau neutrino truncation, late-time
// radiation truncation), so no repacking is ever needed.  All Dormand-Prince
// stage vectors stay in registers; the error norm and max|y| are team
// shuffle max-reductions.  The scalar part of the right-hand side (thermal
// history lookup, background, constraints, tight-coupling slip) is computed
// redundantly by the team's lanes, the multipole recurrences one entry per lane.
//
// Follows: RungeKuttaDP45 (RungeKuttaDP45.f90:94-408), GaugeInterface_ScalEv /
// EvolveScal (equations.f90:212-460), initial (equations.f90:1891-2112),
// derivs + source output (equations.f90:2273-2949), Thermo_values and
// IonizationFunctionsAtTime (results.f90:1848-1880, 3069-3108) and the time loop
// of CalcScalarSources (cmbmain.f90:998-1074).  Every spin of the mode loop is
// bounded: a mode that exceeds its derivative-evaluation budget or whose step
// size underflows stores CAMBGPU_ERROR_EVOLUTION in its cosmology's status word.
#pragma once
#include <cuda_runtime.h>

#include "device_tables.cuh"

namespace cgdev {

constexpr int NVAR_MAX = 128;
constexpr long long kMaxEvalsPerMode = 2000000LL;

template <int T>
struct Team {
  unsigned mask;
  int t;
  __device__ __forceinline__ Team() {
    int lane = threadIdx.x & 31;
    t = lane & (T - 1);
    if constexpr (T == 32) mask = 0xffffffffu;
    else mask = ((1u << T) - 1u) << (lane & ~(T - 1));
  }
  __device__ __forceinline__ double bcast(double v, int src) const {
    if constexpr (T == 1) return v;
    else return __shfl_sync(mask, v, src, T);
  }
  __device__ __forceinline__ int bcast_i(int v, int src) const {
    if constexpr (T == 1) return v;
    else return __shfl_sync(mask, v, src, T);
  }
  __device__ __forceinline__ double maxr(double v) const {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(mask, v, o, T));
    return v;
  }
};

// Uniform (team-wide) per-mode control state.
struct Mode {
  double k, ik, k2, ik2, q;
  double denlk1, denlk2_1, denlk_2, denlk2_2, poltruncfac;
  double pig, pigdot, tight_off;
  int lmaxg, lmaxgpol, lmaxnr, g_ix, pol_ix, r_ix, nvar;
  bool tc, hk, nonu, nophot;
};

// special entries whose derivative comes from the scalar part
enum { SP_ETAK = 0, SP_CLXC, SP_CLXB, SP_VB, SP_CLXG, SP_QG, SP_PIG, SP_E2, SP_CLXR, SP_QR, SP_PIR, SP_NONE = 15 };

template <int T>
struct Lanes {
  static constexpr int E = NVAR_MAX / T;
  double A[E], B[E], cOp[E], cCo[E];
  unsigned char sp[E];
  unsigned act;  // bit e: entry e active
};

struct Scal {  // scalar outputs of one right-hand-side evaluation
  double S[11];
};

struct SrcOut {
  double s[3];
};

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

// Thermo_values (results.f90:1848-1880)
// Position of tau on the thermal-history grid, 1 + ln(tau/tau_min)/dln(tau): an FP32
// estimate picks a grid point j, then ln(tau/tau_j) = ln(1 + u) with |u| <= dln(tau) (a few
// 1e-3) is a six-term series in FP64 -- no FP64 log on the FP64 pipe.
__device__ __forceinline__ double thermo_index(const DevCosmo& C, double tau) {
  const float df = __log2f((float)(tau * C.inv_tauminn)) * C.dlntau_inv_log2;
  int j = (int)df;
  j = j < 0 ? 0 : (j > C.nthermo ? C.nthermo : j);
  const double u = fma(tau, C.inv_tgrid[j], -1.0);
  const double l1p = u * (1.0 + u * (-0.5 + u * (1.0 / 3.0 + u * (-0.25 + u * (0.2 - u * (1.0 / 6.0))))));
  return (double)j + l1p * C.dlntau_inv + 1.0;
}

__device__ __forceinline__ void thermo_values(const DevCosmo& C, double tau, double itau, double& a, double& cs2,
                                              double& opac, double& dopac, bool want_dop = true) {
  double d = thermo_index(C, tau);
  int i = (int)d;
  d = d - i;
  if (i < 1) {  // before the table start (never reached: every mode starts after tauminn)
    i = 1;
    d = 0;
  }
  if (i >= C.nthermo) {
    cs2 = C.cs2_end;
    opac = C.dotmu_end;
    a = 1;
    dopac = C.ddotmu_end * itau * C.dlntau_inv;
  } else {
    const double* h = C.thermo_horner + (size_t)(i - 1) * 16;
    cs2 = ldg(h + 0) + d * (ldg(h + 1) + d * (ldg(h + 2) + d * ldg(h + 3)));
    opac = ldg(h + 4) + d * (ldg(h + 5) + d * (ldg(h + 6) + d * ldg(h + 7)));
    a = (ldg(h + 8) + d * (ldg(h + 9) + d * (ldg(h + 10) + d * ldg(h + 11)))) * tau;
    if (want_dop) dopac = (ldg(h + 12) + d * (ldg(h + 13) + d * (ldg(h + 14) + d * ldg(h + 15)))) * itau * C.dlntau_inv;
  }
}

// IonizationFunctionsAtTime (results.f90:3069-3108): visibility and derivatives
__device__ __forceinline__ void ionization(const DevCosmo& C, double tau, double itau, double& opac, double& dopac,
                                           double& vis, double& dvis, double& ddvis, double& expmmu) {
  double a, cs2;
  thermo_values(C, tau, itau, a, cs2, opac, dopac);
  double d = thermo_index(C, tau);
  int i = (int)d;
  d = d - i;
  if (i < 1) {
    i = 1;
    d = 0;
  }
  double ddopac;
  double tdl = tau * C.dlntau;
  if (i < C.nthermo) {
    int j = i - 1;
    double f3a = ldg(C.dddotmu + j), f3b = ldg(C.dddotmu + j + 1);
    double f4a = ldg(C.ddddotmu + j), f4b = ldg(C.ddddotmu + j + 1);
    double ema = ldg(C.emmu + j), emb = ldg(C.emmu + j + 1);
    double dea = ldg(C.demmu + j), deb = ldg(C.demmu + j + 1);
    ddopac = (f3a + d * (f4a + d * (3.0 * (f3b - f3a) - 2.0 * f4a - f4b + d * (f4a + f4b + 2.0 * (f3a - f3b)))) -
              (C.dlntau * C.dlntau) * tau * dopac) /
             (tdl * tdl);
    expmmu = ema + d * (dea + d * (3.0 * (emb - ema) - 2.0 * dea - deb + d * (dea + deb + 2.0 * (ema - emb))));
  } else {
    ddopac = (C.dddotmu_end - (C.dlntau * C.dlntau) * tau * dopac) / (tdl * tdl);
    expmmu = C.emmu_end;
  }
  vis = opac * expmmu;
  dvis = expmmu * (opac * opac + dopac);
  ddvis = expmmu * (opac * opac * opac + 3 * opac * dopac + ddopac);
}

template <int T>
__device__ __forceinline__ double sel(const double (&v)[NVAR_MAX / T], int e) {
  constexpr int E = NVAR_MAX / T;
  double r = v[0];
#pragma unroll
  for (int j = 1; j < E; ++j)
    if (e == j) r = v[j];
  return r;
}

// value of flat variable idx (uniform across the team)
template <int T>
__device__ __forceinline__ double getv(const Team<T>& tm, const double (&v)[NVAR_MAX / T], int idx) {
  return tm.bcast(sel<T>(v, idx / T), idx % T);
}

// Per-entry recurrence coefficients for the mode layout (denlk, denlk2, polfack of
// initial(), equations.f90:1911-1916, flat: Kf = 1).
template <int T>
__device__ void setup_layout(const Mode& M, const Team<T>& tm, Lanes<T>& L) {
  constexpr int E = NVAR_MAX / T;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    int i = e * T + tm.t;
    double A = 0, B = 0, cop = 0, cco = 0;
    int sp = SP_NONE;
    double k = M.k;
    if (i < 4) sp = SP_ETAK + i;
    else if (i < M.pol_ix) {  // photon temperature l
      int l = i - M.g_ix;
      double dl = 1.0 / (2 * l + 1);
      if (l == 0) sp = SP_CLXG;
      else if (l == 1) sp = SP_QG;
      else if (l == 2) sp = SP_PIG;
      else if (l < M.lmaxg) { A = dl * k * l; B = -(dl * k * (l + 1)); cop = 1; }
      else { A = k; cop = 1; cco = M.lmaxg + 1; }
    } else if (i < M.r_ix) {  // photon E polarization l
      int l = i - M.pol_ix;
      double dl = 1.0 / (2 * l + 1);
      if (l == 2) sp = SP_E2;
      else if (l >= 3 && l < M.lmaxgpol) {
        double polfac = (double)((l + 3) * (l - 1)) / (l + 1);
        A = dl * k * l;
        B = -(polfac * k * dl);
        cop = 1;
      } else if (l == M.lmaxgpol) { A = k * M.poltruncfac; cop = 1; cco = M.lmaxgpol + 3; }
    } else if (i < M.nvar) {  // massless neutrinos l
      int l = i - M.r_ix;
      double dl = 1.0 / (2 * l + 1);
      if (l == 0) sp = SP_CLXR;
      else if (l == 1) sp = SP_QR;
      else if (l == 2) sp = SP_PIR;
      else if (l < M.lmaxnr) { A = dl * k * l; B = -(dl * k * (l + 1)); }
      else { A = k; cco = M.lmaxnr + 1; }
    }
    L.A[e] = A;
    L.B[e] = B;
    L.cOp[e] = cop;
    L.cCo[e] = cco;
    L.sp[e] = (unsigned char)sp;
  }
}

// Which entries are propagated (SetupScalarArrayIndices, equations.f90:585-701)
template <int T>
__device__ void update_activity(const Mode& M, const Team<T>& tm, Lanes<T>& L) {
  constexpr int E = NVAR_MAX / T;
  unsigned act = 0;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    int i = e * T + tm.t;
    bool a = false;
    if (i < 4) a = true;
    else if (i < M.pol_ix) { int l = i - M.g_ix; a = !M.nophot && (l <= 1 || !M.tc); }
    else if (i < M.r_ix) { int l = i - M.pol_ix; a = !M.nophot && !M.tc && l >= 2; }
    else if (i < M.nvar) { int l = i - M.r_ix; a = !M.nonu && (l <= 2 || !M.hk); }
    if (a) act |= 1u << e;
  }
  L.act = act;
}

// Right-hand side (derivs, equations.f90:2273-2773) for the flat, Lambda,
// massless-neutrino adiabatic case; with `src` also the CMB sources of
// equations.f90:2775-2912.
template <int T, bool WITH_SRC>
__device__ __forceinline__ void derivs(const DevCosmo& C, Mode& M, const Team<T>& tm, const Lanes<T>& L,
                                       double tau, const double (&y)[NVAR_MAX / T], double (&dy)[NVAR_MAX / T],
                                       SrcOut* so) {
  constexpr int E = NVAR_MAX / T;
  const double k = M.k, ik = M.ik;
  double itau = 1.0 / tau;
  double a, cs2, opac, dopac;
  thermo_values(C, tau, itau, a, cs2, opac, dopac);
  double a2 = a * a, ia = 1.0 / a, ia2 = ia * ia;
  double etak = getv<T>(tm, y, 0), clxc = getv<T>(tm, y, 1), clxb = getv<T>(tm, y, 2), vb = getv<T>(tm, y, 3);
  double grhob_t = C.grhob * ia, grhoc_t = C.grhoc * ia, grhor_t = C.grhornomass * ia2, grhog_t = C.grhog * ia2;
  double grhov_t = C.grhov * a2;
  double dgrho = grhob_t * clxb + grhoc_t * clxc;
  double dgq = grhob_t * vb;
  double grho = (grhob_t + grhoc_t) + grhor_t + grhog_t + grhov_t;
  double gpres_noDE = (grhor_t + grhog_t) / 3;
  double adotoa = sqrt(grho / 3);
  double iad = 1.0 / adotoa;
  double z = 0, dz = 0, clxr, qr, pir, N3 = 0, clxg, qg, pig = 0, T3 = 0, E2 = 0, E3 = 0;
  if (M.nonu) {
    z = (0.5 * dgrho * ik + etak) * iad;
    dz = -adotoa * z - 0.5 * dgrho * ik;
    clxr = -4 * dz * ik;
    qr = -4.0 / 3 * z;
    pir = 0;
  } else {
    clxr = getv<T>(tm, y, M.r_ix);
    qr = getv<T>(tm, y, M.r_ix + 1);
    pir = getv<T>(tm, y, M.r_ix + 2);
    if (!M.hk) N3 = getv<T>(tm, y, M.r_ix + 3);
  }
  if (M.nophot) {
    if (!M.nonu) {
      z = (0.5 * dgrho * ik + etak) * iad;
      dz = -adotoa * z - 0.5 * dgrho * ik;
      clxg = -4 * dz * ik - 4 * ik * opac * (vb + z);
      qg = -4.0 / 3 * z;
    } else {
      clxg = clxr - 4 * ik * opac * (vb + z);
      qg = qr;
    }
  } else {
    clxg = getv<T>(tm, y, M.g_ix);
    qg = getv<T>(tm, y, M.g_ix + 1);
    if (!M.tc) {
      pig = getv<T>(tm, y, M.g_ix + 2);
      T3 = getv<T>(tm, y, M.g_ix + 3);
      E2 = getv<T>(tm, y, M.pol_ix + 2);
      E3 = getv<T>(tm, y, M.pol_ix + 3);
    }
  }
  dgrho = dgrho + grhog_t * clxg + grhor_t * clxr;
  dgq = dgq + grhog_t * qg + grhor_t * qr;
  double photbar = C.photbar_a * ia;
  double pb43 = 4.0 / 3 * photbar;
  z = (0.5 * dgrho * ik + etak) * iad;
  double sigma = z + 1.5 * dgq * M.ik2;
  Scal sc;
  sc.S[SP_ETAK] = 0.5 * dgq;
  sc.S[SP_CLXC] = -k * z;
  double clxbdot = -k * (z + vb);
  sc.S[SP_CLXB] = clxbdot;
  double clxgdot = -k * (4.0 / 3.0 * z + qg);
  double delta_p_b = cs2 * clxb;
  double vbdot, pigdot = 0;
  if (M.tc) {
    double gpres = gpres_noDE - grhov_t;
    double adotdota = (adotoa * adotoa - gpres) / 2;
    double iop = 1.0 / opac, iop2 = iop * iop;
    double i1pb = 1.0 / (1 + pb43);
    pig = 32.0 / 45 * iop * k * (sigma + vb);
    double slip = -(2 * adotoa * i1pb + dopac * iop) * (vb - 3.0 / 4 * qg) +
                  (-adotdota * vb - k / 2 * adotoa * clxg + k * (cs2 * clxbdot - clxgdot / 4)) * iop * i1pb;
    double dgs = grhog_t * pig + grhor_t * pir;
    double sigmadot = -2 * adotoa * sigma - dgs * ik + etak;
    double qgdot_tc = k * (clxg / 4.0 - pig / 2.0) + opac * slip;
    double f11 = dopac * 11.0 / 6.0 * iop2;
    pig = 32.0 / 45 * iop * k * (sigma + 3.0 * qg / 4.0) * (1 + f11) +
          (32.0 / 45.0 * iop2) * k * (sigmadot + 3.0 * qgdot_tc / 4.0) * (-11.0 / 6.0);
    pigdot = -(32.0 / 45.0) * (dopac * iop2) * k * (sigma + 3.0 * qg / 4.0) * (1 + f11) +
             (32.0 / 45.0 * iop) * k * (sigmadot + 3.0 * qgdot_tc / 4.0) * (1 + (11.0 / 6.0) * (dopac * iop2));
    M.pigdot = pigdot;
    vbdot = (-adotoa * vb + cs2 * k * clxb + k / 4 * pb43 * (clxg - 2 * pig)) * i1pb;
    vbdot = vbdot + pb43 * i1pb * slip;
    M.pig = pig;
  } else {
    vbdot = -adotoa * vb + k * delta_p_b - photbar * opac * (4.0 / 3 * vb - qg);
  }
  sc.S[SP_VB] = vbdot;
  double qgdot = 0, polter = 0;
  if (!M.nophot) {
    sc.S[SP_CLXG] = clxgdot;
    double inv_pb43 = 0.75 * a / C.photbar_a;
    qgdot = 4.0 / 3 * (-vbdot - adotoa * vb + delta_p_b * k) * inv_pb43 + M.denlk1 * clxg - M.denlk2_1 * pig;
    sc.S[SP_QG] = qgdot;
    if (!M.tc) {
      polter = pig / 10 + 9.0 / 15 * E2;
      pigdot = M.denlk_2 * qg - M.denlk2_2 * T3 - opac * (pig - polter) + 8.0 / 15.0 * k * sigma;
      sc.S[SP_PIG] = pigdot;
      sc.S[SP_E2] = -opac * (E2 - polter) - k / 3.0 * E3;
    } else {
      sc.S[SP_PIG] = 0;
      sc.S[SP_E2] = 0;
    }
  } else {
    sc.S[SP_CLXG] = sc.S[SP_QG] = sc.S[SP_PIG] = sc.S[SP_E2] = 0;
  }
  double clxrdot = 0, qrdot = 0, pirdot = 0;
  if (!M.nonu) {
    clxrdot = -k * (4.0 / 3.0 * z + qr);
    qrdot = M.denlk1 * clxr - M.denlk2_1 * pir;
    if (M.hk) pirdot = -3 * pir * itau - clxrdot;
    else pirdot = M.denlk_2 * qr - M.denlk2_2 * N3 + 8.0 / 15.0 * k * sigma;
  }
  sc.S[SP_CLXR] = clxrdot;
  sc.S[SP_QR] = qrdot;
  sc.S[SP_PIR] = pirdot;

  // multipole recurrences: d = A*prev + B*next - (cOp*opacity + cCo/tau)*y
  // entries beyond the mode's layout are never active (and skipped below)
  const int eact = (M.nvar + T - 1) / T;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    if (e < eact) {
      double prev, next;
      if constexpr (T == 1) {
        prev = e > 0 ? y[e - 1] : 0.0;
        next = e + 1 < E ? y[e + 1] : 0.0;
      } else {
        double up = __shfl_up_sync(tm.mask, y[e], 1, T);
        double wrapu = __shfl_sync(tm.mask, e > 0 ? y[e > 0 ? e - 1 : 0] : 0.0, T - 1, T);
        prev = tm.t == 0 ? wrapu : up;
        double dn = __shfl_down_sync(tm.mask, y[e], 1, T);
        double wrapd = __shfl_sync(tm.mask, e + 1 < E ? y[e + 1 < E ? e + 1 : e] : 0.0, 0, T);
        next = tm.t == T - 1 ? wrapd : dn;
      }
      double d = L.A[e] * prev + L.B[e] * next - (L.cOp[e] * opac + L.cCo[e] * itau) * y[e];
      int sp = L.sp[e];
      double s = 0;
#pragma unroll
      for (int j = 0; j < 11; ++j)
        if (sp == j) s = sc.S[j];
      d += s;
      dy[e] = ((L.act >> e) & 1u) ? d : 0.0;
    } else {
      dy[e] = 0.0;
    }
  }

  if constexpr (WITH_SRC) {
    // CMB source functions (equations.f90:2775-2912), flat Kf = 1
    double Ed2 = 0, Ed3 = 0, octgdot = 0;
    if (M.nophot) {
      pigdot = 0;
      octgdot = 0;
      qgdot = -4 * dz / 3;
      E2 = E3 = 0;
    } else if (M.tc) {
      double iop = 1.0 / opac;
      E2 = pig / 4 + pigdot * iop * (-5.0 / 8.0);
      E3 = (3.0 / 7.0) * (k * iop) * E2;
      Ed2 = (pigdot / 4.0) * (1 + (5.0 / 2.0) * (dopac * iop * iop));
      Ed3 = 0;
      octgdot = 0;
    } else {
      Ed2 = sc.S[SP_E2];
      Ed3 = getv<T>(tm, dy, M.pol_ix + 3);
      octgdot = getv<T>(tm, dy, M.g_ix + 3);
    }
    if (M.nonu) pirdot = 0;
    double dgpi = grhor_t * pir + grhog_t * pig;
    double pidot_sum = grhog_t * pigdot + grhor_t * pirdot;
    double gpres = gpres_noDE - grhov_t;
    double diff_rhopi = pidot_sum - (4 * dgpi) * adotoa;
    double phi = -((dgrho + 3 * dgq * adotoa * ik) + dgpi) / (2 * M.k2);
    double op2, dop2, vis, dvis, ddvis, exptau;
    ionization(C, tau, itau, op2, dop2, vis, dvis, ddvis, exptau);
    double k2 = M.k2;
    double phidot = 0.5 * (adotoa * (-dgpi - 2 * k2 * phi) + dgq * k - diff_rhopi + k * sigma * (gpres + grho)) * M.ik2;
    double sigmadot = -adotoa * sigma - 0.5 * dgpi * ik + k * phi;
    polter = pig / 10 + 9.0 / 15 * E2;
    double polterdot = (1.0 / 10.0) * pigdot + (3.0 / 5.0) * Ed2;
    double polterddot = -2.0 / 25.0 * adotoa * dgq * ik - 4.0 / 75.0 * adotoa * k * sigma - 4.0 / 75.0 * dgpi -
                        2.0 / 75.0 * dgrho - 3.0 / 50.0 * k * octgdot + (1.0 / 25.0) * k * qgdot - 1.0 / 5.0 * k * Ed3 +
                        (-1.0 / 10.0 * pig + (7.0 / 10.0) * polter - 3.0 / 5.0 * E2) * dop2 +
                        (-1.0 / 10.0 * pigdot + (7.0 / 10.0) * polterdot - 3.0 / 5.0 * Ed2) * op2;
    double ISW = 2 * phidot * exptau;
    double monopole_source = (-etak * ik + 2 * phi + clxg / 4) * vis;
    double doppler = ((sigma + vb) * dvis + (sigmadot + vbdot) * vis) * ik;
    double quadrupole_source =
        (5.0 / 8.0) * (3 * polter * ddvis + 6 * polterdot * dvis + (k2 * polter + 3 * polterddot) * vis) * M.ik2;
    so->s[0] = ISW + doppler + monopole_source + quadrupole_source;
    double ang = C.tau0 - tau;
    so->s[1] = tau < C.tau0 ? vis * polter * (15.0 / 8.0) / (ang * ang * k2) : 0.0;
    so->s[2] = 0;
    if (C.nsrc > 2 && tau > C.tau_maxvis && ang > 0.1)
      so->s[2] = -2 * phi * (tau - C.tau_maxvis) / ((C.tau0 - C.tau_maxvis) * ang);
  }
}

// Dormand-Prince 5(4) tableau (RungeKuttaDP45.f90:108-133)
namespace dp {
constexpr double a21 = 1.0 / 5.0, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0, a41 = 44.0 / 45.0, a42 = -56.0 / 15.0,
                 a43 = 32.0 / 9.0, a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0,
                 a54 = -212.0 / 729.0, a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0,
                 a64 = 49.0 / 176.0, a65 = -5103.0 / 18656.0, b1 = 35.0 / 384.0, b3 = 500.0 / 1113.0,
                 b4 = 125.0 / 192.0, b5 = -2187.0 / 6784.0, b6 = 11.0 / 84.0, e1 = 71.0 / 57600.0,
                 e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0, e6 = 22.0 / 525.0,
                 e7 = -1.0 / 40.0;
constexpr double eps = 2.220446049250313e-16, tiny = 2.2250738585072014e-308;
}  // namespace dp

// Persistent step-control state (RungeKuttaDP45Settings fields that survive calls)
struct RK {
  double h, err, ms_user;
  int fails;
  bool fsal;   // first_derivative_valid
  bool reset;  // ind == 1 on the next call
  long long evals;
};

template <int T>
struct Regs {
  static constexpr int E = NVAR_MAX / T;
  double y[E], k1[E], k2[E], k3[E], k4[E], k5[E], k6[E], yt[E];
};

// one call of RungeKuttaDP45 from x to xend (ind = 1 or 3 on entry)
template <int T>
__device__ int dp45(const DevCosmo& C, Mode& M, const Team<T>& tm, const Lanes<T>& L, Regs<T>& R, RK& rk,
                    double& x, double xend, double tol) {
  constexpr int E = NVAR_MAX / T;
  using namespace dp;
  bool first = rk.reset;
  double hmax_user = rk.reset ? 0.0 : rk.ms_user;  // settings reset wipes max_step_size
  if (rk.reset) {
    rk.fsal = false;
    rk.fails = 0;
    rk.reset = false;
  }
  SrcOut dummy;
  bool need_f = true;
  const double g1 = 2.0 / 0.9, g2 = g1 * g1;
  const double grow_lim = g2 * g2 * g1;  // (2/0.9)**5
  for (;;) {
    if (rk.evals > kMaxEvalsPerMode) return -1;
    if (need_f) {
      if (rk.fsal) rk.fsal = false;
      else {
        derivs<T, false>(C, M, tm, L, x, R.y, R.k1, &dummy);
        rk.evals++;
      }
    }
    need_f = false;
    double ny = 0;
#pragma unroll
    for (int e = 0; e < E; ++e)
      if ((L.act >> e) & 1u) ny = fmax(ny, fabs(R.y[e]));
    ny = fmin(tm.maxr(ny), 1.0);
    double hmin = 10.0 * fmax(tiny, eps * fmax(ny / tol, fabs(x)));
    double hmax = hmax_user != 0.0 ? hmax_user : 20.0;
    if (hmin > hmax) return -2;
    if (first) {
      rk.h = hmax * pow(tol, 0.2);
      first = false;
    } else if (rk.fails <= 1) {
      double t2 = 2.0 * rk.h;
      if (tol < grow_lim * rk.err) t2 = 0.9 * pow(tol / rk.err, 0.2) * rk.h;
      rk.h = fmax(t2, 0.5 * rk.h);
    } else {
      rk.h = 0.5 * rk.h;
    }
    rk.h = fmin(rk.h, hmax);
    rk.h = fmax(rk.h, hmin);
    double rem = fabs(xend - x), xt;
    if (rk.h < rem && (rem > 1.2 * rk.h || rem > hmax)) {
      rk.h = fmin(rk.h, 0.5 * rem);
      xt = x + copysign(rk.h, xend - x);
    } else {
      rk.h = rem;
      xt = xend;
    }
    const double hs = xt - x;
#pragma unroll
    for (int e = 0; e < E; ++e) R.yt[e] = R.y[e] + hs * a21 * R.k1[e];
    derivs<T, false>(C, M, tm, L, x + hs / 5.0, R.yt, R.k2, &dummy);
#pragma unroll
    for (int e = 0; e < E; ++e) R.yt[e] = R.y[e] + hs * (a31 * R.k1[e] + a32 * R.k2[e]);
    derivs<T, false>(C, M, tm, L, x + hs * (3.0 / 10.0), R.yt, R.k3, &dummy);
#pragma unroll
    for (int e = 0; e < E; ++e) R.yt[e] = R.y[e] + hs * (a41 * R.k1[e] + a42 * R.k2[e] + a43 * R.k3[e]);
    derivs<T, false>(C, M, tm, L, x + hs * (4.0 / 5.0), R.yt, R.k4, &dummy);
#pragma unroll
    for (int e = 0; e < E; ++e)
      R.yt[e] = R.y[e] + hs * (a51 * R.k1[e] + a52 * R.k2[e] + a53 * R.k3[e] + a54 * R.k4[e]);
    derivs<T, false>(C, M, tm, L, x + hs * (8.0 / 9.0), R.yt, R.k5, &dummy);
#pragma unroll
    for (int e = 0; e < E; ++e)
      R.yt[e] = R.y[e] + hs * (a61 * R.k1[e] + a62 * R.k2[e] + a63 * R.k3[e] + a64 * R.k4[e] + a65 * R.k5[e]);
    derivs<T, false>(C, M, tm, L, x + hs, R.yt, R.k6, &dummy);
#pragma unroll
    for (int e = 0; e < E; ++e)
      R.yt[e] = R.y[e] + hs * (b1 * R.k1[e] + b3 * R.k3[e] + b4 * R.k4[e] + b5 * R.k5[e] + b6 * R.k6[e]);
    // stage 7 (FSAL) into k2's registers
    derivs<T, false>(C, M, tm, L, x + hs, R.yt, R.k2, &dummy);
    rk.evals += 6;
    double m = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if ((L.act >> e) & 1u) {
        double ee = e1 * R.k1[e] + e3 * R.k3[e] + e4 * R.k4[e] + e5 * R.k5[e] + e6 * R.k6[e] + e7 * R.k2[e];
        m = fmax(m, fabs(ee) / fmax(1.0, fabs(R.y[e])));
      }
    }
    m = tm.maxr(m);
    rk.err = m * rk.h;
    if (rk.err <= tol) {
      x = xt;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        R.y[e] = R.yt[e];
        R.k1[e] = R.k2[e];
      }
      rk.fails = 0;
      if (x == xend) {
        rk.fsal = true;  // reuse_first_derivative: stage 7 seeds the next call
        return 0;
      }
    } else {
      rk.fails++;
      if (rk.h <= hmin) return -3;
    }
  }
}

// set one flat variable (uniform idx) to v
template <int T>
__device__ __forceinline__ void setv(const Team<T>& tm, double (&v)[NVAR_MAX / T], int idx, double val) {
  constexpr int E = NVAR_MAX / T;
  int e = idx / T;
  if (tm.t == idx % T) {
#pragma unroll
    for (int j = 0; j < E; ++j)
      if (j == e) v[j] = val;
  }
}

template <int T>
__device__ __forceinline__ void zero_inactive(const Lanes<T>& L, double (&v)[NVAR_MAX / T]) {
  constexpr int E = NVAR_MAX / T;
#pragma unroll
  for (int e = 0; e < E; ++e)
    if (!((L.act >> e) & 1u)) v[e] = 0.0;
}

// GaugeInterface_ScalEv (equations.f90:212-234)
template <int T>
__device__ int scal_ev(const DevCosmo& C, Mode& M, const Team<T>& tm, const Lanes<T>& L, Regs<T>& R, RK& rk,
                       double& tau, double tauend) {
  if (M.q < 2e-3 && tau <= C.taurend) rk.ms_user = 2.0;
  else rk.ms_user = 20.0 / C.IntTolBoost;
  return dp45<T>(C, M, tm, L, R, rk, tau, tauend, C.tol1);
}

// GaugeInterface_EvolveScal (equations.f90:261-460), switches as a loop
template <int T>
__device__ int evolve_scal(const DevCosmo& C, Mode& M, const Team<T>& tm, Lanes<T>& L, Regs<T>& R, RK& rk,
                           double& tau, double tauend) {
  for (int guard = 0; guard < 16; ++guard) {
    double noSwitch = C.tau0 + 1;
    double smallTime = fmin(tau, M.ik) / 100;
    double switchBoost = C.AccuracyBoost * C.TimeSwitchBoost;
    double t_ktau = noSwitch, t_nonu = noSwitch, t_nophot = noSwitch;
    if (!M.hk && !M.nonu) t_ktau = (double)max(20, M.lmaxnr - 4) / M.k;
    if (!M.nonu) t_nonu = fmax(15 / M.k * switchBoost, fmin(C.taurend, C.matter_verydom_tau));
    if (!M.nophot && M.k > 0.03 * switchBoost) t_nophot = fmax(15 / M.k, C.taurend) * switchBoost;
    double next = fmin(fmin(t_ktau, M.tight_off), fmin(fmin(t_nonu, t_nophot), noSwitch));
    if (!(next < tauend)) return scal_ev<T>(C, M, tm, L, R, rk, tau, tauend);
    if (next > tau + smallTime) {
      int rc = scal_ev<T>(C, M, tm, L, R, rk, tau, next);
      if (rc) return rc;
    }
    if (next == M.tight_off) {
      // leave tight coupling: seed pi_g, G_3, E_2, E_3 with the 2nd-order TC values
      M.tc = false;
      M.tight_off = noSwitch;
      rk.reset = true;
      update_activity<T>(M, tm, L);
      double itau = 1.0 / tau, a, cs2, opac, dopac;
      thermo_values(C, tau, itau, a, cs2, opac, dopac);
      double kb = M.k, op2 = opac * opac;
      double g2 = M.pig;
      double g3 = (3.0 / 7.0) * g2 * (kb / opac) * (1.0 + dopac / op2) + (3.0 / 7.0) * M.pigdot * (kb / op2) * (-1.0);
      double p2 = M.pig / 4 + M.pigdot * (1.0 / opac) * (-5.0 / 8.0 - (25.0 / 16.0) * dopac / op2) +
                  M.pig * (kb / opac) * (kb / opac) * (-5.0 / 56.0);
      double p3 = (3.0 / 7.0) * (kb / opac) * p2 * (1.0 + dopac / op2) +
                  (3.0 / 7.0) * (kb / op2) * ((M.pigdot / 4.0) * (1.0 + (5.0 / 2.0) * dopac / op2)) * (-1.0);
      zero_inactive<T>(L, R.y);
      setv<T>(tm, R.y, M.g_ix + 2, g2);
      setv<T>(tm, R.y, M.g_ix + 3, g3);
      setv<T>(tm, R.y, M.pol_ix + 2, p2);
      setv<T>(tm, R.y, M.pol_ix + 3, p3);
    } else if (next == t_ktau) {
      M.hk = true;
      update_activity<T>(M, tm, L);
      zero_inactive<T>(L, R.y);
    } else if (next == t_nonu) {
      rk.reset = true;
      M.nonu = true;
      update_activity<T>(M, tm, L);
      zero_inactive<T>(L, R.y);
    } else if (next == t_nophot) {
      rk.reset = true;
      M.nophot = true;
      update_activity<T>(M, tm, L);
      zero_inactive<T>(L, R.y);
    }
    rk.fsal = false;
  }
  return -4;
}

// initial (equations.f90:1891-2112), adiabatic mode, flat, massless neutrinos
template <int T>
__device__ void initial(const DevCosmo& C, const Mode& M, const Team<T>& tm, Regs<T>& R, double tau) {
  constexpr int E = NVAR_MAX / T;
#pragma unroll
  for (int e = 0; e < E; ++e) R.y[e] = 0;
  double k = M.k;
  double x = k * tau, x2 = x * x, x3 = x2 * x;
  double grhonu = C.grhornomass;
  double om = (C.grhob + C.grhoc) / sqrt(3 * (C.grhog + grhonu));
  double omtau = om * tau;
  double Rv = grhonu / (grhonu + C.grhog);
  double Rp15 = 4 * Rv + 15;
  double iv_clxg = -1.0 / 3 * x2 * (1 - omtau / 5);
  double iv_clxb = 0.75 * iv_clxg;
  double iv_qg = iv_clxg * x / 9.0;
  double iv_qr = -(4 * Rv + 23) / Rp15 * x3 / 27;
  double iv_vb = 0.75 * iv_qg;
  double iv_pir = 4.0 / 3 * x2 / Rp15 * (1 + omtau / 4 * (4 * Rv - 5) / (2 * Rv + 15));
  double iv_aj3r = 4 / 21.0 / Rp15 * x3;
  double iv_eta = -2 * (1 - x2 / 12 * (-10.0 / Rp15 + 1));
  setv<T>(tm, R.y, 0, iv_eta * k / 2);
  setv<T>(tm, R.y, 1, -iv_clxb);
  setv<T>(tm, R.y, 2, -iv_clxb);
  setv<T>(tm, R.y, 3, -iv_vb);
  setv<T>(tm, R.y, M.g_ix, -iv_clxg);
  setv<T>(tm, R.y, M.g_ix + 1, -iv_qg);
  setv<T>(tm, R.y, M.r_ix, -iv_clxg);
  setv<T>(tm, R.y, M.r_ix + 1, -iv_qr);
  setv<T>(tm, R.y, M.r_ix + 2, -iv_pir);
  if (M.lmaxnr > 2) setv<T>(tm, R.y, M.r_ix + 3, -iv_aj3r);
}

// CalcScalarSources (cmbmain.f90:998-1074) for one mode
template <int T>
__device__ void evolve_mode(const DevCosmo& C, int q_ix, const Team<T>& tm) {
  const CambGpuModeSpec ms = C.modes[q_ix];
  Mode M;
  M.q = ms.q;
  M.k = ms.q;
  M.ik = 1.0 / M.k;
  M.k2 = M.k * M.k;
  M.ik2 = 1.0 / M.k2;
  M.lmaxg = ms.lmaxg;
  M.lmaxgpol = ms.lmaxgpol;
  M.lmaxnr = ms.lmaxnr;
  M.g_ix = 4;
  M.pol_ix = M.g_ix + M.lmaxg + 1;
  M.r_ix = M.pol_ix + M.lmaxgpol + 1;
  M.nvar = M.r_ix + M.lmaxnr + 1;
  M.denlk1 = (1.0 / 3) * M.k;
  M.denlk2_1 = (1.0 / 3) * M.k * 2;
  M.denlk_2 = (1.0 / 5) * M.k * 2;
  M.denlk2_2 = (1.0 / 5) * M.k * 3;
  M.poltruncfac = (double)M.lmaxgpol / max(1, M.lmaxgpol - 2);
  M.pig = 0;
  M.pigdot = 0;
  M.tight_off = ms.tight_switch_tau;
  M.tc = true;
  M.hk = false;
  M.nonu = false;
  M.nophot = false;
  const int nsrc = C.nsrc, nk = C.nk;
  if (M.nvar > NVAR_MAX) {
    if (tm.t == 0) atomicExch(C.status, (int)CAMBGPU_ERROR_UNSUPPORTED_PARAMS);
    return;
  }
  Lanes<T> L;
  setup_layout<T>(M, tm, L);
  update_activity<T>(M, tm, L);
  Regs<T> R;
  initial<T>(C, M, tm, R, ms.taustart);
  double tau = ms.taustart;
  RK rk;
  rk.h = 0;
  rk.err = 0;
  rk.ms_user = 0;
  rk.fails = 0;
  rk.fsal = false;
  rk.reset = true;
  rk.evals = 0;
  double* out = C.linear_src;
  for (int j = 1; j < C.ntau; ++j) {
    double tauend = C.tau_points[j];
    if (M.q * tauend > C.max_etak_scalar && tauend > C.taurend && !C.want_late_time) {
      // rest of the sources stay zero (buffer cleared before launch)
      break;
    }
    int rc = evolve_scal<T>(C, M, tm, L, R, rk, tau, tauend);
    if (rc) {
      if (tm.t == 0) atomicExch(C.status, (int)CAMBGPU_ERROR_EVOLUTION);
      return;
    }
    constexpr int E = NVAR_MAX / T;
    double dy[E];
    SrcOut so;
    derivs<T, true>(C, M, tm, L, tau, R.y, dy, &so);
    rk.evals++;
    if (tm.t == 0) {
      for (int s = 0; s < nsrc; ++s) out[((size_t)j * nsrc + s) * nk + q_ix] = so.s[s];
    }
  }
  if (tm.t == 0) {
    atomicAdd(C.evals, (unsigned long long)rk.evals);
    if (C.mode_evals) C.mode_evals[q_ix] = (unsigned)rk.evals;
  }
}

template <int T>
__global__ void __launch_bounds__(128) ode_persistent_kernel(const DevCosmo* __restrict__ cosmos,
                                                             const WorkItem* __restrict__ items, int nitems,
                                                             int* __restrict__ counter) {
  Team<T> tm;
  for (;;) {
    int w = 0;
    if (tm.t == 0) w = atomicAdd(counter, 1);
    w = tm.bcast_i(w, 0);
    if (w >= nitems) break;
    WorkItem it = items[w];
    if (cosmos[it.cosmo].nu_eig > 0 || cosmos[it.cosmo].transfer_only) {  // massless CMB layout only
      if (tm.t == 0) atomicExch(cosmos[it.cosmo].status, (int)CAMBGPU_ERROR_UNSUPPORTED_PARAMS);
      continue;
    }
    evolve_mode<T>(cosmos[it.cosmo], it.mode, tm);
  }
}

// ---------------------------------------------------------------------------
// Thread-per-mode variant (team size 1).  On GB300 the FP64 pipe is the binding
// resource; the warp-per-mode kernel above evaluates the scalar part of every
// right-hand side on all 32 lanes.  Here one thread owns one k-mode: the state and
// Dormand-Prince stage vectors live in the thread's local memory (interleaved per
// warp, L1/L2 resident), and the per-thread loop is a flat state machine in which
// every iteration performs exactly one trial step, so threads of a warp never wait
// for one another's integration intervals.  Work items are handed out in order of
// decreasing q, so a warp integrates neighbouring k-modes whose switch times and
// step-size histories are close.
// ---------------------------------------------------------------------------
namespace tpm {

constexpr int NV = 448;  // largest packed scalar system handled (mode_init rejects larger ones)
// Dormand-Prince 5(4) with FSAL needs seven live rows per mode: y, the stage input, and
// k1..k5; k6 takes k2's row (k2 is dead once the stage-6 input is formed, b2 = e2 = 0) and
// k7 takes k4's (dead once the fifth-order solution and the error combination are formed).
constexpr int kRows = 7;
// Unroll of the multipole sweeps of the right-hand side and of the stage combinations.
// Measured on the 256-draw lmax-2500 batch (team 7, balanced queue): unrolled groups keep
// more row loads in flight, but the rows miss L1 and L2 and the wider bursts lose --
// 4 / 4 took 1266 ms, 8 / 4 1332, 8 / 8 1448, 2 / 4 1237, 2 / 1 1202 (stage / sweep).
#ifndef CG_RHS_UNROLL
#define CG_RHS_UNROLL 1
#endif
#ifndef CG_STAGE_UNROLL
#define CG_STAGE_UNROLL 2
#endif
constexpr int kRhsUnroll = CG_RHS_UNROLL;
constexpr int kStageUnroll = CG_STAGE_UNROLL;
constexpr int NL = 256;  // multipoles of any hierarchy: l < 256 (lAccuracyBoost up to ~3.9)
constexpr int NUE = 3;

// l-only factors of the multipole recurrences (initial(), equations.f90:1911-1916):
// denlk = k a_l, denlk2 = k b_l, polfack = k p_l with a_l = l/(2l+1), b_l = (l+1)/(2l+1),
// p_l = (l+3)(l-1)/((l+1)(2l+1)).  One table for every mode (k is applied in the
// recurrence), read with uniform addresses across a warp instead of per-thread copies.
struct RecTab {
  double a[NL], b[NL], p[NL];
};
constexpr RecTab make_rec_tab() {
  RecTab t{};
  for (int l = 0; l < NL; ++l) {
    t.a[l] = l / (2.0 * l + 1);
    t.b[l] = (l + 1) / (2.0 * l + 1);
    t.p[l] = l >= 1 ? ((double)((l + 3) * (l - 1)) / (l + 1)) / (2.0 * l + 1) : 0.0;
  }
  return t;
}
static __device__ const RecTab kRec = make_rec_tab();

// x**(1/5) for the step-size update: FP32 seed, two Newton steps on y^5 = x in FP64
__device__ __forceinline__ double fifth_root(double x) {
  if (!(x > 1e-300) || !(x < 1e300)) return pow(x, 0.2);
  double y = (double)exp2f(0.2f * log2f((float)x));
  double y4 = (y * y) * (y * y);
  y = 0.8 * y + 0.2 * x / y4;
  y4 = (y * y) * (y * y);
  y = 0.8 * y + 0.2 * x / y4;
  return y;
}

// Massive-neutrino background in units of one massless eigenstate, as a function of
// a*m/(k_B T_nu) (fits of massive_neutrinos.f90:186-216 and 325-347).
namespace nuf {
constexpr double zeta3 = 1.2020569031595942853997, zeta5 = 1.0369277551433699263313, zeta7 = 1.0083492773819228268397;
constexpr double pi = 3.1415926535897932384626433832795;
constexpr double fdc = 7.0 / 120 * pi * pi * pi * pi;
constexpr double const2 = 5.0 / 7.0 / (pi * pi);
__device__ __forceinline__ void rho_P(double am, double& rhonu, double& pnu) {
  const double amin = 0.42, amax = 70.0;
  if (am <= amin) {
    const double am2 = am * am, am4 = am2 * am2;
    rhonu = 1.0 + const2 * am2 + am4 * (-1.872929199948838302e-02 + am2 * 1.831728681837861694e-02);
    pnu = (1.0 - const2 * am2) / 3.0 + am4 * (1.667044572156534468e-02 + am2 * -2.277471498716537868e-02);
    return;
  }
  if (am >= amax) {
    rhonu = 3 / (2 * fdc) * (zeta3 * am + ((15 * zeta5) / 2 - 945.0 / 16 * zeta7 / (am * am)) / am);
    pnu = 900.0 / 120.0 / fdc * (zeta5 - 63.0 / 4 * zeta7 / (am * am)) / am;
    return;
  }
  const double fc = 5.422176684690383;   // sqrt(0.42 * 70)
  const double izm = (amax + fc) / (amax - fc);
  const double z = ((am - fc) / (am + fc)) * izm;
  const double rfit = (((((-2.544964203886362908e-03 * z + 2.123075360029347963e-02) * z - 8.378996019212282820e-02) * z +
                         1.545077526625578401e-01) * z + 1.188066888581748443e-01) * z + 7.499710425926954249e-01);
  const double pfit = ((((((-1.965863329520473827e-03 * z + 2.378742143669706002e-03) * z + 4.067958090718486880e-02) * z -
                          2.509793530357270000e-02) * z - 2.435843189264263742e-01) * z + 3.156134695375645838e-01) * z +
                       9.283417043601330798e-01);
  rhonu = (1.0 + 3.0 * zeta3 / (2.0 * fdc) * am) * rfit;
  pnu = pfit / (1.0 + fdc / ((900.0 / 120.0) * zeta5) * am);
}
__device__ __forceinline__ double drho(double am, double adotoa) {
  const double amin = 0.3, amax = 70.0;
  if (am <= amin) {
    const double am2 = am * am;
    return am2 * (2 * const2 + am2 * (.4399706676e-1 * log(am) - .2970400378e-2 - .29331377855e-1 * am)) * adotoa;
  }
  if (am >= amax) return 3 / (2 * fdc) * (zeta3 * am + (-(15 * zeta5) / 2 + 2835.0 / 16 * zeta7 / (am * am)) / am) * adotoa;
  const double fc = 4.58257569495584;  // sqrt(0.3 * 70)
  const double izm = (amax + fc) / (amax - fc);
  const double z = ((am - fc) / (am + fc)) * izm;
  const double D = (((((-3.877662402660121861e-03 * z + 1.056591590995091534e-02) * z + 3.167230341650149189e-02) * z -
                       1.602709049602861757e-01) * z + 1.801974470841860576e-01) * z + 5.800497880734221123e-01);
  return am * am / (1.0 + 2.0 * am) * D * adotoa;
}
}  // namespace nuf

// W = 1: one thread integrates one mode.  W = 32: the 32 lanes of a warp integrate one
// mode together -- every lane evaluates the scalar part of the equations (identical
// values, identical control flow), the multipole hierarchies, momentum bins and stage
// combinations are split across lanes, and the state rows live in shared memory.
template <int W>
__device__ __forceinline__ int wlane() {
  if constexpr (W == 1) return 0;
  else return threadIdx.x & 31;
}
template <int W>
__device__ __forceinline__ void wsync() {
  if constexpr (W > 1) __syncwarp();
}
// butterfly sum: every lane ends with the same bits (each level adds the same pair)
template <int W>
__device__ __forceinline__ double wsum(double v) {
  if constexpr (W > 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}
template <int W>
__device__ __forceinline__ double wmax(double v) {
  if constexpr (W > 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}
template <int W>
__device__ __forceinline__ unsigned long long wmax_u64(unsigned long long v) {
  if constexpr (W > 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
      v = t > v ? t : v;
    }
  }
  return v;
}

// per-mode control state (EvolutionVars, equations.f90:66-151), indices 0-based
struct St {
  double q, k, ik, k2, ik2;
  double pig, pigdot, tight_off, poltruncfac, kptf;
  int lmaxg, lmaxgpol, lmaxnr, lmaxnu, nvar, n;
  int g_ix, pol0, r_ix, nu_pert_ix, lmaxnu_pert;
  int nu_ix[NUE], nq[NUE], lmaxnu_tau[NUE];
  bool tc, hk, nonu, nophot, has_nu_rel;
  bool approx[NUE], nonrel[NUE];
  double approx_time[NUE], G11[NUE], G30[NUE], lboost[NUE];
  bool out_src;  // transfer path: the output evaluation forms the CMB sources, not outtransf's
};

// SetupScalarArrayIndices (equations.f90:585-701): the propagated variables are packed
// [etak clxc clxb vb | photon T | photon E (l>=2) | massless nu | nu perturbation | massive nu]
static __device__ void setup_indices(const DevCosmo& C, St& M, bool want_max) {
  int neq = 4;
  if (!M.nophot) {
    M.g_ix = 4;
    if (M.tc) neq += 2;
    else {
      neq += M.lmaxg + 1;
      M.pol0 = neq - 2;
      neq += M.lmaxgpol - 1;
    }
  }
  if (!M.nonu) {
    M.r_ix = neq;
    neq += M.hk ? 3 : M.lmaxnr + 1;
  }
  int maxeq = 4 + (M.lmaxg + 1) + (M.lmaxnr + 1) + M.lmaxgpol - 1;
  M.has_nu_rel = false;
  if (C.nu_eig > 0) {
    for (int i = 0; i < C.nu_eig; ++i) M.has_nu_rel |= M.nq[i] != C.nqmax;
    if (M.has_nu_rel) {
      M.lmaxnu_pert = M.lmaxnu;
      M.nu_pert_ix = neq;
      neq += M.lmaxnu_pert + 1;
      maxeq += M.lmaxnu_pert + 1;
    } else {
      M.lmaxnu_pert = 0;
    }
    for (int i = 0; i < C.nu_eig; ++i) {
      const double b = M.lboost[i];
      int lt;
      if (M.hk) lt = (int)(4 * b);
      else {
        lt = max(min((int)llrint(0.8 * M.q * C.nu_tau_nonrel[i] * b), M.lmaxnu), 3);
        if (M.nonrel[i]) lt = min(lt, (int)llrint(4 * b));
      }
      M.lmaxnu_tau[i] = min(M.lmaxnu, lt);
      M.nu_ix[i] = neq;
      neq += M.approx[i] ? 4 : M.nq[i] * (M.lmaxnu_tau[i] + 1);
      maxeq += C.nqmax * (M.lmaxnu + 1);
    }
  }
  M.n = neq;
  if (want_max) M.nvar = maxeq;
}

// CopyScalarVariableArray (equations.f90:703-791) from layout O to layout N
template <int W>
__device__ void copy_vars(const DevCosmo& C, const St& O, const St& N, const double* __restrict__ y,
                          double* __restrict__ yo) {
  for (int i = wlane<W>(); i < N.nvar; i += W) yo[i] = 0;
  wsync<W>();  // the copies below are made by every lane
  for (int i = 0; i < 4; ++i) yo[i] = y[i];
  if (!O.nophot && !N.nophot) {
    int lmax = (O.tc || N.tc) ? 1 : min(O.lmaxg, N.lmaxg);
    for (int l = 0; l <= lmax; ++l) yo[N.g_ix + l] = y[O.g_ix + l];
    if (!O.tc && !N.tc) {
      lmax = min(O.lmaxgpol, N.lmaxgpol);
      for (int l = 2; l <= lmax; ++l) yo[N.pol0 + l] = y[O.pol0 + l];
    }
  }
  if (!O.nonu && !N.nonu) {
    const int lmax = (O.hk || N.hk) ? 2 : min(O.lmaxnr, N.lmaxnr);
    for (int l = 0; l <= lmax; ++l) yo[N.r_ix + l] = y[O.r_ix + l];
  }
  for (int i = 0; i < C.nu_eig; ++i) {
    const int off = O.nu_ix[i], off2 = N.nu_ix[i];
    if (O.approx[i] && N.approx[i]) {
      for (int j = 0; j < 4; ++j) yo[off2 + j] = y[off + j];
    } else if (!O.approx[i] && !N.approx[i]) {
      const int lmax = min(O.lmaxnu_tau[i], N.lmaxnu_tau[i]);
      const int nq = min(O.nq[i], N.nq[i]);
      for (int iq = 0; iq < nq; ++iq) {
        const int a = off + iq * (O.lmaxnu_tau[i] + 1), b = off2 + iq * (N.lmaxnu_tau[i] + 1);
        for (int l = 0; l <= lmax; ++l) yo[b + l] = y[a + l];
      }
      for (int iq = nq; iq < N.nq[i]; ++iq) {
        int lm = min(N.lmaxnu_tau[i], O.lmaxnr);
        const int b = off2 + iq * (N.lmaxnu_tau[i] + 1);
        for (int l = 0; l <= lm; ++l) yo[b + l] = y[O.r_ix + l];
        const double qq = C.nu_q[iq];
        const double ps = (C.nu_masses[i] / qq) * (C.nu_masses[i] / qq) / 2;
        lm = min(lm, O.lmaxnu_pert);
        for (int l = 0; l <= lm; ++l) yo[b + l] = yo[b + l] + y[O.nu_pert_ix + l] * ps;
      }
    }
  }
  if (N.has_nu_rel && O.has_nu_rel) {
    const int lmax = min(N.lmaxnu_pert, O.lmaxnu_pert);
    for (int l = 0; l <= lmax; ++l) yo[N.nu_pert_ix + l] = y[O.nu_pert_ix + l];
  }
}

// Per momentum bin of one eigenstate at scale factor a: a m/q, 1/sqrt(1+(a m/q)^2) and
// sqrt(1+(a m/q)^2), formed once per right-hand side and shared by the momentum
// integrals, the equations of motion and the source terms (q^-1 is tabulated).
constexpr int NQ = 16;
struct NuBins {
  double aq[NQ], v[NQ], s[NQ];
};

template <int W>
__device__ __forceinline__ void nu_bins(const DevCosmo& C, double a, int i, NuBins& b) {
  const double am = a * C.nu_masses[i];
  for (int iq = wlane<W>(); iq < C.nqmax; iq += W) {
    const double aq = am * C.nu_inv_q[iq];
    const double s2 = fma(aq, aq, 1.0);
    const double v = rsqrt(s2);
    b.aq[iq] = aq;
    b.v[iq] = v;
    b.s[iq] = s2 * v;
  }
  wsync<W>();
}

// Nu_Integrate_L01/L012 (equations.f90:1178-1270): momentum integrals of one eigenstate
template <bool L2, int W, class YV>
__device__ __forceinline__ void nu_integrate(const DevCosmo& C, const St& M, const YV y,
                                             const NuBins& b, int i, double& drhonu, double& fnu, double& dpnu,
                                             double& pinu) {
  drhonu = fnu = dpnu = pinu = 0;
  const int lane = wlane<W>();
  int ind = M.nu_ix[i] + lane * (M.lmaxnu_tau[i] + 1);
  for (int iq = lane; iq < M.nq[i]; iq += W) {
    const double w = C.nu_int_kernel[iq];
    drhonu += w * y[ind] * b.s[iq];
    fnu += w * y[ind + 1];
    if (L2) {
      dpnu += w * y[ind] * b.v[iq];
      pinu += w * y[ind + 2] * b.v[iq];
    }
    ind += W * (M.lmaxnu_tau[i] + 1);
  }
  ind = M.nu_pert_ix;
  for (int iq = M.nq[i] + lane; iq < C.nqmax; iq += W) {
    const double w = C.nu_int_kernel[iq];
    const double mq = C.nu_masses[i] * C.nu_inv_q[iq], ps = mq * mq * 0.5;
    const double tmp = w * (y[M.r_ix] + ps * y[ind]);
    drhonu += tmp * b.s[iq];
    fnu += w * (y[M.r_ix + 1] + ps * y[ind + 1]);
    if (L2) {
      dpnu += tmp * b.v[iq];
      pinu += w * (y[M.r_ix + 2] + ps * y[ind + 2]) * b.v[iq];
    }
  }
  if constexpr (W > 1) {
    drhonu = wsum<W>(drhonu);
    fnu = wsum<W>(fnu);
    if (L2) {
      dpnu = wsum<W>(dpnu);
      pinu = wsum<W>(pinu);
    }
  }
  if (L2) dpnu = dpnu / 3;
}

// Nu_pinudot (equations.f90:1272-1313)
template <int W, class YV>
__device__ double nu_pinudot(const DevCosmo& C, const St& M, const YV y,
                             const double* __restrict__ ydot, const NuBins& b, double adotoa, int i) {
  double pinudot = 0;
  const int lane = wlane<W>();
  int ind = M.nu_ix[i] + 2 + lane * (M.lmaxnu_tau[i] + 1);
  for (int iq = lane; iq < M.nq[i]; iq += W) {
    const double aq = b.aq[iq], v = b.v[iq];
    const double vdot = -aq * (aq * adotoa) * (v * v * v);
    pinudot += C.nu_int_kernel[iq] * (ydot[ind] * v + y[ind] * vdot);
    ind += W * (M.lmaxnu_tau[i] + 1);
  }
  ind = M.nu_pert_ix + 2;
  for (int iq = M.nq[i] + lane; iq < C.nqmax; iq += W) {
    const double aq = b.aq[iq], v = b.v[iq];
    const double mq = C.nu_masses[i] * C.nu_inv_q[iq], ps = mq * mq * 0.5;
    const double vdot = -aq * (aq * adotoa) * (v * v * v);
    const double psi2dot = ydot[M.r_ix + 2] + ps * ydot[ind];
    const double psi2 = y[M.r_ix + 2] + ps * y[ind];
    pinudot += C.nu_int_kernel[iq] * (psi2dot * v + psi2 * vdot);
  }
  return wsum<W>(pinudot);
}

// derivs (equations.f90:2273-2773) + sources (2775-2912), one mode per thread (W = 1)
// or per warp (W = 32, sbins: the warp's momentum-bin factors in shared memory)
//
// Multipole recurrences: one thread per mode reads the l-only factors from the global
// table (uniform addresses across the warp) and applies k; a warp per mode (lanes at
// different l) reads the mode's k-scaled factors from its shared memory (wrec: denlk,
// denlk2, polfack, NL entries each).
template <bool TR, int W, class YV>
__device__ __forceinline__ void derivs1(const DevCosmo& C, St& M, double tau, const YV y, double* __restrict__ dy,
                                        double* src, NuBins* sbins = nullptr, const double* wrec = nullptr) {
  const int lane = wlane<W>();
  const double* __restrict__ ra = kRec.a;
  const double* __restrict__ rb = kRec.b;
  const double* __restrict__ rp = kRec.p;
  const double* __restrict__ dl = wrec;
  const double* __restrict__ dl2 = wrec + NL;
  const double* __restrict__ pf = wrec + 2 * NL;
  const double k = M.k, ik = M.ik;
  const double itau = 1.0 / tau;
  double a, cs2, opac, dopac = 0;
  thermo_values(C, tau, itau, a, cs2, opac, dopac, M.tc || src != nullptr);
  const double a2 = a * a, ia = 1.0 / a, ia2 = ia * ia;
  const double etak = y[0], clxc = y[1], clxb = y[2], vb = y[3];
  const double grhob_t = C.grhob * ia, grhoc_t = C.grhoc * ia, grhor_t = C.grhornomass * ia2,
               grhog_t = C.grhog * ia2, grhov_t = C.grhov * a2;
  double dgrho = grhob_t * clxb + grhoc_t * clxc;
  double dgq = grhob_t * vb;
  double grhonu_t = 0, gpres_nu = 0, wnu[NUE] = {0, 0, 0};
  NuBins lbins[W == 1 ? NUE : 1];
  NuBins* const bins = W == 1 ? lbins : sbins;
  for (int i = 0; i < C.nu_eig; ++i) {  // MassiveNuVars (equations.f90:1358-1401)
    const double gm_t = C.grhormass[i] * ia2;
    double rhonu, pnu, clxnu, qnu;
    nuf::rho_P(a * C.nu_masses[i], rhonu, pnu);
    const double ir = 1.0 / rhonu;
    if (M.approx[i]) {
      clxnu = y[M.nu_ix[i]];
      qnu = y[M.nu_ix[i] + 2];
    } else {
      nu_bins<W>(C, a, i, bins[i]);
      double dp, pn;
      nu_integrate<false, W>(C, M, y, bins[i], i, clxnu, qnu, dp, pn);
      qnu = qnu * ir;
      clxnu = clxnu * ir;
    }
    const double g_t = gm_t * rhonu;
    grhonu_t += g_t;
    gpres_nu += gm_t * pnu;
    dgrho += g_t * clxnu;
    dgq += g_t * qnu;
    wnu[i] = pnu * ir;
  }
  const double dgrho_matter = dgrho, grho_matter = grhonu_t + grhob_t + grhoc_t;
  const double grho = (grhonu_t + grhob_t + grhoc_t) + grhor_t + grhog_t + grhov_t;
  const double gpres_noDE = gpres_nu + (grhor_t + grhog_t) * (1.0 / 3);
  const double g3 = grho * (1.0 / 3);
  const double iad = rsqrt(g3);
  const double adotoa = g3 * iad;
  double z = 0, dz = 0, clxr, qr, pir, clxg, qg, pig = 0;
  const int g = M.g_ix, pol = M.pol0, r = M.r_ix;
  if (M.nonu) {
    z = (0.5 * dgrho * ik + etak) * iad;
    dz = -adotoa * z - 0.5 * dgrho * ik;
    clxr = -4 * dz * ik;
    qr = -4.0 / 3 * z;
    pir = 0;
  } else {
    clxr = y[r];
    qr = y[r + 1];
    pir = y[r + 2];
  }
  if (M.nophot) {
    if (!M.nonu) {
      z = (0.5 * dgrho * ik + etak) * iad;
      dz = -adotoa * z - 0.5 * dgrho * ik;
      clxg = -4 * dz * ik - 4 * ik * opac * (vb + z);
      qg = -4.0 / 3 * z;
    } else {
      clxg = clxr - 4 * ik * opac * (vb + z);
      qg = qr;
    }
  } else {
    clxg = y[g];
    qg = y[g + 1];
    if (!M.tc) pig = y[g + 2];
  }
  dgrho = dgrho + grhog_t * clxg + grhor_t * clxr;
  dgq = dgq + grhog_t * qg + grhor_t * qr;
  const double photbar = C.photbar_a * ia;
  const double pb43 = 4.0 / 3 * photbar;
  z = (0.5 * dgrho * ik + etak) * iad;
  const double sigma = z + 1.5 * dgq * M.ik2;
  dy[0] = 0.5 * dgq;
  dy[1] = -k * z;
  const double clxbdot = -k * (z + vb);
  dy[2] = clxbdot;
  const double clxgdot = -k * (4.0 / 3.0 * z + qg);
  const double delta_p_b = cs2 * clxb;
  double vbdot, pigdot = 0;
  if (M.tc) {
    const double gpres = gpres_noDE - grhov_t;
    const double adotdota = (adotoa * adotoa - gpres) / 2;
    const double iop = 1.0 / opac, iop2 = iop * iop;
    const double i1pb = 1.0 / (1 + pb43);
    pig = 32.0 / 45 * iop * k * (sigma + vb);
    const double slip = -(2 * adotoa * i1pb + dopac * iop) * (vb - 3.0 / 4 * qg) +
                        (-adotdota * vb - k / 2 * adotoa * clxg + k * (cs2 * clxbdot - clxgdot / 4)) * iop * i1pb;
    const double dgs = grhog_t * pig + grhor_t * pir;
    const double sigmadot = -2 * adotoa * sigma - dgs * ik + etak;
    const double qgdot_tc = k * (clxg / 4.0 - pig / 2.0) + opac * slip;
    const double f11 = dopac * 11.0 / 6.0 * iop2;
    pig = 32.0 / 45 * iop * k * (sigma + 3.0 * qg / 4.0) * (1 + f11) +
          (32.0 / 45.0 * iop2) * k * (sigmadot + 3.0 * qgdot_tc / 4.0) * (-11.0 / 6.0);
    pigdot = -(32.0 / 45.0) * (dopac * iop2) * k * (sigma + 3.0 * qg / 4.0) * (1 + f11) +
             (32.0 / 45.0 * iop) * k * (sigmadot + 3.0 * qgdot_tc / 4.0) * (1 + (11.0 / 6.0) * (dopac * iop2));
    M.pigdot = pigdot;
    vbdot = (-adotoa * vb + cs2 * k * clxb + k / 4 * pb43 * (clxg - 2 * pig)) * i1pb;
    vbdot = vbdot + pb43 * i1pb * slip;
    M.pig = pig;
  } else {
    vbdot = -adotoa * vb + k * delta_p_b - photbar * opac * (4.0 / 3 * vb - qg);
  }
  dy[3] = vbdot;
  double qgdot = 0, polter = 0, E2 = 0;
  if (!M.nophot) {
    dy[g] = clxgdot;
    const double inv_pb43 = a * C.photbar_fac;  // 3/(4 photbar)
    qgdot = 4.0 / 3 * (-vbdot - adotoa * vb + delta_p_b * k) * inv_pb43 + k * ((1.0 / 3) * clxg - (2.0 / 3) * pig);
    dy[g + 1] = qgdot;
    if (!M.tc) {
      E2 = y[pol + 2];
      polter = pig * 0.1 + 9.0 / 15 * E2;
      const double g3v = y[g + 3];
      pigdot = k * (0.4 * qg - 0.6 * g3v) - opac * (pig - polter) + 8.0 / 15.0 * k * sigma;
      dy[g + 2] = pigdot;
      const int lg = M.lmaxg;
      const int lp = M.lmaxgpol;
      if constexpr (W == 1) {
        // one read of each entry: the neighbours travel in registers
        double ym = pig, y0 = g3v;
#pragma unroll kRhsUnroll
        for (int l = 3; l < lg; ++l) {
          const double yp = y[g + l + 1];
          dy[g + l] = k * (__ldg(ra + l) * ym - __ldg(rb + l) * yp) - opac * y0;
          ym = y0;
          y0 = yp;
        }
        dy[g + lg] = k * ym - (lg + 1) * itau * y0 - opac * y0;
        const double p3v = y[pol + 3];
        dy[pol + 2] = -opac * (E2 - polter) - k * (1.0 / 3.0) * p3v;
        ym = E2;
        y0 = p3v;
#pragma unroll kRhsUnroll
        for (int l = 3; l < lp; ++l) {
          const double yp = y[pol + l + 1];
          dy[pol + l] = -opac * y0 + k * (__ldg(ra + l) * ym - __ldg(rp + l) * yp);
          ym = y0;
          y0 = yp;
        }
        dy[pol + lp] = -opac * y0 + M.kptf * ym - (lp + 3) * itau * y0;
      } else {
        for (int l = 3 + lane; l < lg; l += W)
          dy[g + l] = (dl[l] * y[g + l - 1] - dl2[l] * y[g + l + 1]) - opac * y[g + l];
        dy[g + lg] = k * y[g + lg - 1] - (lg + 1) * itau * y[g + lg] - opac * y[g + lg];
        dy[pol + 2] = -opac * (E2 - polter) - k * (1.0 / 3.0) * y[pol + 3];
        for (int l = 3 + lane; l < lp; l += W)
          dy[pol + l] = -opac * y[pol + l] + (dl[l] * y[pol + l - 1] - pf[l] * y[pol + l + 1]);
        dy[pol + lp] = -opac * y[pol + lp] + M.kptf * y[pol + lp - 1] - (lp + 3) * itau * y[pol + lp];
      }
    }
  }
  double clxrdot = 0, pirdot = 0;
  if (!M.nonu) {
    clxrdot = -k * (4.0 / 3.0 * z + qr);
    dy[r] = clxrdot;
    dy[r + 1] = k * ((1.0 / 3) * clxr - (2.0 / 3) * pir);
    if (M.hk) {
      pirdot = -3 * pir * itau - clxrdot;
      dy[r + 2] = pirdot;
    } else {
      const double n3v = y[r + 3];
      pirdot = k * (0.4 * qr - 0.6 * n3v) + 8.0 / 15.0 * k * sigma;
      dy[r + 2] = pirdot;
      const int ln = M.lmaxnr;
      if constexpr (W == 1) {
        double ym = pir, y0 = n3v;
#pragma unroll kRhsUnroll
        for (int l = 3; l < ln; ++l) {
          const double yp = y[r + l + 1];
          dy[r + l] = k * (__ldg(ra + l) * ym - __ldg(rb + l) * yp);
          ym = y0;
          y0 = yp;
        }
        dy[r + ln] = k * ym - (ln + 1) * itau * y0;
      } else {
        for (int l = 3 + lane; l < ln; l += W) dy[r + l] = dl[l] * y[r + l - 1] - dl2[l] * y[r + l + 1];
        dy[r + ln] = k * y[r + ln - 1] - (ln + 1) * itau * y[r + ln];
      }
    }
  }
  // massive neutrinos (equations.f90:2710-2773)
  for (int i = 0; i < C.nu_eig; ++i) {
    if (M.approx[i]) {
      const double G11_t = M.G11[i] * ia * ia2, G30_t = M.G30[i] * ia * ia2;
      const int off = M.nu_ix[i];
      const double w = wnu[i];
      dy[off] = -k * z * (w + 1) + 3 * adotoa * (w * y[off] - y[off + 1]) - k * y[off + 2];
      dy[off + 1] = (3 * w - 2) * adotoa * y[off + 1] - 5.0 / 3 * k * z * w - k / 3 * G11_t;
      dy[off + 2] = (3 * w - 1) * adotoa * y[off + 2] - k * (2.0 / 3 * y[off + 3] - y[off + 1]);
      dy[off + 3] = (3 * w - 2) * adotoa * y[off + 3] + 2 * w * k * sigma - k / 5 * (3 * G30_t - 2 * G11_t);
    } else if constexpr (W == 1) {
      int ind = M.nu_ix[i];
      const int lt = M.lmaxnu_tau[i];
      for (int iq = 0; iq < M.nq[i]; ++iq) {
        const double v = bins[i].v[iq], vk = v * k;
        const double y0v = y[ind], y1v = y[ind + 1], y2v = y[ind + 2];
        const double d0 = -k * (4.0 / 3.0 * z + v * y1v);
        dy[ind] = d0;
        dy[ind + 1] = vk * ((1.0 / 3) * y0v - (2.0 / 3) * y2v);
        if (lt == 2) {
          dy[ind + 2] = -d0 - 3 * itau * y2v;
        } else {
          const double y3v = y[ind + 3];
          dy[ind + 2] = vk * (0.4 * y1v - 0.6 * y3v) + k * 8.0 / 15.0 * sigma;
          double ym = y2v, yc = y3v;
#pragma unroll kRhsUnroll
          for (int l = 3; l < lt; ++l) {
            const double yp = y[ind + l + 1];
            dy[ind + l] = vk * (__ldg(ra + l) * ym - __ldg(rb + l) * yp);
            ym = yc;
            yc = yp;
          }
          dy[ind + lt] = k * v * ym - (lt + 1) * itau * yc;
        }
        ind += lt + 1;
      }
    } else {
      // the (momentum bin, l) entries of the eigenstate, flattened over the lanes
      const int lt = M.lmaxnu_tau[i], lt1 = lt + 1, tot = M.nq[i] * lt1;
      int iq = lane / lt1, l = lane - iq * lt1;
      for (int e = lane; e < tot; e += W) {
        const int ind = M.nu_ix[i] + iq * lt1;
        const double v = bins[i].v[iq], vk = v * k;
        double d;
        if (l == 0) d = -k * (4.0 / 3.0 * z + v * y[ind + 1]);
        else if (l == 1) d = vk * ((1.0 / 3) * y[ind] - (2.0 / 3) * y[ind + 2]);
        else if (l == 2 && lt == 2) d = k * (4.0 / 3.0 * z + v * y[ind + 1]) - 3 * itau * y[ind + 2];
        else if (l == 2) d = vk * (0.4 * y[ind + 1] - 0.6 * y[ind + 3]) + k * 8.0 / 15.0 * sigma;
        else if (l < lt) d = v * (dl[l] * y[ind + l - 1] - dl2[l] * y[ind + l + 1]);
        else d = k * v * y[ind + lt - 1] - (lt + 1) * itau * y[ind + lt];
        dy[ind + l] = d;
        l += W;
        while (l >= lt1) {
          l -= lt1;
          ++iq;
        }
      }
    }
  }
  if (M.has_nu_rel) {
    const int p0 = M.nu_pert_ix, lp = M.lmaxnu_pert;
    if constexpr (W == 1) {
      double pm = y[p0], pc = y[p0 + 1], rm = y[r], rc = y[r + 1];
      dy[p0] = k * a2 * qr - k * pc;
#pragma unroll kRhsUnroll
      for (int l = 1; l < lp; ++l) {
        const double rpv = y[r + l + 1], pp = y[p0 + l + 1];
        const double al = __ldg(ra + l), bl = __ldg(rb + l);
        dy[p0 + l] = k * (-a2 * (al * rm - bl * rpv) + (al * pm - bl * pp));
        rm = rc;
        rc = rpv;
        pm = pc;
        pc = pp;
      }
      dy[p0 + lp] = k * (pm - a2 * rm) - (lp + 1) * itau * pc;
    } else {
      dy[p0] = k * a2 * qr - k * y[p0 + 1];
      for (int l = 1 + lane; l < lp; l += W)
        dy[p0 + l] = -a2 * (dl[l] * y[r + l - 1] - dl2[l] * y[r + l + 1]) + (dl[l] * y[p0 + l - 1] - dl2[l] * y[p0 + l + 1]);
      dy[p0 + lp] = k * (y[p0 + lp - 1] - a2 * y[r + lp - 1]) - (lp + 1) * itau * y[p0 + lp];
    }
  }
  if (src) {
    wsync<W>();  // the source terms read derivatives written by other lanes
    double Ed2 = 0, Ed3 = 0, octgdot = 0, E2s = 0;
    if (M.nophot) {
      pigdot = 0;
      qgdot = -4 * dz / 3;
    } else if (M.tc) {
      const double iop = 1.0 / opac;
      E2s = pig / 4 + pigdot * iop * (-5.0 / 8.0);
      Ed2 = (pigdot / 4.0) * (1 + (5.0 / 2.0) * (dopac * iop * iop));
    } else {
      E2s = E2;
      Ed2 = dy[pol + 2];
      Ed3 = dy[pol + 3];
      octgdot = dy[g + 3];
    }
    if (M.nonu) pirdot = 0;
    double dgpi = grhor_t * pir + grhog_t * pig;
    double dgpi_diff = 0;
    double pidot_sum = grhog_t * pigdot + grhor_t * pirdot;
    double grhonu_out = 0, dgrhonu_out = 0;
    for (int i = 0; i < C.nu_eig; ++i) {  // MassiveNuVarsOut (equations.f90:1113-1176)
      const double gm_t = C.grhormass[i] * ia2;
      double rhonu, pnu, pinu, pinudot, clxnu;
      nuf::rho_P(a * C.nu_masses[i], rhonu, pnu);
      if (M.approx[i]) {
        clxnu = y[M.nu_ix[i]];
        pinu = y[M.nu_ix[i] + 3];
        pinudot = dy[M.nu_ix[i] + 3];
      } else {
        double qnu, dpnu;
        nu_integrate<true, W>(C, M, y, bins[i], i, clxnu, qnu, dpnu, pinu);
        clxnu = clxnu / rhonu;
        pinu = pinu / rhonu;
        const double rhonudot = nuf::drho(a * C.nu_masses[i], adotoa);
        pinudot = nu_pinudot<W>(C, M, y, dy, bins[i], adotoa, i);
        pinudot = pinudot / rhonu - rhonudot / rhonu * pinu;
      }
      const double g_t = gm_t * rhonu, gp_t = gm_t * pnu;
      grhonu_out += g_t;
      dgrhonu_out += g_t * clxnu;
      dgpi += g_t * pinu;
      dgpi_diff += pinu * (3 * gp_t - g_t);
      pidot_sum += g_t * pinudot;
    }
    const double gpres = gpres_noDE - grhov_t;
    const double diff_rhopi = pidot_sum - (4 * dgpi + dgpi_diff) * adotoa;
    const double phi = -((dgrho + 3 * dgq * adotoa * ik) + dgpi) / (2 * M.k2);
    if (TR && !M.out_src) {  // outtransf's variables (equations.f90:2832-2845), src holds 13
      src[0] = k / C.hubble_h;
      src[1] = clxc;
      src[2] = clxb;
      src[3] = clxg;
      src[4] = clxr;
      src[5] = C.nu_eig > 0 ? dgrhonu_out / grhonu_out : 0.0;
      src[6] = dgrho_matter / grho_matter;
      src[7] = (grhob_t * clxb + grhoc_t * clxc) / (grhob_t + grhoc_t);
      src[8] = dgrho / grho_matter;
      src[9] = M.k2 * phi;
      src[10] = -k * sigma / adotoa;
      src[11] = -k * (vb + sigma) / adotoa;
      src[12] = vb;
      return;
    }
    double op2, dop2, vis, dvis, ddvis, exptau;
    ionization(C, tau, itau, op2, dop2, vis, dvis, ddvis, exptau);
    const double k2 = M.k2;
    const double phidot =
        0.5 * (adotoa * (-dgpi - 2 * k2 * phi) + dgq * k - diff_rhopi + k * sigma * (gpres + grho)) * M.ik2;
    const double sigmadot = -adotoa * sigma - 0.5 * dgpi * ik + k * phi;
    polter = pig / 10 + 9.0 / 15 * E2s;
    const double polterdot = (1.0 / 10.0) * pigdot + (3.0 / 5.0) * Ed2;
    const double polterddot = -2.0 / 25.0 * adotoa * dgq * ik - 4.0 / 75.0 * adotoa * k * sigma - 4.0 / 75.0 * dgpi -
                              2.0 / 75.0 * dgrho - 3.0 / 50.0 * k * octgdot + (1.0 / 25.0) * k * qgdot -
                              1.0 / 5.0 * k * Ed3 + (-1.0 / 10.0 * pig + (7.0 / 10.0) * polter - 3.0 / 5.0 * E2s) * dop2 +
                              (-1.0 / 10.0 * pigdot + (7.0 / 10.0) * polterdot - 3.0 / 5.0 * Ed2) * op2;
    const double ISW = 2 * phidot * exptau;
    const double monopole_source = (-etak * ik + 2 * phi + clxg / 4) * vis;
    const double doppler = ((sigma + vb) * dvis + (sigmadot + vbdot) * vis) * ik;
    const double quadrupole_source =
        (5.0 / 8.0) * (3 * polter * ddvis + 6 * polterdot * dvis + (k2 * polter + 3 * polterddot) * vis) * M.ik2;
    src[0] = ISW + doppler + monopole_source + quadrupole_source;
    const double ang = C.tau0 - tau;
    src[1] = tau < C.tau0 ? vis * polter * (15.0 / 8.0) / (ang * ang * k2) : 0.0;
    src[2] = 0;
    if (C.nsrc > 2 && tau > C.tau_maxvis && ang > 0.1)
      src[2] = -2 * phi * (tau - C.tau_maxvis) / ((C.tau0 - C.tau_maxvis) * ang);
  }
}

#ifndef CG_RHS_CALL
#define CG_RHS_CALL 1
#endif
// (the warp-per-mode kernels keep it inline: out of line they ran 176 against 172 ms on one
// lensed lmax-2500 cosmology and 65 against 58 ms on one lmax-1000 cosmology)
#ifndef CG_RHS_CALL_WARP
#define CG_RHS_CALL_WARP 0
#endif
// The right-hand side as one out-of-line function for the thread-per-mode kernels (a
// trial step evaluates it at eight call sites; inlined, each is a copy of the whole
// body): half the code, 0.8 % faster at 256 draws (1212 against 1222 ms)
template <bool TR, int W, class YV>
__device__ __noinline__ void derivs1_call(const DevCosmo& C, St& M, double tau, const YV y, double* __restrict__ dy,
                                          double* src, NuBins* sbins, const double* wrec) {
  derivs1<TR, W>(C, M, tau, y, dy, src, sbins, wrec);
}
template <bool TR, int W, class YV>
__device__ __forceinline__ void rhs(const DevCosmo& C, St& M, double tau, const YV y, double* __restrict__ dy,
                                    double* src, NuBins* sbins, const double* wrec) {
  if constexpr ((W == 1 || CG_RHS_CALL_WARP != 0) && CG_RHS_CALL != 0) derivs1_call<TR, W>(C, M, tau, y, dy, src, sbins, wrec);
  else derivs1<TR, W>(C, M, tau, y, dy, src, sbins, wrec);
}

// Pitch of the rows in a thread's local memory.  Rows packed at the mode's own system size
// (7 x ~85 entries together) ran 11 % slower at 256 draws than rows NV entries apart
// (1319 against 1189 ms): the six rows a stage combination reads at one entry then fall
// on neighbouring addresses instead of spreading over the memory partitions.  Among
// pitches of 448, 456, 480 and 512 entries, 456 ran fastest (1180 against 1191 ms).
#ifndef CG_ROW_PITCH
#define CG_ROW_PITCH 456
#endif
constexpr int kRowPitch = CG_ROW_PITCH;
static_assert(kRowPitch >= NV, "a row holds the largest packed system");

// The stage vectors live in the seven rows of b; every row is named by a slot index so
// that accepting a step swaps indices, not vectors.
struct Work {
  double b[kRows][kRowPitch];
};

// The same rows for a warp's mode, in the warp's slice of shared memory
struct WorkS {
  double* b;  // [kRows][stride]
  int stride;
  NuBins* bins;  // [NUE] momentum-bin factors of the current right-hand side
  double* rec;   // [3][NL] the mode's denlk, denlk2, polfack
};
__device__ __forceinline__ double* row(Work& w, int s) { return w.b[s]; }
__device__ __forceinline__ double* row(const WorkS& w, int s) { return w.b + (size_t)s * w.stride; }
__device__ __forceinline__ NuBins* sbins(Work&) { return nullptr; }
__device__ __forceinline__ NuBins* sbins(const WorkS& w) { return w.bins; }
__device__ __forceinline__ int row_cap(const Work&) { return NV; }

__device__ __forceinline__ int row_cap(const WorkS& w) { return w.stride; }
__device__ __forceinline__ const double* wrec(const Work&) { return nullptr; }
__device__ __forceinline__ const double* wrec(const WorkS& w) { return w.rec; }

// state of one mode's integration, advanced one trial step per loop iteration
struct Run {
  double src[13];  // source functions, or the 13 transfer variables without the CMB
  double tau, target, sw_time, h, err, call_hmax;
  double ny;            // min(max|y|, 1) of the current state (valid when ny_valid)
  int sy, syt, sk1, sk2, sk3, sk4, sk5;  // rows holding y, the trial state and k1..k5 (k6 in sk2, k7 in sk4)
  bool ny_valid;
  long long evals;
  int j, fails, status, sw_kind, sw_eig;
  bool active, target_is_switch, need_f, first, fsal, reset, src_valid;
  // transfer path, a source mode of a run that also wants the CMB: it stops at the source
  // times as well (no output there), in CalcScalarSources' order; st 0: transfer times
  // before the second source time, 1: next stop the source time js, 2: at source time jj
  bool stops, tgt_out;
  int st, js, jj;
};

enum { SW_TC = 1, SW_KTAU, SW_NU_MASSLESS, SW_NU_NONREL, SW_NU_MASSIVE, SW_NONU, SW_NOPHOT };

__device__ __forceinline__ int next_nu_nq(const DevCosmo& C, int nq) {
  if (nq == 0) return 1;
  const int qq = (int)C.nu_q[nq - 1];
  return qq >= 10 ? C.nqmax : nq + 1;
}

template <int W, class WK>
__device__ void mode_init(const DevCosmo& C, int q_ix, St& M, WK& Wk, Run& R) {
  const int lane = wlane<W>();
  const CambGpuModeSpec ms = C.modes[q_ix];
  M.q = ms.q;
  M.k = ms.q;
  M.ik = 1.0 / M.k;
  M.k2 = M.k * M.k;
  M.ik2 = 1.0 / M.k2;
  M.lmaxg = ms.lmaxg;
  M.lmaxgpol = ms.lmaxgpol;
  M.lmaxnr = ms.lmaxnr;
  M.lmaxnu = ms.lmaxnu;
  M.poltruncfac = (double)M.lmaxgpol / max(1, M.lmaxgpol - 2);
  M.kptf = M.k * M.poltruncfac;
  M.pig = M.pigdot = 0;
  M.out_src = false;
  M.tight_off = ms.tight_switch_tau;
  M.tc = true;
  M.hk = M.nonu = M.nophot = false;
  for (int i = 0; i < NUE; ++i) {
    M.nq[i] = ms.nq0[i];
    M.approx[i] = false;
    M.nonrel[i] = false;
    M.lboost[i] = ms.nu_l_boost[i];
    M.approx_time[i] = ms.nu_approx_time[i];
    M.G11[i] = M.G30[i] = 0;
  }
  M.nu_pert_ix = 0;
  M.pol0 = 0;
  setup_indices(C, M, true);
  R.active = true;
  R.status = 0;
  const int lm = max(max(M.lmaxg, M.lmaxgpol), max(M.lmaxnr, M.lmaxnu));
  if (M.nvar > row_cap(Wk) || lm >= NL || C.nu_eig > NUE || C.nqmax > NQ) {
    R.active = false;
    R.status = CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
    return;
  }
  R.sy = 0;
  R.sk1 = 1;
  R.sk2 = 2;
  R.sk3 = 3;
  R.sk4 = 4;
  R.sk5 = 5;
  R.syt = 6;
  R.ny_valid = false;
  double* const Y = row(Wk, R.sy);
  if constexpr (W > 1) {  // the warp's k-scaled recurrence factors (initial(), equations.f90:1911-1916)
    for (int l = 1 + lane; l <= lm; l += W) {
      const double dn = 1.0 / (2 * l + 1);
      Wk.rec[l] = dn * M.k * l;
      Wk.rec[NL + l] = dn * M.k * (l + 1);
      Wk.rec[2 * NL + l] = ((double)((l + 3) * (l - 1)) / (l + 1)) * M.k * dn;
    }
  }
  for (int i = lane; i < M.nvar; i += W) Y[i] = 0;
  wsync<W>();  // the initial values below are written by every lane
  // initial (equations.f90:1891-2112), adiabatic
  const double tau = ms.taustart, k = M.k;
  const double x = k * tau, x2 = x * x, x3 = x2 * x;
  double rhomass = 0;
  for (int i = 0; i < C.nu_eig; ++i) rhomass += C.grhormass[i];
  const double grhonu = rhomass + C.grhornomass;
  const double om = (C.grhob + C.grhoc) / sqrt(3 * (C.grhog + grhonu));
  const double omtau = om * tau;
  const double Rv = grhonu / (grhonu + C.grhog);
  const double Rp15 = 4 * Rv + 15;
  const double iv_clxg = -1.0 / 3 * x2 * (1 - omtau / 5);
  const double iv_clxb = 0.75 * iv_clxg;
  const double iv_qg = iv_clxg * x / 9.0;
  const double iv_qr = -(4 * Rv + 23) / Rp15 * x3 / 27;
  const double iv_vb = 0.75 * iv_qg;
  const double iv_pir = 4.0 / 3 * x2 / Rp15 * (1 + omtau / 4 * (4 * Rv - 5) / (2 * Rv + 15));
  const double iv_aj3r = 4 / 21.0 / Rp15 * x3;
  const double iv_eta = -2 * (1 - x2 / 12 * (-10.0 / Rp15 + 1));
  Y[0] = iv_eta * k / 2;
  Y[1] = -iv_clxb;
  Y[2] = -iv_clxb;
  Y[3] = -iv_vb;
  Y[M.g_ix] = -iv_clxg;
  Y[M.g_ix + 1] = -iv_qg;
  Y[M.r_ix] = -iv_clxg;
  Y[M.r_ix + 1] = -iv_qr;
  Y[M.r_ix + 2] = -iv_pir;
  if (M.lmaxnr > 2) Y[M.r_ix + 3] = -iv_aj3r;
  for (int i = 0; i < C.nu_eig; ++i) {
    int ind = M.nu_ix[i];
    for (int iq = 0; iq < M.nq[i]; ++iq) {
      for (int jj = 0; jj < 3; ++jj) Y[ind + jj] = Y[M.r_ix + jj];
      if (M.lmaxnu_tau[i] > 2) Y[ind + 3] = -iv_aj3r;
      ind += M.lmaxnu_tau[i] + 1;
    }
  }
  wsync<W>();
  R.tau = tau;
  R.j = C.transfer_only ? 0 : 1;
  R.stops = C.transfer_only && q_ix < C.tr_src_modes;
  R.tgt_out = true;
  R.st = 0;
  R.js = 1;
  R.jj = 0;
  R.h = R.err = 0;
  R.fails = 0;
  R.fsal = false;
  R.reset = true;
  R.need_f = false;
  R.first = false;
  R.evals = 0;
  R.target = tau;
  R.target_is_switch = false;
  R.src_valid = false;
  R.call_hmax = 0;
  R.sw_kind = 0;
  R.sw_eig = 0;
}

// Picks the next integration target with the switch logic of EvolveScal
// (equations.f90:261-331) and records which switch the target is.  Returns false
// when the mode is finished.
// The next stop of a source mode on the transfer path of a run that also wants the CMB,
// CalcScalarSources with WantTransfer (cmbmain.f90:1020-1070): the transfer times before the
// second source time, then every source time, each followed by the transfer times inside
// its interval (or within 1e-5 of it, or any left at the last source time -- the reference's
// `goto 101`).  A pure function of the stop state (settling states that consume nothing);
// run_modes advances the state when a stop is reached.  false: no stop left (or, with an
// evolution error in R.status, a state that did not settle).
__device__ __forceinline__ bool stop_target(const DevCosmo& C, St& M, Run& R, double& tgt) {
  const double* P = C.tau_points;
  const double* TT = C.transfer_times;
  const int ntau = C.ntau, ntt = C.n_tt;
  const bool tr_left = R.j < ntt;
  if (!tr_left && !C.src_out) return false;  // nothing left to store
  if (R.st == 0) {
    if (tr_left && P[1] > TT[R.j]) {
      tgt = TT[R.j];
      R.tgt_out = true;
      M.out_src = false;
      return true;
    }
    R.st = 1;
    R.js = 1;
  }
  if (R.st == 2) {
    const int jj = R.jj;
    if (tr_left) {
      if (jj < ntau - 1 && P[jj] < TT[R.j] && P[jj + 1] > TT[R.j]) {
        tgt = TT[R.j];
        R.tgt_out = true;
        M.out_src = false;
        return true;
      }
      if (fabs(R.tau - TT[R.j]) < 1e-5 || jj == ntau - 1) {
        tgt = R.tau;  // output at the current state
        R.tgt_out = true;
        M.out_src = false;
        return true;
      }
    }
    R.st = 1;
    R.js = jj + 1;
  }
  if (R.js >= ntau) return false;
  // past the last transfer time the reference's late-time cut ends the mode's sources
  if (!tr_left && M.q * P[R.js] > C.max_etak_scalar && P[R.js] > C.taurend && !C.want_late_time &&
      R.tau > TT[ntt - 1])
    return false;
  tgt = P[R.js];
  R.tgt_out = C.src_out != nullptr;  // the CMB sources of a single launch of both halves
  M.out_src = true;
  return true;
}

// run_modes' step after a stop of that kind is reached (the transfer output, if any, done)
__device__ __forceinline__ void stop_reached(const DevCosmo& C, Run& R) {
  if (R.st == 1) {  // a source time: the transfer checks after it
    R.st = 2;
    R.jj = R.js;
    return;
  }
  if (R.st == 2) {  // a transfer output after source time jj: again, or on to the next source time
    const int jj = R.jj;
    if (!(jj < C.ntau - 1 && R.j < C.n_tt && C.tau_points[jj + 1] > C.transfer_times[R.j])) {
      R.st = 1;
      R.js = jj + 1;
    }
  }
}

template <bool TR>
__device__ bool next_target(const DevCosmo& C, St& M, Run& R) {
  double tauend;
  if constexpr (TR) {  // GetTransfer: the transfer times in turn
    if (R.stops) {
      if (!stop_target(C, M, R, tauend)) return false;
    } else {
      if (R.j >= C.n_tt) return false;
      tauend = C.transfer_times[R.j];
    }
  } else {
    if (R.j >= C.ntau) return false;
    tauend = C.tau_points[R.j];
    // CalcScalarSources' late-time cut; a run with transfer functions keeps the mode going
    // until the last transfer time (cmbmain.f90:1032-1035)
    if (M.q * tauend > C.max_etak_scalar && tauend > C.taurend && !C.want_late_time && R.tau > C.src_keep_tau)
      return false;
  }
  const double noSwitch = C.tau0 + 1;
  const double smallTime = fmin(R.tau, M.ik) / 100;
  const double switchBoost = C.AccuracyBoost * C.TimeSwitchBoost;
  double t_ktau = noSwitch, t_nonu = noSwitch, t_nophot = noSwitch;
  double t_massless = noSwitch, t_nonrel = noSwitch, t_massive = noSwitch;
  int e_massless = 0, e_nonrel = 0, e_massive = 0;
  if (!M.hk && !M.nonu) t_ktau = (double)max(20, M.lmaxnr - 4) / M.k;
  for (int i = 0; i < C.nu_eig; ++i) {
    if (M.nq[i] != C.nqmax) {
      const double t = C.nu_tau_notmassless[i * C.nqmax + next_nu_nq(C, M.nq[i]) - 1];
      if (t < t_massless) { t_massless = t; e_massless = i; }
    } else if (!M.nonrel[i]) {
      if (C.nu_tau_nonrel[i] < t_nonrel) { t_nonrel = C.nu_tau_nonrel[i]; e_nonrel = i; }
    } else if (!M.approx[i]) {
      if (M.approx_time[i] < t_massive) { t_massive = M.approx_time[i]; e_massive = i; }
    }
  }
  if (!M.nonu) t_nonu = fmax(15 / M.k * switchBoost, fmin(C.taurend, C.matter_verydom_tau));
  const double lp = fmax(switchBoost, C.late_phot_boost_min);  // latePhotSwitchBoost
  if (!M.nophot && (!C.want_cls || M.k > 0.03 * lp)) t_nophot = fmax(15 / M.k, C.taurend) * lp;
  const double next = fmin(fmin(fmin(t_ktau, t_massless), M.tight_off),
                           fmin(fmin(t_massive, t_nonu), fmin(fmin(t_nophot, t_nonrel), noSwitch)));
  // the order of the reference's if-chain decides ties
  int kind = 0, eig = 0;
  if (next == M.tight_off) kind = SW_TC;
  else if (next == t_ktau) kind = SW_KTAU;
  else if (next == t_massless) { kind = SW_NU_MASSLESS; eig = e_massless; }
  else if (next == t_nonrel) { kind = SW_NU_NONREL; eig = e_nonrel; }
  else if (next == t_massive) { kind = SW_NU_MASSIVE; eig = e_massive; }
  else if (next == t_nonu) kind = SW_NONU;
  else if (next == t_nophot) kind = SW_NOPHOT;
  double tgt;
  bool is_switch;
  if (next < tauend) {
    R.sw_kind = kind;
    R.sw_eig = eig;
    R.sw_time = next;
    if (!(next > R.tau + smallTime)) {  // switch at the current time without integrating
      R.target = R.tau;
      R.target_is_switch = true;
      return true;
    }
    tgt = next;
    is_switch = true;
  } else {
    tgt = tauend;
    is_switch = false;
  }
  // start of a GaugeInterface_ScalEv / RungeKuttaDP45 call
  const double ms_user = (M.q < 2e-3 && R.tau <= C.taurend && C.want_cls) ? 2.0 : 20.0 / C.IntTolBoost;
  R.call_hmax = R.reset ? 0.0 : ms_user;
  R.first = R.reset;
  if (R.reset) {
    R.fsal = false;
    R.fails = 0;
    R.reset = false;
  }
  R.need_f = true;
  R.target = tgt;
  R.target_is_switch = is_switch;
  return true;
}

// the switch branches of EvolveScal (equations.f90:333-451); layout changes repack y via yt
// the trial-state row becomes the state row
__device__ __forceinline__ void swap_rows(Run& R, double*& Y, double*& YT) {
  const int t = R.sy;
  R.sy = R.syt;
  R.syt = t;
  double* p = Y;
  Y = YT;
  YT = p;
}

// A new layout larger than the mode's largest packed system (which sizes its rows): not
// expected, since setup_indices bounds every layout of the mode at its start; the mode
// ends with an evolution error instead of writing past its rows.
__device__ __forceinline__ void layout_overflow(Run& R) { R.status = CAMBGPU_ERROR_EVOLUTION; }

template <int W, class WK>
__device__ void apply_switch(const DevCosmo& C, St& M, WK& Wk, Run& R) {
  const double noSwitch = C.tau0 + 1;
  St N = M;
  double* Y = row(Wk, R.sy);
  double* YT = row(Wk, R.syt);
  R.ny_valid = false;
  const int kind = R.sw_kind, e = R.sw_eig;
  if (kind == SW_TC) {
    N.tc = false;
    N.tight_off = noSwitch;
    setup_indices(C, N, false);
    if (N.n > N.nvar) return layout_overflow(R);
    copy_vars<W>(C, M, N, Y, YT);
    M = N;
    swap_rows(R, Y, YT);
    R.reset = true;
    const double tau = R.tau, itau = 1.0 / tau;
    double a, cs2, opac, dopac;
    thermo_values(C, tau, itau, a, cs2, opac, dopac);
    const double kb = M.k, op2 = opac * opac;
    Y[M.g_ix + 2] = M.pig;
    Y[M.g_ix + 3] = (3.0 / 7.0) * M.pig * (kb / opac) * (1.0 + dopac / op2) + (3.0 / 7.0) * M.pigdot * (kb / op2) * (-1.0);
    const double p2 = M.pig / 4 + M.pigdot * (1.0 / opac) * (-5.0 / 8.0 - (25.0 / 16.0) * dopac / op2) +
                      M.pig * (kb / opac) * (kb / opac) * (-5.0 / 56.0);
    Y[M.pol0 + 2] = p2;
    Y[M.pol0 + 3] = (3.0 / 7.0) * (kb / opac) * p2 * (1.0 + dopac / op2) +
                      (3.0 / 7.0) * (kb / op2) * ((M.pigdot / 4.0) * (1.0 + (5.0 / 2.0) * dopac / op2)) * (-1.0);
  } else if (kind == SW_NU_MASSIVE) {
    // SwitchToMassiveNuApprox (equations.f90:1072-1111)
    const double tau = R.tau, itau = 1.0 / tau;
    double a, cs2, opac, dopac;
    thermo_values(C, tau, itau, a, cs2, opac, dopac, false);
    const double a2 = a * a;
    N.approx[e] = true;
    setup_indices(C, N, false);
    if (N.n > N.nvar) return layout_overflow(R);
    copy_vars<W>(C, M, N, Y, YT);
    double rhonu, pnu, clxnu, qnu, dpnu, pinu;
    nuf::rho_P(a * C.nu_masses[e], rhonu, pnu);
    NuBins lb;
    NuBins* bp;
    if constexpr (W == 1) bp = &lb;
    else bp = sbins(Wk) + e;
    NuBins& b = *bp;
    nu_bins<W>(C, a, e, b);
    nu_integrate<true, W>(C, M, Y, b, e, clxnu, qnu, dpnu, pinu);
    YT[N.nu_ix[e]] = clxnu / rhonu;
    YT[N.nu_ix[e] + 1] = dpnu / rhonu;
    YT[N.nu_ix[e] + 2] = qnu / rhonu;
    YT[N.nu_ix[e] + 3] = pinu / rhonu;
    // Nu_Intvsq (equations.f90:1331-1356) on the old layout
    double G11 = 0, G30 = 0;
    int ind = M.nu_ix[e];
    for (int iq = 0; iq < M.nq[e]; ++iq) {
      const double v = b.v[iq];
      G11 += C.nu_int_kernel[iq] * Y[ind + 1] * v * v;
      if (M.lmaxnu_tau[e] > 2) G30 += C.nu_int_kernel[iq] * Y[ind + 3] * v * v;
      ind += M.lmaxnu_tau[e] + 1;
    }
    N.G11[e] = G11 * a2 * a / rhonu;
    N.G30[e] = G30 * a2 * a / rhonu;
    M = N;
    swap_rows(R, Y, YT);
  } else {
    if (kind == SW_KTAU) {
      N.hk = true;
      for (int i = 0; i < C.nu_eig; ++i) N.nq[i] = C.nqmax;
    } else if (kind == SW_NU_MASSLESS) {
      N.nq[e] = next_nu_nq(C, M.nq[e]);
    } else if (kind == SW_NU_NONREL) {
      N.nonrel[e] = true;
    } else if (kind == SW_NONU) {
      R.reset = true;
      N.nonu = true;
      for (int i = 0; i < C.nu_eig; ++i) N.nq[i] = C.nqmax;
    } else if (kind == SW_NOPHOT) {
      R.reset = true;
      N.nophot = true;
    }
    setup_indices(C, N, false);
    if (N.n > N.nvar) return layout_overflow(R);
    copy_vars<W>(C, M, N, Y, YT);
    M = N;
    swap_rows(R, Y, YT);
  }
  R.fsal = false;
  wsync<W>();
}

// one trial step of RungeKuttaDP45 toward R.target; returns <0 on failure
template <bool TR, int W, class WK>
__device__ int trial_step(const DevCosmo& C, St& M, WK& Wk, Run& R) {
  using namespace dp;
  const double tol = C.tol1;
  const int n = M.n;
  const int lane = wlane<W>();
  NuBins* const sb = sbins(Wk);
  double* __restrict__ y = row(Wk, R.sy);
  double* __restrict__ yt = row(Wk, R.syt);
  double* __restrict__ k1 = row(Wk, R.sk1);
  double* __restrict__ k2 = row(Wk, R.sk2);  // also k6
  double* __restrict__ k3 = row(Wk, R.sk3);  // also the error combination
  double* __restrict__ k4 = row(Wk, R.sk4);  // also k7
  double* __restrict__ k5 = row(Wk, R.sk5);
  if (R.need_f) {
    if (R.fsal) R.fsal = false;
    else {
      rhs<TR, W>(C, M, R.tau, y, k1, nullptr, sb, wrec(Wk));
      wsync<W>();
      R.evals++;
    }
    R.need_f = false;
  }
  if (R.evals > kMaxEvalsPerMode) return -1;
  if (!R.ny_valid) {
    unsigned long long nb = 0;
    for (int i = lane; i < n; i += W) nb = max(nb, (unsigned long long)__double_as_longlong(y[i]) & 0x7fffffffffffffffULL);
    R.ny = __longlong_as_double((long long)wmax_u64<W>(nb));
    R.ny_valid = true;
  }
  const double ny = R.ny < 1.0 ? R.ny : 1.0;
  const double x = R.tau;
  const double hmin = 10.0 * fmax(tiny, eps * fmax(ny / tol, fabs(x)));
  const double hmax = R.call_hmax != 0.0 ? R.call_hmax : 20.0;
  if (hmin > hmax) return -2;
  if (R.first) {
    R.h = hmax * pow(tol, 0.2);
    R.first = false;
  } else if (R.fails <= 1) {
    const double g1 = 2.0 / 0.9, g2 = g1 * g1;
    double t2 = 2.0 * R.h;
    if (tol < g2 * g2 * g1 * R.err) t2 = 0.9 * fifth_root(tol / R.err) * R.h;
    R.h = fmax(t2, 0.5 * R.h);
  } else {
    R.h = 0.5 * R.h;
  }
  R.h = fmin(R.h, hmax);
  R.h = fmax(R.h, hmin);
  const double xend = R.target;
  const double rem = fabs(xend - x);
  double xt;
  if (R.h < rem && (rem > 1.2 * R.h || rem > hmax)) {
    R.h = fmin(R.h, 0.5 * rem);
    xt = x + copysign(R.h, xend - x);
  } else {
    R.h = rem;
    xt = xend;
  }
  const double hs = xt - x;
  const double c21 = hs * a21, c31 = hs * a31, c32 = hs * a32, c41 = hs * a41, c42 = hs * a42, c43 = hs * a43;
  const double c51 = hs * a51, c52 = hs * a52, c53 = hs * a53, c54 = hs * a54;
  const double c61 = hs * a61, c62 = hs * a62, c63 = hs * a63, c64 = hs * a64, c65 = hs * a65;
  const double cb1 = hs * b1, cb3 = hs * b3, cb4 = hs * b4, cb5 = hs * b5, cb6 = hs * b6;
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W) yt[i] = fma(c21, k1[i], y[i]);
  wsync<W>();
  rhs<TR, W>(C, M, x + hs / 5.0, yt, k2, nullptr, sb, wrec(Wk));
  wsync<W>();
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W) yt[i] = fma(c32, k2[i], fma(c31, k1[i], y[i]));
  wsync<W>();
  rhs<TR, W>(C, M, x + hs * (3.0 / 10.0), yt, k3, nullptr, sb, wrec(Wk));
  wsync<W>();
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W) yt[i] = fma(c43, k3[i], fma(c42, k2[i], fma(c41, k1[i], y[i])));
  wsync<W>();
  rhs<TR, W>(C, M, x + hs * (4.0 / 5.0), yt, k4, nullptr, sb, wrec(Wk));
  wsync<W>();
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W) yt[i] = fma(c54, k4[i], fma(c53, k3[i], fma(c52, k2[i], fma(c51, k1[i], y[i]))));
  wsync<W>();
  rhs<TR, W>(C, M, x + hs * (8.0 / 9.0), yt, k5, nullptr, sb, wrec(Wk));
  wsync<W>();
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W)
    yt[i] = fma(c65, k5[i], fma(c64, k4[i], fma(c63, k3[i], fma(c62, k2[i], fma(c61, k1[i], y[i])))));
  wsync<W>();
  rhs<TR, W>(C, M, x + hs, yt, k2, nullptr, sb, wrec(Wk));  // k6 into k2's row
  wsync<W>();
  // the fifth-order solution, the error combination of k1, k3..k6 (k3 is dead afterwards
  // and holds it) and max|yt| for the next step's hmin, in one pass
  unsigned long long nbt = 0;
#pragma unroll kStageUnroll
  for (int i = lane; i < n; i += W) {
    const double a1 = k1[i], a3 = k3[i], a4 = k4[i], a5 = k5[i], a6 = k2[i];
    const double v = fma(cb6, a6, fma(cb5, a5, fma(cb4, a4, fma(cb3, a3, fma(cb1, a1, y[i])))));
    yt[i] = v;
    k3[i] = fma(e6, a6, fma(e5, a5, fma(e4, a4, fma(e3, a3, e1 * a1))));
    nbt = max(nbt, (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL);
  }
  wsync<W>();
  // stage 7 (FSAL) into k4's row; at an output time it is the output() evaluation too
  const bool want_src = (xt == xend) && !R.target_is_switch && R.tgt_out;
  rhs<TR, W>(C, M, x + hs, yt, k4, want_src ? R.src : nullptr, sb, wrec(Wk));
  wsync<W>();
  R.src_valid = want_src;
  R.evals += 6;
  // mixed error norm max |e_i| / max(1, |y_i|) without a division per entry.  Where
  // |y_i| <= 1 the quotient is |e_i| itself, and non-negative doubles order as their bit
  // patterns, so those entries take an integer maximum off the FP64 pipe; only entries
  // with |y_i| > 1 compare cross-multiplied quotients.
  constexpr unsigned long long kAbs = 0x7fffffffffffffffULL, kOne = 0x3ff0000000000000ULL;
  unsigned long long m1 = 0;
  double num = 0, den = 1;
  for (int i = lane; i < n; i += W) {
    const double ee = fma(e7, k4[i], k3[i]);
    const unsigned long long be = (unsigned long long)__double_as_longlong(ee) & kAbs;
    const unsigned long long by = (unsigned long long)__double_as_longlong(y[i]) & kAbs;
    if (by <= kOne) {
      m1 = max(m1, be);
    } else {
      const double ae = __longlong_as_double((long long)be), ay = __longlong_as_double((long long)by);
      if (ae * den > num * ay) {
        num = ae;
        den = ay;
      }
    }
  }
  R.err = fmax(__longlong_as_double((long long)wmax_u64<W>(m1)), wmax<W>(num / den)) * R.h;
  if (R.err <= tol) {
    R.tau = xt;
    // accept: the trial state and k7 become y and k1 by swapping rows
    int t = R.sy;
    R.sy = R.syt;
    R.syt = t;
    t = R.sk1;
    R.sk1 = R.sk4;
    R.sk4 = t;
    R.ny = __longlong_as_double((long long)wmax_u64<W>(nbt));
    R.fails = 0;
    if (xt == xend) R.fsal = true;
  } else {
    R.fails++;
    if (R.h <= hmin) return -3;
  }
  return 0;
}

// The work loop: each thread (W = 1) or warp (W = 32) takes a mode from the queue and
// advances it one trial step per iteration.  The first item is the thread's (warp's)
// global index, so each block starts on consecutive queue entries independent of atomic
// ordering; later items come from the shared counter (past the statically assigned ones),
// or, when no counter is given, at a static stride of nstatic (items first, first +
// nstatic, first + 2 nstatic, ...), so that a warp's lanes keep neighbouring queue entries.
template <bool TR, int W, class WK>
__device__ __forceinline__ void run_modes(const DevCosmo* __restrict__ cosmos, const WorkItem* __restrict__ items,
                                          int nitems, int* __restrict__ counter, WK& Wk, int first, int nstatic) {
  St M;
  Run R;
  int cosmo = -1, q_ix = 0;
  const bool leader = wlane<W>() == 0;
  R.active = false;
  int next_static = first;
  for (;;) {
    if (!R.active) {
      int w = first;
      if (counter == nullptr) {
        w = next_static;
        if (w >= nitems) break;
        next_static += nstatic;
      } else if (first < 0) {
        int t = 0;
        if (leader) t = atomicAdd(counter, 1);
        if constexpr (W > 1) t = __shfl_sync(0xffffffffu, t, 0);
        w = nstatic + t;
      }
      first = -1;
      if (w >= nitems) break;
      const WorkItem it = items[w];
      if (it.cosmo < 0) continue;  // an empty slot of a balanced queue
      cosmo = it.cosmo;
      q_ix = it.mode;
      mode_init<W>(cosmos[cosmo], q_ix, M, Wk, R);
      if (!R.active) {
        if (leader) atomicExch(cosmos[cosmo].status, R.status);
        continue;
      }
      if (!next_target<TR>(cosmos[cosmo], M, R)) {
        R.active = false;
        if (leader) {
          if (R.status) atomicExch(cosmos[cosmo].status, R.status);
          atomicAdd(cosmos[cosmo].evals, (unsigned long long)R.evals);
        }
        continue;
      }
    }
    const DevCosmo& C = cosmos[cosmo];
    int rc = 0;
    if (R.target != R.tau) rc = trial_step<TR, W>(C, M, Wk, R);
    if (rc) {
      if (leader) {
        atomicExch(C.status, (int)CAMBGPU_ERROR_EVOLUTION);
        atomicAdd(C.evals, (unsigned long long)R.evals);
      }
      R.active = false;
      continue;
    }
    if (R.tau == R.target) {
      bool more = true;
      if (R.target_is_switch) {
        apply_switch<W>(C, M, Wk, R);
      } else if (TR && !R.tgt_out) {  // a source-time stop of the transfer path: no output
        stop_reached(C, R);
      } else {
        const bool out_src = TR && M.out_src;  // the CMB sources at a source-time stop
        if (!R.src_valid) {
          rhs<TR, W>(C, M, R.tau, row(Wk, R.sy), row(Wk, R.syt), R.src, sbins(Wk), wrec(Wk));
          wsync<W>();
        }
        R.evals++;  // the output() evaluation of the reference
        const int nk = C.nk;
        if (leader) {
          if (out_src) {
            const int nsrc = C.nsrc;
            for (int s = 0; s < nsrc; ++s) C.src_out[((size_t)R.js * nsrc + s) * C.src_nk + q_ix] = R.src[s];
          } else if constexpr (TR) {
            // TransferData is single precision: store, then divide the stored value by k^2
            float* o = C.transfer_out + ((size_t)R.j * nk + q_ix) * 13;
            o[0] = (float)R.src[0];
            for (int v = 1; v < 13; ++v) o[v] = (float)((double)(float)R.src[v] / M.k2);
          } else {
            const int nsrc = C.nsrc;
            for (int s = 0; s < nsrc; ++s) C.linear_src[((size_t)R.j * nsrc + s) * nk + q_ix] = R.src[s];
          }
        }
        R.src_valid = false;  // consumed (the next stop may be at the same time)
        if (out_src) {
          stop_reached(C, R);
        } else {
          R.j++;
          if (TR && R.stops) stop_reached(C, R);
        }
      }
      int guard = 0;
      for (;;) {
        if (R.status) {  // a switch that could not be applied
          more = false;
          break;
        }
        more = next_target<TR>(C, M, R);
        if (!more || !(R.target_is_switch && R.target == R.tau) || ++guard > 16) break;
        apply_switch<W>(C, M, Wk, R);  // switches due at the current time
      }
      if (guard > 16) R.status = CAMBGPU_ERROR_EVOLUTION, more = false;
      if (!more) {
        if (leader) {
          if (R.status) atomicExch(C.status, R.status);
          atomicAdd(C.evals, (unsigned long long)R.evals);
          if (C.mode_evals) C.mode_evals[q_ix] = (unsigned)R.evals;
        }
        R.active = false;
      }
    }
  }
}

template <int MINB, bool TR>
__global__ void __launch_bounds__(128, MINB) ode_thread_kernel(const DevCosmo* __restrict__ cosmos,
                                                               const WorkItem* __restrict__ items, int nitems,
                                                               int* __restrict__ counter) {
  Work Wk;
  run_modes<TR, 1>(cosmos, items, nitems, counter, Wk, blockIdx.x * blockDim.x + threadIdx.x,
                   gridDim.x * blockDim.x);
}

// Warp per mode, one warp per block: the block's dynamic shared memory holds the seven
// state rows of `stride` entries, the recurrence factors and the momentum-bin factors.
inline size_t warp_smem_bytes(int stride) { return ((size_t)kRows * stride + 3 * NL) * sizeof(double) + NUE * sizeof(NuBins); }

template <bool TR>
__global__ void __launch_bounds__(32) ode_warp_kernel(const DevCosmo* __restrict__ cosmos,
                                                      const WorkItem* __restrict__ items, int nitems,
                                                      int* __restrict__ counter, int stride) {
  extern __shared__ double wsm[];
  WorkS Wk;
  Wk.b = wsm;
  Wk.stride = stride;
  Wk.rec = wsm + (size_t)kRows * stride;
  Wk.bins = reinterpret_cast<NuBins*>(Wk.rec + 3 * NL);
  run_modes<TR, 32>(cosmos, items, nitems, counter, Wk, blockIdx.x, gridDim.x);
}

}  // namespace tpm

}  // namespace cgdev
