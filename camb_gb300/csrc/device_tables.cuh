// Device-side view of one cosmology's tables (device pointers), shared by the
// ODE, source-spline, line-of-sight and C_l kernels.
#pragma once
#include <cstdint>

#include "../../include/cambgpu.h"

namespace cgdev {

struct DevCosmo {
  // background
  double grhog, grhornomass, grhoc, grhob, grhov, tau0, taurend, tau_maxvis, matter_verydom_tau;
  double photbar_a;  // grhog/grhob: photon/baryon density ratio times a
  // massive neutrinos
  int nu_eig, nqmax;
  double nu_masses[3], grhormass[3], nu_tau_nonrel[3];
  const double* nu_q;
  const double* nu_int_kernel;
  const double* nu_tau_notmassless;  // [nu_eig][nqmax]
  // thermal history
  const double* thermo_horner;  // [nthermo][16]
  const double* dddotmu;
  const double* ddddotmu;
  const double* emmu;
  const double* demmu;
  int nthermo;
  double tauminn, inv_tauminn, dlntau, dlntau_inv;
  double cs2_end, dotmu_end, ddotmu_end, dddotmu_end, emmu_end;
  // time grid
  const double* tau_points;
  const double* tau_dpoints;
  int ntau;
  // source k grid
  const CambGpuModeSpec* modes;
  const double* q_evolve;
  int nk;
  // outputs / work
  double* linear_src;  // [ntau][nsrc][nk]
  double* dd_src;      // [ntau][nsrc][nk] spline second derivatives in k
  double* delta;       // [nq][nl][nsrc]
  double* icl;         // [nl][6]
  int* status;         // per-cosmology status word
  unsigned long long* evals;  // derivative evaluations (shared counter)
  // integration grid and l sampling
  const double* q_int;
  const double* dq_int;
  int nq;
  const int* ls;
  int nl;
  // Bessel table
  const double* bess_x;
  const double* bessel_horner;  // [nl][num_xx-1][4]
  int num_xx;
  // settings
  int nsrc, want_late_time;
  double max_etak_scalar, tol1, AccuracyBoost, IntTolBoost, TimeSwitchBoost, BessIntBoost, LimberBoost;
  double As, ns, nrun, pivot_scalar, Alens;
};

struct WorkItem {
  int cosmo;
  int mode;
};

}  // namespace cgdev
