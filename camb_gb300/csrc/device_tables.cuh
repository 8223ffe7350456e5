// Device-side view of one cosmology's tables (device pointers), shared by the
// ODE, source-spline, line-of-sight and C_l kernels.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/cambgpu.h"

namespace cgdev {

constexpr int kBessSegMax = 8;
constexpr int kTimeSegMax = 8;

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
  const double* nu_inv_q;            // 1/nu_q
  double photbar_fac;                // 3/(4 photbar_a)
  // thermal history
  const double* thermo_horner;  // [nthermo][16]
  const double* dddotmu;
  const double* ddddotmu;
  const double* emmu;
  const double* demmu;
  int nthermo;
  double tauminn, inv_tauminn, dlntau, dlntau_inv;
  const double* inv_tgrid;  // [nthermo+1] 1/(tauminn exp(j dlntau)), the ideal log grid
  float dlntau_inv_log2;    // ln 2 / dlntau
  double cs2_end, dotmu_end, ddotmu_end, dddotmu_end, emmu_end;
  // time grid
  const double* tau_points;
  const double* tau_dpoints;
  const double* tau_dist;  // [ntau] tau0 - tau_i (mixed projection staging)
  const float* tau_dpf;     // [ntau] dtau_i in FP32 (mixed projection staging)
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
  double* all_cl;      // [max_l+1][6] InterpolateCls output, TT EE TE PP PT PE
  double* lensed;      // [lmax_lensed+1][4] TT EE BB TE (lensed cosmologies only)
  int max_l, lmax_lensed;
  double cl_template_scale;
  // matter transfer functions only: every mode evolved to each transfer time
  int transfer_only, n_tt, want_cls;
  const double* transfer_times;  // [n_tt], increasing
  float* transfer_out;           // [n_tt][nk][13] (TransferData order, single precision)
  double* sigma8;                // [n_tt][2]: sigma8, sigma2_vdelta_8
  double hubble_h, late_phot_boost_min;
  int* status;         // per-cosmology status word
  unsigned long long* evals;  // derivative evaluations (shared counter)
  unsigned* mode_evals;       // [nk] evaluations of each mode in the last run (queue ordering)
  // integration grid and l sampling
  const double* q_int;
  const double* dq_int;
  int nq;
  double* pk_w;  // [nq] A_s P(q) dq/q of the current primordial power (the C_l k-integral weights)
  const int* ls;
  int nl;
  const double* l_xlim;  // [nl] max(0, l - 4.2 l^(1/3))
  const double* l_limb;  // [nl] sqrt(pi / (2 l + 1))
  const double* l_doint;  // [nl] max(850, l) 3 BessIntBoost / tau0 1.2 (lensed-run integration test)
  // Bessel table
  const double* bess_x;
  const double* bessel_horner;  // [nl][num_xx-1][4]
  const float4* bessel_f32;     // [nl][num_xx-1] the same coefficients in FP32 (mixed precision)
  const float* bess_inv_dxf;    // [num_xx-1] 1 / (x_{i+1} - x_i) in FP32
  // the x grid as runs of uniform spacing (nseg = 0: none recorded, bisect instead)
  int nseg;
  double seg_x0[kBessSegMax];   // first point of each run
  double seg_inv_h[kBessSegMax];
  int seg_i0[kBessSegMax];      // grid index of the first point
  int seg_n[kBessSegMax];       // intervals in the run
  // the source time grid as runs of uniform spacing (ntseg = 0: more than kTimeSegMax)
  int ntseg;
  double tseg_x0[kTimeSegMax], tseg_inv_h[kTimeSegMax];
  int tseg_i0[kTimeSegMax], tseg_n[kTimeSegMax];
  int num_xx;
  // settings
  int nsrc, want_late_time;
  double src_keep_tau;  // source modes keep evolving until tau passes it (runs with transfers)
  int tr_src_modes;     // transfer path: leading modes that also stop at the source times
  double* src_out;      // and store their CMB sources there ([ntau][nsrc][src_nk]), or null
  int src_nk;
  double max_etak_scalar, tol1, AccuracyBoost, IntTolBoost, TimeSwitchBoost, BessIntBoost, LimberBoost;
  double As, ns, nrun, pivot_scalar, Alens;
};

struct WorkItem {
  int cosmo;
  int mode;
};

// theta grid and Legendre / Wigner-d table of the lensing correlation sums
struct LensGeomDev {
  const double* tab;     // [7][lmax+1][npts]: P, dP, d11, d-11, d22, d2-2, d20
  const double* roots;   // sqrt(l) at [l+1], l in [-1, lmax+4]
  const double* sinth;   // [npts]
  const int* lsj;        // sub-sampled l of the correlation sums
  int nj, lmin, lmax, npts, npoints, apodize_point_width, interp_fac;
  double dtheta;
};

extern const double kHighLTemplate[8001 * 4];  // TT EE TE PP by l (generated at build time)

cudaError_t launch_interp_cls(const DevCosmo* cosmos, int n, const double* tmpl, cudaStream_t s);
cudaError_t launch_lens_geom(double* tab, int lmin, int lmax, int npts, double dtheta, cudaStream_t s);
cudaError_t launch_lensing(const DevCosmo* cosmos, const int* cidx, int nc, const double* tmpl,
                           const LensGeomDev& G, int lmax_lensed_max, double* prep, double* sg, double* corr,
                           cudaStream_t s);
cudaError_t launch_pack_spectra(const DevCosmo* cosmos, int n, int lmax_out, double* unl, double* len, double* pot,
                                cudaStream_t s);

}  // namespace cgdev
