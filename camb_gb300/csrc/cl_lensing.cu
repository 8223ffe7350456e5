// C_l interpolation to every l and CMB lensing of the C_l, on the device.
//
//  interp_cls_kernel    InterpolateCls / InterpolateClArrTemplated (cmbmain.f90:3523-3540,
//                       results.f90:1706-1824): natural cubic spline through the sampled l,
//                       TT/EE/TE on their difference from the high-L template.
//  lens_geom_kernel     the theta-dependent Legendre and Wigner-d recursions of
//                       CorrFuncFullSkyApodized (lensing.f90:440-502).  They depend only on
//                       the theta grid and lmax, so one table serves every cosmology that
//                       shares them and stays cached on the device.
//  lens_prep_kernel     PrepareLensedCLSpectra (lensing.f90:280-336) with the template tail.
//  lens_sigma_kernel    sigma^2(theta), C_gl,2(theta): sums over l of the d-table times the
//                       deflection spectrum, several cosmologies per d-table load.
//  lens_corr_kernel     the second-order correlation-function terms over the sub-sampled l
//                       (lensing.f90:504-613) and the end-of-range taper (:615-622).
//  lens_contrib_kernel  the back-projection sum over theta (lensing.f90:624-641) and the
//                       final lensed C_l (:646-660); one warp holds 32 cosmologies at one l,
//                       so each d-table load is a broadcast and the correlation loads coalesce.
//  pack_spectra_kernel  the CAMBdata getters (camb_python.f90:585-632) into output arrays.
// All arithmetic is FP64.
#include <cuda_runtime.h>

#include "device_tables.cuh"

namespace cgdev {

constexpr int kTmplLmax = 8000;
constexpr int kMaxNl = 512;
constexpr double kPi = 3.1415926535897932384626433832795;

// layout of the per-geometry d-table: [q][l][ii], ii = theta index (fastest)
enum { DQ_P = 0, DQ_DP, DQ_D11, DQ_DM11, DQ_D22, DQ_D2M2, DQ_D20, DQ_N };

__device__ __forceinline__ double tmpl_at(const double* __restrict__ tmpl, int l, int col) {
  return tmpl[(size_t)l * 4 + col];
}

// template value at l for the spline difference; scale != 1 interpolates the template at
// l/scale linearly (results.f90:1780-1793)
__device__ __forceinline__ double tmpl_scaled(const double* __restrict__ tmpl, int il, int col, double scale) {
  if (scale == 1.0) return tmpl_at(tmpl, il, col);
  double tl = il / scale;
  if (tl <= 1.0) return tmpl_at(tmpl, 1, col);
  if (tl >= kTmplLmax) return tmpl_at(tmpl, kTmplLmax, col);
  int lo = (int)tl;
  double frac = tl - lo;
  return (1.0 - frac) * tmpl_at(tmpl, lo, col) + frac * tmpl_at(tmpl, lo + 1, col);
}

// natural cubic spline second derivatives through (ls[i], y[i]), i < n (one thread)
__device__ void spline_d2_serial(const int* ls, const double* y, int n, double* d2, double* u) {
  if (n < 3) {
    for (int i = 0; i < n; ++i) d2[i] = 0;
    return;
  }
  d2[0] = 0;
  u[0] = 0;
  for (int i = 1; i < n - 1; ++i) {
    double x0 = ls[i - 1], x1 = ls[i], x2 = ls[i + 1];
    double sig = (x1 - x0) / (x2 - x0);
    double p = sig * d2[i - 1] + 2.0;
    d2[i] = (sig - 1.0) / p;
    double t = (y[i + 1] - y[i]) / (x2 - x1) - (y[i] - y[i - 1]) / (x1 - x0);
    u[i] = (6.0 * t / (x2 - x0) - sig * u[i - 1]) / p;
  }
  d2[n - 1] = 0;
  for (int k = n - 2; k >= 0; --k) d2[k] = d2[k] * d2[k + 1] + u[k];
}

// InterpolateClArr's evaluation at integer il: interval llo = last knot below il
__device__ double spline_eval(const int* ls, const double* y, const double* d2, int n, int il) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {  // first knot with ls >= il
    int mid = (lo + hi) >> 1;
    if (ls[mid] < il) lo = mid + 1;
    else hi = mid;
  }
  int llo = max(0, min(lo - 1, n - 2));
  int lhi = llo + 1;
  double ho = ls[lhi] - ls[llo];
  double a0 = (ls[lhi] - il) / ho, b0 = 1.0 - a0;
  return a0 * y[llo] + b0 * y[lhi] - a0 * b0 * ((1.0 + a0) * d2[llo] + (1.0 + b0) * d2[lhi]) * ho * ho / 6;
}

// grid (6 columns, cosmologies); all_cl must be zeroed
__global__ void __launch_bounds__(256) interp_cls_kernel(const DevCosmo* __restrict__ cosmos,
                                                         const double* __restrict__ tmpl) {
  const DevCosmo& C = cosmos[blockIdx.y];
  const int col = blockIdx.x;
  __shared__ int s_ls[kMaxNl];
  __shared__ double s_y[kMaxNl], s_d2[kMaxNl], s_u[kMaxNl], s_y2[kMaxNl], s_d22[kMaxNl];
  __shared__ int s_md, s_templ;
  __shared__ double s_scale;
  const int nl = C.nl;
  if (nl < 2 || nl > kMaxNl) return;
  for (int i = threadIdx.x; i < nl; i += blockDim.x) s_ls[i] = C.ls[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    double scale = C.cl_template_scale;
    int md = nl;
    int templ = col < 3;
    if (templ) {
      if (scale == 1.0) {
        while (md > 1 && s_ls[md - 1] > kTmplLmax) --md;
      } else {
        while (md > 1 && s_ls[md - 1] / scale > kTmplLmax) --md;
        if (s_ls[md - 1] / scale > kTmplLmax) {
          templ = 0;
          md = nl;
        }
      }
    }
    for (int i = 0; i < md; ++i) {
      double v = C.icl[(size_t)i * 6 + col];
      s_y[i] = templ ? v - tmpl_scaled(tmpl, s_ls[i], col, scale) : v;
    }
    spline_d2_serial(s_ls, s_y, md, s_d2, s_u);
    if (templ && md < nl) {
      for (int i = 0; i < nl; ++i) s_y2[i] = C.icl[(size_t)i * 6 + col];
      spline_d2_serial(s_ls, s_y2, nl, s_d22, s_u);
    }
    s_md = md;
    s_templ = templ;
    s_scale = scale;
  }
  __syncthreads();
  const int md = s_md, l0 = s_ls[0], ltop = s_ls[md - 1], lend = s_ls[nl - 1];
  const int lover = (s_templ && md < nl) ? s_ls[max(0, md - 3)] : lend + 1;
  for (int il = l0 + threadIdx.x; il <= lend; il += blockDim.x) {
    double v;
    if (il >= lover) v = spline_eval(s_ls, s_y2, s_d22, nl, il);
    else if (il <= ltop) {
      v = spline_eval(s_ls, s_y, s_d2, md, il);
      if (s_templ) v += tmpl_scaled(tmpl, il, col, s_scale);
    } else {
      v = 0;
    }
    C.all_cl[(size_t)il * 6 + col] = v;
  }
}

// ---- lensing ----

// Legendre and Wigner-d recursions for theta_i = (ii+1) dtheta, l in [2, lmax]
__global__ void lens_geom_kernel(double* __restrict__ tab, int lmin, int lmax, int npts, double dtheta) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= npts) return;
  const size_t L = (size_t)lmax + 1;
  auto at = [&](int q, int l) -> double& { return tab[((size_t)q * L + l) * npts + ii]; };
  const double theta = (ii + 1) * dtheta;
  const double x = cos(theta), sinth = sin(theta);
  const double s2 = sinth * sinth;
  if (lmin == 1) {
    double ch = cos(theta / 2), sh = sin(theta / 2);
    at(DQ_D11, 1) = ch * ch;
    at(DQ_DM11, 1) = sh * sh;
    at(DQ_P, 1) = x;
  }
  double pmm = 1, pmmp1 = x;
  const double fac1 = 1 - x, fac2 = 1 + x, fac = fac1 / fac2;
  for (int l = 2; l <= lmax; ++l) {
    const double Pl = ((2 * l - 1) * x * pmmp1 - (l - 1) * pmm) / l;
    const double dPl = l * (pmmp1 - x * Pl) / s2;
    pmm = pmmp1;
    pmmp1 = Pl;
    const double llp1 = (double)l * (l + 1), lf2 = (double)(l + 2) * (l - 1);
    at(DQ_P, l) = Pl;
    at(DQ_DP, l) = dPl;
    at(DQ_D11, l) = fac1 * dPl / llp1 + Pl;
    at(DQ_DM11, l) = fac2 * dPl / llp1 - Pl;
    at(DQ_D22, l) = (((4 * x - 8) / fac2 + llp1) * Pl + 4 * fac * (fac2 + (x - 2) / llp1) * dPl) / lf2;
    const double theta_cut = 0.244949 / sqrt(3.0 * llp1 - 8.0);
    double d2m2;
    if (theta > theta_cut)
      d2m2 = ((llp1 - (4 * x + 8) / fac1) * Pl + 4 / fac * (-fac1 + (x + 2) / llp1) * dPl) / lf2;
    else {
      const double t2 = theta * theta;
      d2m2 = llp1 * lf2 * (t2 * t2) * (1.0 / 384.0 - (3.0 * llp1 - 8.0) / 23040.0 * t2);
    }
    at(DQ_D2M2, l) = d2m2;
    at(DQ_D20, l) = (2 * x * dPl - llp1 * Pl) / sqrt(llp1 * lf2);
  }
}

__device__ __forceinline__ double cl_weight(int l) { return (2 * l + 1) / (4 * kPi) * (2 * kPi) / ((double)l * (l + 1)); }
__device__ __forceinline__ double phi_weight(int l) { return (l + 0.5) / ((double)(l + 1) * l); }

// prep[c][4][lmax+1]: Cphil3, CTT, CEE, CTE for l in [lmin, lmax]; grid (l blocks, nc)
__global__ void lens_prep_kernel(const DevCosmo* __restrict__ cosmos, const int* __restrict__ cidx,
                                 const double* __restrict__ tmpl, LensGeomDev G, double* __restrict__ prep) {
  const int c = blockIdx.y;
  const DevCosmo& C = cosmos[cidx[c]];
  const int l = G.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > G.lmax) return;
  const size_t L = (size_t)G.lmax + 1;
  double* P = prep + (size_t)c * 4 * L;
  const int ml = C.max_l;
  const double* cl = C.all_cl;
  double cp, tt, ee, te;
  if (l <= ml) {
    const double cpp = cl[(size_t)l * 6 + 3] * ((double)(l + 1) * (l + 1)) / ((double)l * l) / (2 * kPi);
    cp = cpp * phi_weight(l);
    const double fac = cl_weight(l);
    tt = cl[(size_t)l * 6 + 0] * fac;
    double x = (l - 2.0) / (20.0 - 2.0);
    double t = fmax(0.0, fmin(1.0, x));
    ee = cl[(size_t)l * 6 + 1] * fac * (t * t * (3.0 - 2.0 * t));  // LowLEELensingTaper
    te = cl[(size_t)l * 6 + 2] * fac;
    if (l == 10 && cp > 1e-7) atomicExch(C.status, (int)CAMBGPU_ERROR_UNSUPPORTED_PARAMS);
  } else {
    // tail from the template scaled to the spectra at max_l
    const double scm = cl_weight(ml);
    const double cpp_m = cl[(size_t)ml * 6 + 3] * ((double)(ml + 1) * (ml + 1)) / ((double)ml * ml) / (2 * kPi);
    const double ttm = cl[(size_t)ml * 6 + 0] * scm, eem = cl[(size_t)ml * 6 + 1] * scm;
    const double fac2 = ttm / (scm * tmpl_at(tmpl, ml, 0));
    const double fac3 = eem / (scm * tmpl_at(tmpl, ml, 1));
    const double tail_te = sqrt(fmax(0.0, fac2 * fac3));
    const double fac = cpp_m * phi_weight(ml) / (phi_weight(ml) * tmpl_at(tmpl, ml, 3));
    const double sc = cl_weight(l);
    cp = tmpl_at(tmpl, l, 3) * fac * phi_weight(l);
    tt = tmpl_at(tmpl, l, 0) * fac2 * sc;
    ee = tmpl_at(tmpl, l, 1) * fac3 * sc;
    te = tmpl_at(tmpl, l, 2) * tail_te * sc;
  }
  P[l] = cp;
  P[L + l] = tt;
  P[2 * L + l] = ee;
  P[3 * L + l] = te;
}

// sg[c][ii][2] = sigma^2, C_gl,2; grid (theta blocks of 128, cosmology groups of 8)
constexpr int kSigC = 8;
__global__ void __launch_bounds__(128) lens_sigma_kernel(LensGeomDev G, const double* __restrict__ prep, int nc,
                                                         double* __restrict__ sg) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= G.npts) return;
  const int c0 = blockIdx.y * kSigC;
  const int nloc = min(kSigC, nc - c0);
  const size_t L = (size_t)G.lmax + 1;
  const double* d11 = G.tab + (size_t)DQ_D11 * L * G.npts + ii;
  const double* dm11 = G.tab + (size_t)DQ_DM11 * L * G.npts + ii;
  double s[kSigC], g[kSigC];
#pragma unroll
  for (int k = 0; k < kSigC; ++k) s[k] = g[k] = 0;
  for (int l = G.lmin; l <= G.lmax; ++l) {
    const double a = d11[(size_t)l * G.npts], b = dm11[(size_t)l * G.npts];
    const double om = 1 - a;
#pragma unroll
    for (int k = 0; k < kSigC; ++k) {
      if (k < nloc) {
        const double cp = prep[(size_t)(c0 + k) * 4 * L + l];
        s[k] += om * cp;
        g[k] += b * cp;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kSigC; ++k) {
    if (k < nloc) {
      sg[((size_t)(c0 + k) * G.npts + ii) * 2] = s[k];
      sg[((size_t)(c0 + k) * G.npts + ii) * 2 + 1] = g[k];
    }
  }
}

// corr[k][ii][c]: the four correlation sums at theta_i; grid (theta blocks, nc)
__global__ void __launch_bounds__(128) lens_corr_kernel(LensGeomDev G, const double* __restrict__ prep,
                                                        const double* __restrict__ sg, int nc,
                                                        double* __restrict__ corr) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (ii >= G.npts) return;
  const size_t L = (size_t)G.lmax + 1;
  const double* CTT = prep + ((size_t)c * 4 + 1) * L;
  const double* CEE = prep + ((size_t)c * 4 + 2) * L;
  const double* CTE = prep + ((size_t)c * 4 + 3) * L;
  const double sigmasq = sg[((size_t)c * G.npts + ii) * 2], Cg2 = sg[((size_t)c * G.npts + ii) * 2 + 1];
  const double theta = (ii + 1) * G.dtheta;
  const double x = cos(theta), sinth = G.sinth[ii];
  const double fac1 = 1 - x, fac2 = 1 + x, sinfac = 4 / sinth;
  const double Cg2sq = Cg2 * Cg2;
  auto T = [&](int q, int l) { return G.tab[((size_t)q * L + l) * G.npts + ii]; };
  auto R = [&](int l) { return G.roots[l + 1]; };
  double c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  for (int j = 0; j < G.nj; ++j) {
    const int l = G.lsj[j];
    const double llp1 = (double)l * (l + 1), lf2 = (double)(l + 2) * (l - 1);
    const double rootllp1 = R(l) * R(l + 1), rootfac1 = R(l + 2) * R(l - 1), rootfac2 = R(l + 3) * R(l - 2);
    const double Pl = T(DQ_P, l), dPl = T(DQ_DP, l), d11 = T(DQ_D11, l), dm11 = T(DQ_DM11, l);
    double d2m2 = 0, d22 = 0, d20 = 0, d1m2 = 0, d12 = 0;
    if (l >= 2) {
      d2m2 = T(DQ_D2M2, l);
      d22 = T(DQ_D22, l);
      d20 = T(DQ_D20, l);
      d1m2 = sinth / rootfac1 * (dPl - 2 / fac1 * dm11);
      d12 = sinth / rootfac1 * (dPl - 2 / fac2 * d11);
    }
    double d1m3 = 0, d2m3 = 0, d3m3 = 0, d13 = 0;
    if (l >= 3) {
      d1m3 = (-(x + 0.5) * d1m2 * sinfac - lf2 * dm11 / rootfac1) / rootfac2;
      d2m3 = (-fac2 * d2m2 * sinfac - rootfac1 * d1m2) / rootfac2;
      d3m3 = (-(x + 1.5) * d2m3 * sinfac - rootfac1 * d1m3) / rootfac2;
      d13 = ((x - 0.5) * d12 * sinfac - lf2 * d11 / rootfac1) / rootfac2;
    }
    double d04 = 0, d2m4 = 0, d4m4 = 0, rootfac3 = 0;
    if (l >= 4) {
      rootfac3 = R(l - 3) * R(l + 4);
      d04 = ((-llp1 + (18 * x * x + 6) / (sinth * sinth)) * d20 - 6 * x * lf2 * dPl / sqrt(llp1 * lf2)) /
            (rootfac2 * rootfac3);
      d2m4 = (-(6 * x + 4) * d2m3 / sinth - rootfac2 * d2m2) / rootfac3;
      d4m4 = (-7 / 5.0 * (llp1 - 6) * d2m2 + 12 / 5.0 * (-llp1 + (9 * x + 26) / fac1) * d3m3) / (llp1 - 12);
    }
    const double X000 = exp(-llp1 * sigmasq / 4);
    const double X022 = X000 * (1 + sigmasq);
    const double X220 = sqrt(llp1 * lf2) / 4 * X000;
    const double X121 = -0.5 * rootfac1 * X000;
    const double X132 = -0.5 * rootfac2 * X000;
    const double X242 = 0.25 * rootfac2 * rootfac3 * X022;
    const double dX000 = -llp1 / 4 * X000;
    const double dX022 = (1 - llp1 / 4) * X022;
    const double f1 = dX000 * dX000, f3 = X220 * X220;
    const double sc = j >= 14 ? (double)G.interp_fac : 1.0;
    double fac = ((X000 * X000 - 1) + Cg2sq * f1) * Pl + Cg2sq * f3 * d2m2 + 8 / llp1 * f1 * Cg2 * dm11;
    c0 += sc * CTT[l] * fac;
    const double f2 = (Cg2 * dX022) * (Cg2 * dX022) + (X022 * X022 - 1);
    fac = 2 * Cg2 * X121 * X132 * d13 + f2 * d22 + Cg2sq * X242 * X220 * d04;
    c1 += sc * CEE[l] * fac;
    fac = (f3 * Pl + X242 * X242 * d4m4) * Cg2sq / 2 + Cg2 * (X121 * X121 * dm11 + X132 * X132 * d3m3) + f2 * d2m2;
    c2 += sc * CEE[l] * fac;
    fac = (X000 * X022 - 1) * d20 + 2 * dX000 * Cg2 * (X121 * d11 + X132 * d1m3) / rootllp1 +
          Cg2sq * (X220 / 2 * d2m4 * X242 + (f3 / 2 + dX022 * dX000) * d20);
    c3 += sc * CTE[l] * fac;
  }
  const int i = ii + 1;
  if (i > G.npoints - G.apodize_point_width) {
    double taper = (double)(G.npoints - i) / (double)G.apodize_point_width;
    taper = fmax(0.0, fmin(1.0, taper));
    taper = taper * taper * taper * (10.0 + taper * (-15.0 + 6.0 * taper));
    c0 *= taper;
    c1 *= taper;
    c2 *= taper;
    c3 *= taper;
  }
  const size_t st = (size_t)G.npts * nc;
  corr[(size_t)ii * nc + c] = c0;
  corr[st + (size_t)ii * nc + c] = c1;
  corr[2 * st + (size_t)ii * nc + c] = c2;
  corr[3 * st + (size_t)ii * nc + c] = c3;
}

// lensed C_l: block (32 cosmologies, 8 l), grid (l blocks, cosmology blocks)
__global__ void __launch_bounds__(256) lens_contrib_kernel(const DevCosmo* __restrict__ cosmos,
                                                           const int* __restrict__ cidx, LensGeomDev G,
                                                           const double* __restrict__ corr, int nc, int lmax_out) {
  const int c = blockIdx.y * 32 + threadIdx.x;
  const int l = G.lmin + blockIdx.x * 8 + threadIdx.y;
  if (c >= nc || l > lmax_out) return;
  const DevCosmo& C = cosmos[cidx[c]];
  if (l > C.lmax_lensed) return;
  const size_t L = (size_t)G.lmax + 1;
  const double* tP = G.tab + ((size_t)DQ_P * L + l) * G.npts;
  const double* t22 = G.tab + ((size_t)DQ_D22 * L + l) * G.npts;
  const double* t2m2 = G.tab + ((size_t)DQ_D2M2 * L + l) * G.npts;
  const double* t20 = G.tab + ((size_t)DQ_D20 * L + l) * G.npts;
  const size_t st = (size_t)G.npts * nc;
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (int ii = 0; ii < G.npts; ++ii) {
    const double s = G.sinth[ii], hs = s / 2;
    const size_t o = (size_t)ii * nc + c;
    a0 += corr[o] * tP[ii] * s;
    const double T2 = corr[st + o] * t22[ii], T4 = corr[2 * st + o] * t2m2[ii];
    a1 += (T2 + T4) * hs;
    a2 += (T2 - T4) * hs;
    a3 += corr[3 * st + o] * t20[ii] * s;
  }
  const double fac = (double)l * (l + 1) / (2 * kPi) * G.dtheta * (2 * kPi);
  const double* u = C.all_cl + (size_t)l * 6;
  double* o = C.lensed + (size_t)l * 4;
  o[0] = a0 * fac + u[0];
  o[1] = a1 * fac + u[1];
  o[2] = a2 * fac;
  o[3] = a3 * fac + u[2];
}

// CAMB_SetUnlensedScalCls / SetlensedScalCls / SetLensPotentialCls (camb_python.f90:585-632)
// into [n][lmax_out+1][4], [n][lmax_out+1][4], [n][lmax_out+1][3]; grid (l blocks, n)
__global__ void pack_spectra_kernel(const DevCosmo* __restrict__ cosmos, int lmax_out, double* __restrict__ unl,
                                    double* __restrict__ len, double* __restrict__ pot) {
  const int c = blockIdx.y;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l > lmax_out) return;
  const DevCosmo& C = cosmos[c];
  const double* a = C.all_cl + (size_t)l * 6;
  const bool in = l >= 2 && l <= C.max_l;
  if (unl) {
    double* o = unl + ((size_t)c * (lmax_out + 1) + l) * 4;
    o[0] = in ? a[0] : 0.0;
    o[1] = in ? a[1] : 0.0;
    o[2] = 0.0;
    o[3] = in ? a[2] : 0.0;
  }
  if (len) {
    double* o = len + ((size_t)c * (lmax_out + 1) + l) * 4;
    const bool li = C.lensed && l >= 2 && l <= C.lmax_lensed;
    for (int k = 0; k < 4; ++k) o[k] = li ? C.lensed[(size_t)l * 4 + k] : 0.0;
  }
  if (pot) {
    double* o = pot + ((size_t)c * (lmax_out + 1) + l) * 3;
    if (in && C.lensed) {
      // the reference forms these factors in default (single) precision: real(l + 1)/l
      const float r = (float)(l + 1) / (float)l;
      const float r2 = r * r, r15 = powf(r, 1.5f);
      o[0] = a[3] * (double)r2 / (2 * kPi);
      o[1] = a[4] * ((double)r15 / (2 * kPi));
      o[2] = a[5] * ((double)r15 / (2 * kPi));
    } else {
      o[0] = o[1] = o[2] = 0.0;
    }
  }
}

// Transfer_Get_sigmas (results.f90:4115-4182) at R = 8 Mpc/h: trapezoid in ln k over the
// transfer k grid of the single-precision transfer functions, delta = total matter
// (Transfer_tot) and v = Newtonian CDM velocity; one thread per (cosmology, redshift),
// summing in the reference's k order.
__global__ void sigma8_kernel(const DevCosmo* __restrict__ cosmos, int n) {
  const int c = blockIdx.x;
  const int z = threadIdx.x;
  if (c >= n) return;
  const DevCosmo& C = cosmos[c];
  if (!C.transfer_only || z >= C.n_tt) return;
  const int nk = C.nk;
  const double h = C.hubble_h;
  double lnko = 0, dsig8o = 0, sig8 = 0, dsigvo = 0, sigv = 0;
  for (int ik = 0; ik < nk; ++ik) {
    const double kh = C.transfer_out[(size_t)ik * 13];
    if (kh == 0) continue;
    const double k = kh * h;
    const float* T = C.transfer_out + ((size_t)z * nk + ik) * 13;
    const double delta = T[6];
    double dsig8 = delta * delta;
    double dsigv = delta * (double)T[10];
    const double x = kh * 8.0;
    const double win = x < 1e-2 ? 1.0 - x * x / 10 : 3 * (sin(x) - x * cos(x)) / (x * x * x);
    const double lnk = log(k);
    const double dlnk = ik == 0 ? 0.5 : lnk - lnko;
    const double lnrat = log(k / C.pivot_scalar);
    const double pk = C.As * exp(lnrat * (C.ns - 1 + lnrat * (C.nrun / 2)));
    const double powers = (win * k * k) * (win * k * k) * pk;
    dsig8 = powers * dsig8;
    sig8 += (dsig8 + dsig8o) * dlnk / 2;
    dsig8o = dsig8;
    dsigv = powers * dsigv;
    sigv += (dsigv + dsigvo) * dlnk / 2;
    dsigvo = dsigv;
    lnko = lnk;
  }
  C.sigma8[2 * z] = sqrt(sig8);
  C.sigma8[2 * z + 1] = sigv;
}

// ---- launch helpers (called from the C API) ----
cudaError_t launch_sigma8(const DevCosmo* cosmos, int n, cudaStream_t s) {
  sigma8_kernel<<<n, 32, 0, s>>>(cosmos, n);
  return cudaGetLastError();
}

cudaError_t launch_interp_cls(const DevCosmo* cosmos, int n, const double* tmpl, cudaStream_t s) {
  interp_cls_kernel<<<dim3(6, n), 256, 0, s>>>(cosmos, tmpl);
  return cudaGetLastError();
}

cudaError_t launch_lens_geom(double* tab, int lmin, int lmax, int npts, double dtheta, cudaStream_t s) {
  lens_geom_kernel<<<(npts + 63) / 64, 64, 0, s>>>(tab, lmin, lmax, npts, dtheta);
  return cudaGetLastError();
}

cudaError_t launch_lensing(const DevCosmo* cosmos, const int* cidx, int nc, const double* tmpl,
                           const LensGeomDev& G, int lmax_lensed_max, double* prep, double* sg, double* corr,
                           cudaStream_t s) {
  lens_prep_kernel<<<dim3((G.lmax - G.lmin + 1 + 255) / 256, nc), 256, 0, s>>>(cosmos, cidx, tmpl, G, prep);
  lens_sigma_kernel<<<dim3((G.npts + 127) / 128, (nc + kSigC - 1) / kSigC), 128, 0, s>>>(G, prep, nc, sg);
  lens_corr_kernel<<<dim3((G.npts + 127) / 128, nc), 128, 0, s>>>(G, prep, sg, nc, corr);
  lens_contrib_kernel<<<dim3((lmax_lensed_max - G.lmin + 1 + 7) / 8, (nc + 31) / 32), dim3(32, 8), 0, s>>>(
      cosmos, cidx, G, corr, nc, lmax_lensed_max);
  return cudaGetLastError();
}

cudaError_t launch_pack_spectra(const DevCosmo* cosmos, int n, int lmax_out, double* unl, double* len, double* pot,
                                cudaStream_t s) {
  pack_spectra_kernel<<<dim3((lmax_out + 1 + 127) / 128, n), 128, 0, s>>>(cosmos, lmax_out, unl, len, pot);
  return cudaGetLastError();
}

}  // namespace cgdev
