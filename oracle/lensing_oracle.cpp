// ORACLE -- test infrastructure only.
//
// CPU restatement of the reference's C_l interpolation and CMB lensing, used by
// tests/ as the checker of the CUDA library.  Nothing in the product links or calls
// this file.  It follows, in scalar form with the reference's index conventions:
//   InterpolateClArr / InterpolateClArrTemplated   fortran/results.f90:1706-1824
//   InterpolateCls (template per spectrum)         fortran/cmbmain.f90:3523-3540
//   LensingExtrapLmax / InitLensedClArrays         fortran/lensing.f90:161-177, 230-247
//   LensingClWeight / LensingPhiWeight             fortran/lensing.f90:249-278
//   PrepareLensedCLSpectra (template tail)         fortran/lensing.f90:280-336
//   CorrFuncFullSkyApodized (lensing method 1)     fortran/lensing.f90:338-678
//   CorrFuncFullSky (lensing method 4)             fortran/lensing.f90:680-941
// The template is the [8001][4] table (TT, EE, TE, PP rows by l) the reference loads
// from HighLExtrapTemplate_lenspotentialCls.dat (config.f90:93-116).
#include <algorithm>
#include <cmath>
#include <vector>

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;
constexpr int kTemplateLmax = 8000;  // lmax_extrap_highl, config.f90:55
constexpr int kConvolutionGap = 50;  // lens_convolution_gap, config.f90:60

inline double T_(const double* tmpl, int l, int col) { return tmpl[(size_t)l * 4 + col]; }

// forutils cubic_spline_second_derivs with natural end conditions
void spline_d2(const double* x, const double* y, int n, double* d2) {
  std::vector<double> u(n);
  if (n < 3) {
    for (int i = 0; i < n; ++i) d2[i] = 0;
    return;
  }
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

// InterpolateClArr: spline of iCl[0..max_ind) on ls to every l in [ls[0], ls[max_ind-1]]
// written to all[l]
void interp_arr(const int* ls, const double* iCl, int max_ind, double* all) {
  std::vector<double> xl(max_ind), d2(max_ind);
  for (int i = 0; i < max_ind; ++i) xl[i] = ls[i];
  spline_d2(xl.data(), iCl, max_ind, d2.data());
  int llo = 0;  // 0-based
  for (int il = ls[0]; il <= ls[max_ind - 1]; ++il) {
    if (il > ls[llo + 1] && llo + 1 < max_ind) ++llo;
    int lhi = std::min(llo + 1, max_ind - 1);
    double ho = ls[lhi] - ls[llo];
    double a0 = (ls[lhi] - il) / ho, b0 = 1.0 - a0;
    all[il] = a0 * iCl[llo] + b0 * iCl[lhi] - a0 * b0 * ((1.0 + a0) * d2[llo] + (1.0 + b0) * d2[lhi]) * ho * ho / 6;
  }
}

// InterpolateClArrTemplated for template column col (TT 0, EE 1, TE 2)
void interp_templated(const int* ls, int nl, const double* iCl, const double* tmpl, int col, double scale,
                      double* all) {
  int maxdelta = nl;
  std::vector<double> delta(nl);
  if (scale == 1.0) {
    while (ls[maxdelta - 1] > kTemplateLmax) --maxdelta;
    for (int i = 0; i < maxdelta; ++i) delta[i] = iCl[i] - T_(tmpl, ls[i], col);
    interp_arr(ls, delta.data(), maxdelta, all);
    for (int il = ls[0]; il <= ls[maxdelta - 1]; ++il) all[il] += T_(tmpl, il, col);
  } else {
    while (maxdelta > 1 && ls[maxdelta - 1] / scale > kTemplateLmax) --maxdelta;
    if (ls[maxdelta - 1] / scale > kTemplateLmax) {
      interp_arr(ls, iCl, nl, all);
      return;
    }
    int lo_l = ls[0], hi_l = ls[maxdelta - 1];
    std::vector<double> tc(hi_l + 1);
    for (int il = lo_l; il <= hi_l; ++il) {
      double tl = il / scale;
      if (tl <= 1.0) tc[il] = T_(tmpl, 1, col);
      else if (tl >= kTemplateLmax) tc[il] = T_(tmpl, kTemplateLmax, col);
      else {
        int lo = (int)tl;
        double frac = tl - lo;
        tc[il] = (1.0 - frac) * T_(tmpl, lo, col) + frac * T_(tmpl, lo + 1, col);
      }
    }
    for (int i = 0; i < maxdelta; ++i) delta[i] = iCl[i] - tc[ls[i]];
    interp_arr(ls, delta.data(), maxdelta, all);
    for (int il = lo_l; il <= hi_l; ++il) all[il] += tc[il];
  }
  if (maxdelta < nl) {
    std::vector<double> tmp(ls[nl - 1] + 1);
    interp_arr(ls, iCl, nl, tmp.data());
    for (int il = ls[maxdelta - 3]; il <= ls[nl - 1]; ++il) all[il] = tmp[il];
  }
}

double cl_weight(int l) { return (2 * l + 1) / (4 * kPi) * (2 * kPi) / ((double)l * (l + 1)); }
double phi_weight(int l) { return (l + 0.5) / ((double)(l + 1) * l); }
double ee_taper(int l) {
  double x = (l - 2.0) / (20.0 - 2.0);
  double t = std::max(0.0, std::min(1.0, x));
  return t * t * (3.0 - 2.0 * t);
}

// Weighted spectra for l in [lmin, lmax] (PrepareLensedCLSpectra, curved-sky weights,
// EE taper on).  cl: [max_l+1][4] TT EE TE and Cl_scalar(C_Phi).  Returns false when
// the lensing amplitude check of the reference fails.
bool prepare_spectra(const double* cl, int max_l, int lmin, int lmax, const double* tmpl, std::vector<double>& Cphil3,
                     std::vector<double>& CTT, std::vector<double>& CEE, std::vector<double>& CTE) {
  Cphil3.assign(lmax + 1, 0);
  CTT.assign(lmax + 1, 0);
  CEE.assign(lmax + 1, 0);
  CTE.assign(lmax + 1, 0);
  for (int l = lmin; l <= max_l; ++l) {
    double cpp = cl[(size_t)l * 4 + 3] * ((double)(l + 1) * (l + 1)) / ((double)l * l) / (2 * kPi);
    Cphil3[l] = cpp * phi_weight(l);
    double fac = cl_weight(l);
    CTT[l] = cl[(size_t)l * 4 + 0] * fac;
    CEE[l] = cl[(size_t)l * 4 + 1] * fac * ee_taper(l);
    CTE[l] = cl[(size_t)l * 4 + 2] * fac;
  }
  if (max_l >= 10 && Cphil3[10] > 1e-7) return false;
  if (lmax > max_l) {
    int l = max_l;
    double sc = cl_weight(l);
    double fac2 = CTT[max_l] / (sc * T_(tmpl, max_l, 0));
    double fac3 = CEE[max_l] / (sc * T_(tmpl, max_l, 1));
    double tail_te = std::sqrt(std::max(0.0, fac2 * fac3));
    double fac = Cphil3[max_l] / (phi_weight(l) * T_(tmpl, max_l, 3));
    for (l = max_l + 1; l <= lmax; ++l) {
      sc = cl_weight(l);
      Cphil3[l] = T_(tmpl, l, 3) * fac * phi_weight(l);
      CTT[l] = T_(tmpl, l, 0) * fac2 * sc;
      CEE[l] = T_(tmpl, l, 1) * fac3 * sc;
      CTE[l] = T_(tmpl, l, 2) * tail_te * sc;
    }
  }
  return true;
}

}  // namespace

extern "C" {

// Lensing l range: LensingExtrapLmax and InitLensedClArrays.  out2 = {lmax, lmax_lensed}.
void oracle_lensing_lrange(const int* ls, int nl, int max_l, int lens_output_margin, double lens_accuracy_boost,
                           int* out2) {
  int output_lmax = max_l - lens_output_margin;
  int extrap = std::max(750, (int)std::ceil((0.45 * output_lmax + 400.0) * lens_accuracy_boost));
  int lmax = output_lmax + kConvolutionGap + extrap;
  lmax = std::min(kTemplateLmax, lmax);
  lmax = std::max(lmax, max_l);
  int ix = nl - 2;  // max_lensed_ix = nl - 1 (1-based)
  while (ls[ix] > max_l - (lens_output_margin - kConvolutionGap)) --ix;
  out2[0] = lmax;
  out2[1] = std::max(ls[ix], max_l - lens_output_margin);
}

// InterpolateCls: icl [nl][6] (TT EE TE PP TP EP) at the sampled ls to all[l][6] for
// l in [ls[0], ls[nl-1]]; TT, EE, TE on the difference from the template.
void oracle_interpolate_cls(const int* ls, int nl, const double* icl, const double* tmpl, double scale,
                            double* all) {
  const double template_scale = std::fabs(scale - 1.0) > 0.01 ? scale : 1.0;  // results.f90:1517-1520
  int lmax = ls[nl - 1];
  std::vector<double> col(nl), out(lmax + 1);
  for (int c = 0; c < 6; ++c) {
    for (int i = 0; i < nl; ++i) col[i] = icl[(size_t)i * 6 + c];
    std::fill(out.begin(), out.end(), 0.0);
    if (c < 3) interp_templated(ls, nl, col.data(), tmpl, c, template_scale, out.data());
    else interp_arr(ls, col.data(), nl, out.data());
    for (int l = ls[0]; l <= lmax; ++l) all[(size_t)l * 6 + c] = out[l];
  }
}

// CorrFuncFullSkyApodized (AccurateBB false).  cl: [max_l+1][4] TT EE TE Cl_scalar(C_Phi);
// out: [lmax_lensed+1][4] TT EE BB TE for l in [lmin, lmax_lensed].  Returns 0, or 1
// when the lensing amplitude check fails.
int oracle_lens_cls_apodized(const double* cl, int max_l, int lmin, int lmax, int lmax_lensed,
                             int lens_output_margin, double lens_accuracy_boost, const double* tmpl, double* out) {
  std::vector<double> Cphil3, CTT, CEE, CTE;
  if (!prepare_spectra(cl, max_l, lmin, lmax, tmpl, Cphil3, CTT, CEE, CTE)) return 1;
  double high_l_lensed_lmax = (double)(max_l - lens_output_margin);
  double ramp = std::min(1.0, std::max(0.0, (high_l_lensed_lmax - 2500.0) / 1000.0));
  ramp = ramp * ramp * (3.0 - 2.0 * ramp);
  double LensRangeBoost = lens_accuracy_boost;
  double ThetaSampleBoost = lens_accuracy_boost * (1.6 + 0.6 * ramp);  // AccuracyTarget > 0
  int npoints = (int)(max_l * 2 * ThetaSampleBoost);
  double dtheta = kPi / npoints;
  int apodize_point_width = (int)std::lround(0.012 / dtheta);
  npoints = (int)(kPi / dtheta);
  double range_fac = std::max(1.0, 32 / LensRangeBoost);
  npoints = (int)(npoints / range_fac);
  int interp_fac = std::max(1, std::min((int)std::lround(10 / LensRangeBoost), (int)(range_fac * 2) - 1));
  std::vector<int> lsj;
  std::vector<double> lfacs(lmax + 1), lfacs2(lmax + 1), lrootfacs(lmax + 1), theta_cut(lmax + 1), roots(lmax + 6);
  for (int l = lmin; l <= lmax; ++l) {
    if (l <= 15 || (l - 15) % interp_fac == interp_fac / 2) lsj.push_back(l);
    lfacs[l] = (double)l * (l + 1);
    lfacs2[l] = (double)(l + 2) * (l - 1);
    lrootfacs[l] = std::sqrt(lfacs[l] * lfacs2[l]);
  }
  for (int l = 2; l <= lmax; ++l) theta_cut[l] = 0.244949 / std::sqrt(3.0 * lfacs[l] - 8.0);
  for (int l = 0; l <= lmax + 4; ++l) roots[l + 1] = std::sqrt((double)l);  // roots(l) at [l+1]
  roots[0] = 0;                                                              // roots(-1)
  auto R = [&](int l) { return roots[l + 1]; };
  std::vector<double> contrib((size_t)(lmax_lensed + 1) * 4, 0.0);
  std::vector<double> P(lmax + 1), dP(lmax + 1), d_11(lmax + 1), d_m11(lmax + 1), d_22(lmax + 1), d_2m2(lmax + 1),
      d_20(lmax + 1);
  for (int i = 1; i <= npoints - 1; ++i) {
    double theta = i * dtheta;
    double x = std::cos(theta), sinth = std::sin(theta), halfsinth = sinth / 2;
    double pmm = 1, pmmp1 = x, Cg2 = 0, sigmasq = 0;
    if (lmin == 1) {
      d_11[1] = std::cos(theta / 2) * std::cos(theta / 2);
      d_m11[1] = std::sin(theta / 2) * std::sin(theta / 2);
      sigmasq += (1 - d_11[1]) * Cphil3[lmin];
      Cg2 += d_m11[1] * Cphil3[lmin];
      P[1] = x;
      d_22[1] = d_2m2[1] = d_20[1] = 0;
    }
    for (int l = 2; l <= lmax; ++l) {
      P[l] = ((2 * l - 1) * x * pmmp1 - (l - 1) * pmm) / l;
      dP[l] = l * (pmmp1 - x * P[l]) / (sinth * sinth);
      pmm = pmmp1;
      pmmp1 = P[l];
      double llp1 = lfacs[l], fac1 = 1 - x, fac2 = 1 + x, fac = fac1 / fac2;
      d_11[l] = fac1 * dP[l] / llp1 + P[l];
      d_m11[l] = fac2 * dP[l] / llp1 - P[l];
      sigmasq += (1 - d_11[l]) * Cphil3[l];
      Cg2 += d_m11[l] * Cphil3[l];
      d_22[l] = (((4 * x - 8) / fac2 + llp1) * P[l] + 4 * fac * (fac2 + (x - 2) / llp1) * dP[l]) / lfacs2[l];
      if (theta > theta_cut[l])
        d_2m2[l] = ((llp1 - (4 * x + 8) / fac1) * P[l] + 4 / fac * (-fac1 + (x + 2) / llp1) * dP[l]) / lfacs2[l];
      else
        d_2m2[l] = lfacs[l] * lfacs2[l] * std::pow(theta, 4) *
                   (1.0 / 384.0 - (3.0 * lfacs[l] - 8.0) / 23040.0 * theta * theta);
      d_20[l] = (2 * x * dP[l] - llp1 * P[l]) / lrootfacs[l];
    }
    double corr[4] = {0, 0, 0, 0};
    for (size_t j = 1; j <= lsj.size(); ++j) {
      int l = lsj[j - 1];
      double fac1 = 1 - x, fac2 = 1 + x, llp1 = lfacs[l];
      double rootllp1 = R(l) * R(l + 1), rootfac1 = R(l + 2) * R(l - 1), rootfac2 = R(l + 3) * R(l - 2), rootfac3;
      double dm11 = d_m11[l], d11 = d_11[l];
      double d2m2, d22, d20, d1m2, d12, d1m3, d2m3, d3m3, d13, d23, d33, d04, d2m4, d4m4;
      if (l < 2) {
        d2m2 = d22 = d20 = d1m2 = d12 = 0;
      } else {
        d2m2 = d_2m2[l];
        d22 = d_22[l];
        d20 = d_20[l];
        d1m2 = sinth / rootfac1 * (dP[l] - 2 / fac1 * dm11);
        d12 = sinth / rootfac1 * (dP[l] - 2 / fac2 * d11);
      }
      if (l < 3) {
        d1m3 = d2m3 = d3m3 = d13 = d23 = d33 = 0;
      } else {
        double sinfac = 4 / sinth;
        d1m3 = (-(x + 0.5) * d1m2 * sinfac - lfacs2[l] * dm11 / rootfac1) / rootfac2;
        d2m3 = (-fac2 * d2m2 * sinfac - rootfac1 * d1m2) / rootfac2;
        d3m3 = (-(x + 1.5) * d2m3 * sinfac - rootfac1 * d1m3) / rootfac2;
        d13 = ((x - 0.5) * d12 * sinfac - lfacs2[l] * d11 / rootfac1) / rootfac2;
        d23 = (-fac1 * d22 * sinfac + rootfac1 * d12) / rootfac2;
        d33 = (-(x - 1.5) * d23 * sinfac - rootfac1 * d13) / rootfac2;
      }
      (void)d33;
      if (l < 4) {
        d04 = d2m4 = d4m4 = 0;
        rootfac3 = 0;
      } else {
        rootfac3 = R(l - 3) * R(l + 4);
        d04 = ((-llp1 + (18 * x * x + 6) / (sinth * sinth)) * d20 - 6 * x * lfacs2[l] * dP[l] / lrootfacs[l]) /
              (rootfac2 * rootfac3);
        d2m4 = (-(6 * x + 4) * d2m3 / sinth - rootfac2 * d2m2) / rootfac3;
        d4m4 = (-7 / 5.0 * (llp1 - 6) * d2m2 + 12 / 5.0 * (-llp1 + (9 * x + 26) / fac1) * d3m3) / (llp1 - 12);
      }
      double X000 = std::exp(-llp1 * sigmasq / 4);
      double X022 = X000 * (1 + sigmasq);
      double X220 = lrootfacs[l] / 4 * X000;
      double X121 = -0.5 * rootfac1 * X000;
      double X132 = -0.5 * rootfac2 * X000;
      double X242 = 0.25 * rootfac2 * rootfac3 * X022;
      double dX000 = -llp1 / 4 * X000;
      double dX022 = (1 - llp1 / 4) * X022;
      double f1 = dX000 * dX000, f3 = X220 * X220, Cg2sq = Cg2 * Cg2;
      double fac = ((X000 * X000 - 1) + Cg2sq * f1) * P[l] + Cg2sq * f3 * d2m2 + 8 / llp1 * f1 * Cg2 * dm11;
      double sc = j > 14 ? (double)interp_fac : 1.0;
      corr[0] += sc * CTT[l] * fac;
      double f2 = (Cg2 * dX022) * (Cg2 * dX022) + (X022 * X022 - 1);
      fac = 2 * Cg2 * X121 * X132 * d13 + f2 * d22 + Cg2sq * X242 * X220 * d04;
      corr[1] += sc * CEE[l] * fac;
      fac = (f3 * P[l] + X242 * X242 * d4m4) * Cg2sq / 2 + Cg2 * (X121 * X121 * dm11 + X132 * X132 * d3m3) + f2 * d2m2;
      corr[2] += sc * CEE[l] * fac;
      fac = (X000 * X022 - 1) * d20 + 2 * dX000 * Cg2 * (X121 * d11 + X132 * d1m3) / rootllp1 +
            Cg2sq * (X220 / 2 * d2m4 * X242 + (f3 / 2 + dX022 * dX000) * d20);
      corr[3] += sc * CTE[l] * fac;
    }
    if (i > npoints - apodize_point_width) {
      double taper = (double)(npoints - i) / (double)apodize_point_width;
      taper = std::max(0.0, std::min(1.0, taper));
      taper = taper * taper * taper * (10.0 + taper * (-15.0 + 6.0 * taper));
      for (double& c : corr) c *= taper;
    }
    for (int l = lmin; l <= lmax_lensed; ++l) {
      double* o = &contrib[(size_t)l * 4];
      o[0] += corr[0] * P[l] * sinth;
      double T2 = corr[1] * d_22[l], T4 = corr[2] * d_2m2[l];
      o[1] += (T2 + T4) * halfsinth;
      o[2] += (T2 - T4) * halfsinth;
      o[3] += corr[3] * d_20[l] * sinth;
    }
  }
  for (int l = lmin; l <= lmax_lensed; ++l) {
    double fac = (double)l * (l + 1) / (2 * kPi) * dtheta * (2 * kPi);
    const double* c = &contrib[(size_t)l * 4];
    out[(size_t)l * 4 + 0] = c[0] * fac + cl[(size_t)l * 4 + 0];
    out[(size_t)l * 4 + 1] = c[1] * fac + cl[(size_t)l * 4 + 1];
    out[(size_t)l * 4 + 2] = c[2] * fac;
    out[(size_t)l * 4 + 3] = c[3] * fac + cl[(size_t)l * 4 + 2];
  }
  return 0;
}

}  // extern "C"
