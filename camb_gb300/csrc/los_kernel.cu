// Source k-spline, flat line-of-sight projection and C_l k-integral (FP64).
//
//   source_spline_kernel  InitSourceInterpolation (cmbmain.f90:1249-1265): natural
//                         cubic spline in k of every (tau, source) row of LinearSrc.
//   los_flat_kernel       SourceToTransfers -> InterpolateSources -> DoFlatIntegration
//                         (cmbmain.f90:543-562, 1351-1480, 1639-1862): one CTA per
//                         integration wavenumber q; the interpolated sources, the Bessel
//                         table index and weight of every time step are staged in
//                         shared memory once, then one warp per sampled l sums
//                         S(q,tau_n) j_l(q(tau0-tau_n)) dtau_n over its window.
//   los_flat_mixed_kernel the same projection with the Bessel table and sources in FP32
//                         and FP64 accumulation of FP32 chunk sums (mixed precision).
//   scal_cls_kernel       CalcScalCls (cmbmain.f90:3179-3343): one CTA per sampled l,
//                         block reduction over q of P(k) Delta_X Delta_Y dlnk.
#include <cuda_runtime.h>

#include "device_tables.cuh"

namespace cgdev {

__device__ __forceinline__ double ldgd(const double* p) { return __ldg(p); }

// 0-based index i with x[i] <= v < x[i+1], clamped to [0, n-2]
__device__ __forceinline__ int bsearch_lo(const double* __restrict__ x, int n, double v) {
  if (v <= x[0]) return 0;
  if (v >= x[n - 1]) return n - 2;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (v >= ldgd(x + mid)) lo = mid;
    else hi = mid;
  }
  return lo;
}

// TRanges%IndexOf on the time grid as used in DoFlatIntegration: 1-based index of
// the last point <= v (0 below the grid, ntau at or above its end).
__device__ __forceinline__ int time_index_of(const double* __restrict__ x, int n, double v) {
  if (v < x[0]) return 0;
  if (v >= x[n - 1]) return n;
  return bsearch_lo(x, n, v) + 1;
}

// spl: per-cosmology spline factors on the source k grid, laid out [5][nk]:
// inv_dx[i] = 1/(x[i+1]-x[i]), sig[i], pinv[i] = 1/(sig*fac[i-1]+2), fac[i] = (sig-1)*pinv,
// c6[i] = 6/(x[i+1]-x[i-1]).
__global__ void source_spline_kernel(const DevCosmo* __restrict__ cosmos, const double* const* __restrict__ spl_ptrs) {
  const DevCosmo& C = cosmos[blockIdx.y];
  int rows = C.ntau * C.nsrc;
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int n = C.nk;
  const double* spl = spl_ptrs[blockIdx.y];
  const double *inv_dx = spl, *sig = spl + n, *pinv = spl + 2 * n, *fac = spl + 3 * n, *c6 = spl + 4 * n;
  const double* y = C.linear_src + (size_t)r * n;
  double* d2 = C.dd_src + (size_t)r * n;
  // forward sweep: d2 temporarily holds u
  double u_prev = 0, sl_prev = (y[1] - y[0]) * ldgd(inv_dx);
  d2[0] = 0;
  for (int i = 1; i < n - 1; ++i) {
    double sl = (y[i + 1] - y[i]) * ldgd(inv_dx + i);
    double u = (ldgd(c6 + i) * (sl - sl_prev) - ldgd(sig + i) * u_prev) * ldgd(pinv + i);
    d2[i] = u;
    u_prev = u;
    sl_prev = sl;
  }
  d2[n - 1] = 0;
  double next = 0;
  for (int k = n - 2; k >= 1; --k) {
    double v = ldgd(fac + k) * next + d2[k];
    d2[k] = v;
    next = v;
  }
  d2[0] = 0;
}

constexpr int LOS_THREADS = 256;

// One CTA per integration wavenumber q.  F32 selects the mixed-precision projection:
// Bessel table (float4 Horner coefficients) and staged sources in FP32, products summed
// in FP32 over chunks of kChunk time steps per lane and the chunk sums accumulated in
// FP64.  Everything before the projection (source k-interpolation, Bessel interval
// search) and the Limber branch stay FP64.
constexpr int kChunk = 16;
constexpr int kLosMaxL = 512;  // sampled l per cosmology (the host rejects more)

template <bool F32>
__device__ __forceinline__ void los_flat_body(const DevCosmo& C, int q_ix, double* smem) {
  const int ntau = C.ntau, nsrc = C.nsrc, nk = C.nk;
  double* s_src = smem;                                      // [ntau][3] (FP64 variant)
  float* s_srcf = reinterpret_cast<float*>(smem);            // [ntau][3] (FP32 variant)
  double* s_w = s_src + (size_t)ntau * 3;                    // [ntau] Horner variable (left weight)
  float* s_wf = reinterpret_cast<float*>(s_w);               // [ntau] (FP32 variant)
  double* s_raw3 = s_w + ntau;                               // [ntau] lensing source without dtau (Limber)
  int* s_bix = (int*)(s_raw3 + ntau);                        // [ntau] 0-based Bessel interval
  const double q = C.q_int[q_ix];
  const double tau0 = C.tau0;
  const double max_etak = C.want_late_time ? 0.0 : C.max_etak_scalar;
  const bool ignore_etak = C.want_late_time != 0;
  // InterpolateSources: interval of q in the source k grid
  int klo;
  if (q <= C.q_evolve[0]) klo = 0;
  else if (q >= C.q_evolve[nk - 1]) klo = nk - 2;
  else klo = bsearch_lo(C.q_evolve, nk, q);
  const int khi = klo + 1;
  const double ho = C.q_evolve[khi] - C.q_evolve[klo];
  const double a0 = (C.q_evolve[khi] - q) / ho, b0 = (q - C.q_evolve[klo]) / ho;
  const double ho2o6 = ho * ho / 6.0, a03 = a0 * a0 * a0 - a0, b03 = b0 * b0 * b0 - b0;
  // SourceSteps: the time steps with q*tau < max_etak (unless late-time sources) and
  // q*(tau0-tau) > 1e-8 form a prefix starting at point 2
  __shared__ int s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  int cnt = 0;
  for (int i = 1 + threadIdx.x; i < ntau; i += blockDim.x) {
    double tau = C.tau_points[i];
    bool ok = (ignore_etak || q * tau < max_etak) && q * (tau0 - tau) > 1e-8;
    cnt += ok ? 1 : 0;
  }
  atomicAdd(&s_cnt, cnt);
  __syncthreads();
  const int source_steps = max(2, 1 + s_cnt);  // 1-based count of rows filled (row 1 is zero)
  const int nbx = C.num_xx;
  for (int i = threadIdx.x; i < source_steps; i += blockDim.x) {
    double tau = C.tau_points[i];
    double xx = fabs(q * (tau0 - tau));
    int bi = bsearch_lo(C.bess_x, nbx, xx);
    double x_hi = ldgd(C.bess_x + bi + 1), dx = x_hi - ldgd(C.bess_x + bi);
    s_bix[i] = bi;
    if (F32) s_wf[i] = (float)((x_hi - xx) / dx);
    else s_w[i] = (x_hi - xx) / dx;
    const double dt = C.tau_dpoints[i];
    for (int s = 0; s < 3; ++s) {
      double v = 0;
      if (s < nsrc && i >= 1 && i < 1 + s_cnt) {
        size_t b = ((size_t)i * nsrc + s) * nk;
        v = a0 * C.linear_src[b + klo] + b0 * C.linear_src[b + khi] +
            (a03 * C.dd_src[b + klo] + b03 * C.dd_src[b + khi]) * ho2o6;
      }
      // the time weight dtau_n is folded into the staged source
      if (F32) s_srcf[i * 3 + s] = (float)(v * dt);
      else s_src[i * 3 + s] = v * dt;
      if (s == 2) s_raw3[i] = v;
    }
  }
  __syncthreads();
  // DoSourceIntegration (flat): last l to integrate
  int llmax = (int)llrint(q * tau0);
  if (llmax < 15) llmax = 17;
  else llmax = (int)llrint(q * (tau0 + 6 * 3.14159265358979323846 / q));
  const double BessIntBoost = C.AccuracyBoost * C.BessIntBoost;
  const double limber_l = 400 * sqrt(C.AccuracyBoost * C.LimberBoost);
  const double* __restrict__ tp = C.tau_points;
  // Per sampled l: the integration window in time steps, whether to integrate, and the
  // Limber value of the lensing source -- computed by one thread per l (the scalar FP64
  // set-up would otherwise run once per warp on the FP64 pipe for each l).
  __shared__ int s_ns[kLosMaxL], s_ne[kLosMaxL], s_flag[kLosMaxL];
  __shared__ double s_limb[kLosMaxL];
  enum { F_SKIP = 1, F_INT = 2, F_LIMBER = 4 };
  for (int j = threadIdx.x; j < C.nl; j += blockDim.x) {
    const int l = C.ls[j];
    int flag = 0, ns = 0, ne = -1;
    double limb = 0;
    if (l > llmax) flag = F_SKIP;
    else {
      const double xlim = fmax(0.0, l - 4.2 * cbrt((double)l));
      const double xlmax1 = 80 * l * BessIntBoost;
      const double tmin = fmax(tp[1], tau0 - xlmax1 / q);
      const double tmax = tau0 - xlim / q;
      if (tmax < tp[1]) flag = F_SKIP;
      else {
        bool doint = true;
        if (nsrc > 2) doint = q < max(850, l) * 3 * BessIntBoost / tau0 * 1.2;
        if (doint) {
          flag |= F_INT;
          ns = time_index_of(tp, ntau, tmin);
          ne = min(source_steps, time_index_of(tp, ntau, tmax));
        }
        if (nsrc > 2 && (!doint || l > limber_l)) {
          // Limber approximation for the lensing potential (cmbmain.f90:1821-1832)
          flag |= F_LIMBER;
          double xf = tau0 - (l + 0.5) / q;
          if (xf < tp[ntau - 1] && xf > tp[0]) {
            int n = time_index_of(tp, ntau, xf);  // 1-based
            double f = (xf - tp[n - 1]) / (tp[n] - tp[n - 1]);
            double s_lo = (n - 1 < source_steps) ? s_raw3[n - 1] : 0.0;
            double s_hi = (n < source_steps) ? s_raw3[n] : 0.0;
            limb = (s_lo * (1 - f) + f * s_hi) * sqrt(3.14159265358979323846 / 2 / (l + 0.5)) / q;
          }
        }
      }
    }
    s_flag[j] = flag;
    s_ns[j] = ns;
    s_ne[j] = ne;
    s_limb[j] = limb;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int j = warp; j < C.nl; j += nwarps) {
    const int flag = s_flag[j];
    if (flag & F_SKIP) {  // nothing to integrate: the transfer function is zero
      if (lane == 0) {
        double* D = C.delta + ((size_t)q_ix * C.nl + j) * nsrc;
        for (int s = 0; s < nsrc; ++s) D[s] = 0;
      }
      continue;
    }
    double acc0 = 0, acc1 = 0, acc2 = 0;
    if (flag & F_INT) {
      const int nstart = s_ns[j], nend = s_ne[j];
      if (F32) {
        const float4* __restrict__ H = C.bessel_f32 + (size_t)j * (nbx - 1);
        float f0 = 0.f, f1 = 0.f, f2 = 0.f;
        int k = 0;
        int n = nstart + lane;
        // four independent table gathers in flight per lane
        for (; n + 96 <= nend; n += 128) {
          float J[4];
          int ii[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) ii[u] = n - 1 + 32 * u;
          float4 c[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) c[u] = __ldg(H + s_bix[ii[u]]);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float a2 = s_wf[ii[u]];
            J[u] = fmaf(a2, fmaf(a2, fmaf(a2, c[u].w, c[u].z), c[u].y), c[u].x);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            f0 = fmaf(s_srcf[ii[u] * 3 + 0], J[u], f0);
            f1 = fmaf(s_srcf[ii[u] * 3 + 1], J[u], f1);
            f2 = fmaf(s_srcf[ii[u] * 3 + 2], J[u], f2);
          }
          k += 4;
          if (k >= kChunk) {
            acc0 += f0;
            acc1 += f1;
            acc2 += f2;
            f0 = f1 = f2 = 0.f;
            k = 0;
          }
        }
        for (; n <= nend; n += 32) {
          const int i = n - 1;
          const float a2 = s_wf[i];
          const float4 c = __ldg(H + s_bix[i]);
          const float J = fmaf(a2, fmaf(a2, fmaf(a2, c.w, c.z), c.y), c.x);
          f0 = fmaf(s_srcf[i * 3 + 0], J, f0);
          f1 = fmaf(s_srcf[i * 3 + 1], J, f1);
          f2 = fmaf(s_srcf[i * 3 + 2], J, f2);
        }
        acc0 += f0;
        acc1 += f1;
        acc2 += f2;
      } else {
        const double* __restrict__ H = C.bessel_horner + (size_t)j * (nbx - 1) * 4;
        for (int n = nstart + lane; n <= nend; n += 32) {
          const int i = n - 1;  // 0-based row
          const double a2 = s_w[i];
          const double2* hp = reinterpret_cast<const double2*>(H + (size_t)s_bix[i] * 4);
          const double2 c01 = __ldg(hp), c23 = __ldg(hp + 1);
          const double J = c01.x + a2 * (c01.y + a2 * (c23.x + a2 * c23.y));
          acc0 += s_src[i * 3 + 0] * J;
          acc1 += s_src[i * 3 + 1] * J;
          acc2 += s_src[i * 3 + 2] * J;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
        acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
        acc2 += __shfl_xor_sync(0xffffffffu, acc2, o);
      }
    }
    if (flag & F_LIMBER) acc2 = s_limb[j];
    if (lane == 0) {
      double* D = C.delta + ((size_t)q_ix * C.nl + j) * nsrc;
      D[0] = acc0;
      D[1] = acc1;
      if (nsrc > 2) D[2] = acc2;
    }
  }
}

__global__ void __launch_bounds__(LOS_THREADS) los_flat_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  if ((int)blockIdx.x >= C.nq || C.nl > kLosMaxL) return;
  extern __shared__ double smem[];
  los_flat_body<false>(C, blockIdx.x, smem);
}

__global__ void __launch_bounds__(LOS_THREADS) los_flat_mixed_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  if ((int)blockIdx.x >= C.nq || C.nl > kLosMaxL) return;
  extern __shared__ double smem[];
  los_flat_body<true>(C, blockIdx.x, smem);
}

constexpr int CLS_THREADS = 256;

__global__ void __launch_bounds__(CLS_THREADS) scal_cls_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  const int j = blockIdx.x;
  if (j >= C.nl) return;
  const int nsrc = C.nsrc, nl = C.nl;
  double c[6] = {0, 0, 0, 0, 0, 0};
  for (int q_ix = threadIdx.x; q_ix < C.nq; q_ix += blockDim.x) {
    double k = C.q_int[q_ix];
    double dlnk = C.dq_int[q_ix] / k;
    double lnrat = log(k / C.pivot_scalar);
    double ap = C.As * exp(lnrat * (C.ns - 1 + lnrat * (C.nrun / 2)));
    const double* D = C.delta + ((size_t)q_ix * nl + j) * nsrc;
    double w = ap * dlnk;
    double d0 = D[0], d1 = D[1];
    c[0] += w * d0 * d0;
    c[1] += w * d1 * d1;
    c[2] += w * d0 * d1;
    if (nsrc > 2) {
      double d2 = D[2];
      c[3] += w * d2 * d2;
      c[4] += w * d2 * d0;
      c[5] += w * d2 * d1;
    }
  }
  __shared__ double red[CLS_THREADS / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    double v = c[m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][m] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[6] = {0, 0, 0, 0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      for (int m = 0; m < 6; ++m) t[m] += red[w][m];
    const double fourpi = 4 * 3.14159265358979323846, twopi = 2 * 3.14159265358979323846;
    double ell = C.ls[j];
    double ctnorm = (ell * ell - 1) * (ell + 2) * ell;
    double dbletmp = (ell * (ell + 1)) / twopi * fourpi;
    double* o = C.icl + (size_t)j * 6;
    o[0] = t[0] * dbletmp;
    o[1] = t[1] * dbletmp * ctnorm;
    o[2] = t[2] * dbletmp * sqrt(ctnorm);
    if (nsrc > 2) {
      o[3] = C.Alens * t[3] * fourpi * ell * ell * ell * ell;
      o[4] = sqrt(C.Alens) * t[4] * fourpi * ell * ell * ell;
      o[5] = sqrt(C.Alens) * t[5] * fourpi * ell * ell * ell * sqrt(ctnorm);
    } else {
      o[3] = o[4] = o[5] = 0;
    }
  }
}

}  // namespace cgdev
