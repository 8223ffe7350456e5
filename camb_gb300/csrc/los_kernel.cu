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
//   source_spline_f32_kernel  the same spline, leaving FP32 {source, d2} pairs.
//   los_flat_mixed_kernel the same projection with the staged sources, Bessel weights,
//                         table and products in FP32 and compensated FP32 sums
//                         (mixed precision).
//   pk_weight_kernel      the primordial-power weights A_s P(q) dq/q, once per (cosmology, q).
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
// c6[i] = 6/(x[i+1]-x[i-1]).  F32OUT (mixed precision): the row's slots of dd_src end up
// holding float2 {source, second derivative} per k instead of the FP64 derivative.
template <bool F32OUT>
__device__ __forceinline__ void source_spline_body(const DevCosmo* __restrict__ cosmos,
                                                   const double* const* __restrict__ spl_ptrs) {
  const DevCosmo& C = cosmos[blockIdx.y];
  int rows = C.ntau * C.nsrc;
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int n = C.nk;
  const double* spl = spl_ptrs[blockIdx.y];
  const double *inv_dx = spl, *sig = spl + n, *pinv = spl + 2 * n, *fac = spl + 3 * n, *c6 = spl + 4 * n;
  const double* y = C.linear_src + (size_t)r * n;
  double* d2 = C.dd_src + (size_t)r * n;
  float2* out = reinterpret_cast<float2*>(d2);
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
  if (F32OUT) out[n - 1] = make_float2((float)y[n - 1], 0.f);
  else d2[n - 1] = 0;
  double next = 0;
  for (int k = n - 2; k >= 1; --k) {
    double v = ldgd(fac + k) * next + d2[k];
    if (F32OUT) out[k] = make_float2((float)y[k], (float)v);  // slot k is read before it is overwritten
    else d2[k] = v;
    next = v;
  }
  if (F32OUT) out[0] = make_float2((float)y[0], 0.f);
  else d2[0] = 0;
}

__global__ void source_spline_kernel(const DevCosmo* __restrict__ cosmos, const double* const* __restrict__ spl_ptrs) {
  source_spline_body<false>(cosmos, spl_ptrs);
}

__global__ void source_spline_f32_kernel(const DevCosmo* __restrict__ cosmos,
                                         const double* const* __restrict__ spl_ptrs) {
  source_spline_body<true>(cosmos, spl_ptrs);
}

constexpr int LOS_THREADS = 256;
constexpr int kChunk = 16;
constexpr int kLosMaxL = 512;  // sampled l per cosmology (the host rejects more)

// SourceSteps: the number of time steps i in [1, ntau) with q*tau_i < max_etak (unless
// late-time sources) and q*(tau0-tau_i) > 1e-8.  Both hold on a prefix of the increasing
// time grid (the rounded products are monotone in tau), so warp 0 locates the first
// failing step by a 32-way search rather than testing every step.
__device__ int source_row_count(const DevCosmo& C, double q, int* s_cnt) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const double tau0 = C.tau0;
    const double max_etak = C.want_late_time ? 0.0 : C.max_etak_scalar;
    const bool ignore_etak = C.want_late_time != 0;
    int lo = 1, hi = C.ntau;  // steps below lo pass; the first failing step is in [lo, hi]
    while (lo < hi) {
      const int step = (hi - lo + 31) >> 5;
      const int p = lo + lane * step;
      bool fail = false;
      if (p < hi) {
        const double tau = C.tau_points[p];
        fail = !((ignore_etak || q * tau < max_etak) && q * (tau0 - tau) > 1e-8);
      }
      const unsigned fm = __ballot_sync(0xffffffffu, fail);
      const unsigned pm = __ballot_sync(0xffffffffu, p < hi);
      const int base = lo;
      if (fm) {
        const int f = __ffs(fm) - 1;
        hi = base + f * step;
        if (f > 0) lo = base + (f - 1) * step + 1;
      } else {
        lo = base + (31 - __clz(pm)) * step + 1;
      }
    }
    if (lane == 0) *s_cnt = lo - 1;
  }
  __syncthreads();
  return *s_cnt;
}

// time_index_of from the time grid's runs of uniform spacing: an FP32 estimate of the
// interval, then FP64 comparisons against the grid points settle the exact answer (the
// largest i with tau_i <= v, as the bisection finds it), falling back to the bisection if
// the estimate is more than four intervals off
__device__ __forceinline__ int time_index_runs(const DevCosmo& C, const double* __restrict__ tp, double v) {
  const int n = C.ntau;
  if (C.ntseg == 0) return time_index_of(tp, n, v);
  if (v < tp[0]) return 0;
  if (v >= tp[n - 1]) return n;
  const float vf = (float)v;
  int r = 0;
  for (int t = 1; t < C.ntseg; ++t) r = vf >= (float)C.tseg_x0[t] ? t : r;
  int i = (int)((vf - (float)C.tseg_x0[r]) * (float)C.tseg_inv_h[r]);
  i = C.tseg_i0[r] + min(max(i, 0), C.tseg_n[r] - 1);
  i = min(max(i, 0), n - 2);
  for (int g = 0; g < 4 && tp[i] > v; ++g) --i;       // tp[0] <= v: stops at 0 at the latest
  for (int g = 0; g < 4 && tp[i + 1] <= v; ++g) ++i;  // tp[n-1] > v: stops at n-2 at the latest
  if (tp[i] > v || tp[i + 1] <= v) return time_index_of(tp, n, v);
  return i + 1;
}

// Interval of x in the Bessel x grid from its runs of uniform spacing, in FP32: the exact
// interval or a neighbour of it.
__device__ __forceinline__ int bess_interval_estimate(const float* s_x0, const float* s_ih, const int* s_i0,
                                                      const int* s_n, int nseg, int nbx, float xf) {
  int r = 0;
  for (int t = 1; t < nseg; ++t) r = xf >= s_x0[t] ? t : r;
  int i = (int)((xf - s_x0[r]) * s_ih[r]);
  i = s_i0[r] + min(max(i, 0), s_n[r] - 1);
  return min(max(i, 0), nbx - 2);
}

struct SegShared {
  float x0[kBessSegMax], ih[kBessSegMax];
  int i0[kBessSegMax], n[kBessSegMax];
};

__device__ __forceinline__ void load_segments(const DevCosmo& C, SegShared& S) {
  if (threadIdx.x < C.nseg) {
    S.x0[threadIdx.x] = (float)C.seg_x0[threadIdx.x];
    S.ih[threadIdx.x] = (float)C.seg_inv_h[threadIdx.x];
    S.i0[threadIdx.x] = C.seg_i0[threadIdx.x];
    S.n[threadIdx.x] = C.seg_n[threadIdx.x];
  }
}

enum { F_SKIP = 1, F_INT = 2, F_LIMBER = 4 };

// Per sampled l (DoSourceIntegration, flat): the integration window in time steps,
// whether to integrate, and the Limber value of the lensing source -- one thread per l
// (the scalar FP64 set-up would otherwise run once per warp on the FP64 pipe for each l).
// FAST (mixed precision): the l-only factors come from the per-cosmology tables and 1/q is
// formed once, instead of a cube root, two divisions and a square root per (q, l).
template <bool FAST, typename RawT>
__device__ __forceinline__ void window_setup(const DevCosmo& C, double q, int source_steps, const RawT* s_raw3,
                                             int* s_ns, int* s_ne, int* s_flag, double* s_limb) {
  const int ntau = C.ntau, nsrc = C.nsrc;
  const double tau0 = C.tau0;
  int llmax = (int)llrint(q * tau0);
  if (llmax < 15) llmax = 17;
  else llmax = (int)llrint(q * (tau0 + 6 * 3.14159265358979323846 / q));
  const double BessIntBoost = C.AccuracyBoost * C.BessIntBoost;
  const double limber_l = 400 * sqrt(C.AccuracyBoost * C.LimberBoost);
  const double* __restrict__ tp = C.tau_points;
  const double inv_q = FAST ? 1.0 / q : 0.0;
  for (int j = threadIdx.x; j < C.nl; j += blockDim.x) {
    const int l = C.ls[j];
    int flag = 0, ns = 0, ne = -1;
    double limb = 0;
    if (l > llmax) flag = F_SKIP;
    else {
      const double xlim = FAST ? C.l_xlim[j] : fmax(0.0, l - 4.2 * cbrt((double)l));
      const double xlmax1 = 80 * l * BessIntBoost;
      const double tmin = fmax(tp[1], FAST ? tau0 - xlmax1 * inv_q : tau0 - xlmax1 / q);
      const double tmax = FAST ? tau0 - xlim * inv_q : tau0 - xlim / q;
      if (tmax < tp[1]) flag = F_SKIP;
      else {
        bool doint = true;
        if (nsrc > 2) doint = q < (FAST ? C.l_doint[j] : max(850, l) * 3 * BessIntBoost / tau0 * 1.2);
        if (doint) {
          flag |= F_INT;
          ns = FAST ? time_index_runs(C, tp, tmin) : time_index_of(tp, ntau, tmin);
          ne = min(source_steps, FAST ? time_index_runs(C, tp, tmax) : time_index_of(tp, ntau, tmax));
        }
        if (nsrc > 2 && (!doint || l > limber_l)) {
          // Limber approximation for the lensing potential (cmbmain.f90:1821-1832)
          flag |= F_LIMBER;
          double xf = FAST ? tau0 - (l + 0.5) * inv_q : tau0 - (l + 0.5) / q;
          if (xf < tp[ntau - 1] && xf > tp[0]) {
            int n = FAST ? time_index_runs(C, tp, xf) : time_index_of(tp, ntau, xf);  // 1-based
            double f = (xf - tp[n - 1]) / (tp[n] - tp[n - 1]);
            double s_lo = (n - 1 < source_steps) ? (double)s_raw3[n - 1] : 0.0;
            double s_hi = (n < source_steps) ? (double)s_raw3[n] : 0.0;
            limb = FAST ? (s_lo * (1 - f) + f * s_hi) * C.l_limb[j] * inv_q
                        : (s_lo * (1 - f) + f * s_hi) * sqrt(3.14159265358979323846 / 2 / (l + 0.5)) / q;
          }
        }
      }
    }
    s_flag[j] = flag;
    s_ns[j] = ns;
    s_ne[j] = ne;
    s_limb[j] = limb;
  }
}

// InterpolateSources: interval and cubic-spline weights of q on the source k grid
struct KInterp {
  int klo, khi;
  double a0, b0, a03, b03, ho2o6;
};

// the same for every thread of a CTA (one q): thread 0 computes it, the others read it
// from shared memory (saves the bisection and divisions on the FP64 pipe of every warp)
__device__ __forceinline__ KInterp k_interp_shared(const DevCosmo& C, double q, KInterp* s_K);

__device__ __forceinline__ KInterp k_interp(const DevCosmo& C, double q) {
  const int nk = C.nk;
  KInterp K;
  if (q <= C.q_evolve[0]) K.klo = 0;
  else if (q >= C.q_evolve[nk - 1]) K.klo = nk - 2;
  else K.klo = bsearch_lo(C.q_evolve, nk, q);
  K.khi = K.klo + 1;
  const double ho = C.q_evolve[K.khi] - C.q_evolve[K.klo];
  K.a0 = (C.q_evolve[K.khi] - q) / ho;
  K.b0 = (q - C.q_evolve[K.klo]) / ho;
  K.ho2o6 = ho * ho / 6.0;
  K.a03 = K.a0 * K.a0 * K.a0 - K.a0;
  K.b03 = K.b0 * K.b0 * K.b0 - K.b0;
  return K;
}

__device__ __forceinline__ KInterp k_interp_shared(const DevCosmo& C, double q, KInterp* s_K) {
  if (threadIdx.x == 0) *s_K = k_interp(C, q);
  __syncthreads();
  return *s_K;
}

// One CTA per integration wavenumber q, FP64 throughout (the plain form): the interpolated
// sources, the Bessel table interval and weight of every time step are staged in shared
// memory once, then one warp per sampled l sums S(q,tau_n) j_l(q(tau0-tau_n)) dtau_n over
// its window.
__device__ __forceinline__ void los_flat_body(const DevCosmo& C, int q_ix, double* smem) {
  const int ntau = C.ntau, nsrc = C.nsrc, nk = C.nk;
  double* s_src = smem;                // [ntau][3]
  double* s_w = s_src + (size_t)ntau * 3;   // [ntau] Horner variable (left weight)
  double* s_raw3 = s_w + ntau;         // [ntau] lensing source without dtau (Limber)
  int* s_bix = (int*)(s_raw3 + ntau);  // [ntau] 0-based Bessel interval
  __shared__ int s_cnt;
  __shared__ SegShared S;
  const double q = C.q_int[q_ix];
  const double tau0 = C.tau0;
  load_segments(C, S);
  __shared__ KInterp s_K;
  const KInterp K = k_interp_shared(C, q, &s_K);
  const int cnt = source_row_count(C, q, &s_cnt);  // synchronises (segments visible after)
  const int source_steps = max(2, 1 + cnt);        // 1-based count of rows filled (row 1 is zero)
  const int nbx = C.num_xx;
  for (int i = threadIdx.x; i < source_steps; i += blockDim.x) {
    double tau = C.tau_points[i];
    double xx = fabs(q * (tau0 - tau));
    int bi;
    if (C.nseg > 0) {
      // arithmetic estimate, then the exact interval by FP64 comparison (as bisection gives)
      bi = bess_interval_estimate(S.x0, S.ih, S.i0, S.n, C.nseg, nbx, (float)xx);
      while (bi > 0 && xx < ldgd(C.bess_x + bi)) --bi;
      while (bi < nbx - 2 && xx >= ldgd(C.bess_x + bi + 1)) ++bi;
    } else {
      bi = bsearch_lo(C.bess_x, nbx, xx);
    }
    double x_hi = ldgd(C.bess_x + bi + 1), dx = x_hi - ldgd(C.bess_x + bi);
    s_bix[i] = bi;
    s_w[i] = (x_hi - xx) / dx;
    const double dt = C.tau_dpoints[i];
    for (int s = 0; s < 3; ++s) {
      double v = 0;
      if (s < nsrc && i >= 1 && i < 1 + cnt) {
        size_t b = ((size_t)i * nsrc + s) * nk;
        v = K.a0 * C.linear_src[b + K.klo] + K.b0 * C.linear_src[b + K.khi] +
            (K.a03 * C.dd_src[b + K.klo] + K.b03 * C.dd_src[b + K.khi]) * K.ho2o6;
      }
      // the time weight dtau_n is folded into the staged source
      s_src[i * 3 + s] = v * dt;
      if (s == 2) s_raw3[i] = v;
    }
  }
  __syncthreads();
  __shared__ int s_ns[kLosMaxL], s_ne[kLosMaxL], s_flag[kLosMaxL];
  __shared__ double s_limb[kLosMaxL];
  window_setup<false>(C, q, source_steps, s_raw3, s_ns, s_ne, s_flag, s_limb);
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

// s + e = a + b exactly (Knuth's branch-free two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// hi + lo += f, compensated
__device__ __forceinline__ void comp_add(float& hi, float& lo, float f) {
  float s, e;
  two_sum(hi, f, s, e);
  hi = s;
  lo += e;
}

// Mixed precision: the same projection with everything on the FP32 pipe except the
// per-q and per-l set-up.  Sources come from the FP32 {source, d2} pairs written by
// source_spline_f32_kernel and are interpolated in FP32; the Bessel interval comes from
// the grid's uniform runs and its weight from an FP64 offset rounded to FP32; the table
// (float4 Horner coefficients) and the products are FP32, summed over chunks of kChunk
// time steps per lane and accumulated (across chunks and across the warp) as compensated
// FP32 pairs, which are converted to FP64 once per (q, l).
__device__ __forceinline__ void los_mixed_body(const DevCosmo& C, int q_ix, float* smem) {
  const int ntau = C.ntau, nsrc = C.nsrc, nk = C.nk;
  float* s_srcf = smem;                  // [ntau][3] source * dtau
  float* s_wf = s_srcf + (size_t)ntau * 3;  // [ntau] Horner variable (left weight)
  float* s_raw3 = s_wf + ntau;           // [ntau] lensing source without dtau (Limber)
  int* s_bix = (int*)(s_raw3 + ntau);    // [ntau] 0-based Bessel interval
  __shared__ int s_cnt;
  __shared__ SegShared S;
  const double q = C.q_int[q_ix];
  load_segments(C, S);
  __shared__ KInterp s_K;
  const KInterp K = k_interp_shared(C, q, &s_K);
  const float a0 = (float)K.a0, b0 = (float)K.b0, a3 = (float)(K.a03 * K.ho2o6), b3 = (float)(K.b03 * K.ho2o6);
  const int cnt = source_row_count(C, q, &s_cnt);
  const int source_steps = max(2, 1 + cnt);
  const int nbx = C.num_xx;
  const float2* __restrict__ LD = reinterpret_cast<const float2*>(C.dd_src);
  for (int i = threadIdx.x; i < source_steps; i += blockDim.x) {
    const double xx = fabs(q * C.tau_dist[i]);
    int bi;
    if (C.nseg > 0) bi = bess_interval_estimate(S.x0, S.ih, S.i0, S.n, C.nseg, nbx, (float)xx);
    else bi = bsearch_lo(C.bess_x, nbx, xx);
    s_bix[i] = bi;
    s_wf[i] = (float)(ldgd(C.bess_x + bi + 1) - xx) * __ldg(C.bess_inv_dxf + bi);
    const float dt = __ldg(C.tau_dpf + i);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      float v = 0.f;
      if (s < nsrc && i >= 1 && i < 1 + cnt) {
        const size_t b = ((size_t)i * nsrc + s) * nk;
        const float2 lo = LD[b + K.klo], hi = LD[b + K.khi];
        v = fmaf(a0, lo.x, fmaf(b0, hi.x, fmaf(a3, lo.y, b3 * hi.y)));
      }
      s_srcf[i * 3 + s] = v * dt;
      if (s == 2) s_raw3[i] = v;
    }
  }
  __syncthreads();
  __shared__ int s_ns[kLosMaxL], s_ne[kLosMaxL], s_flag[kLosMaxL];
  __shared__ double s_limb[kLosMaxL];
  __shared__ float2 s_res[kLosMaxL * 3];
  window_setup<true>(C, q, source_steps, s_raw3, s_ns, s_ne, s_flag, s_limb);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int j = warp; j < C.nl; j += nwarps) {
    const int flag = s_flag[j];
    if (!(flag & F_INT)) continue;
    const int nstart = s_ns[j], nend = s_ne[j];
    const float4* __restrict__ H = C.bessel_f32 + (size_t)j * (nbx - 1);
    float h0 = 0.f, h1 = 0.f, h2 = 0.f, e0 = 0.f, e1 = 0.f, e2 = 0.f;
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
        comp_add(h0, e0, f0);
        comp_add(h1, e1, f1);
        comp_add(h2, e2, f2);
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
    comp_add(h0, e0, f0);
    comp_add(h1, e1, f1);
    comp_add(h2, e2, f2);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float s, e;
      two_sum(h0, __shfl_xor_sync(0xffffffffu, h0, o), s, e);
      e0 += __shfl_xor_sync(0xffffffffu, e0, o) + e;
      h0 = s;
      two_sum(h1, __shfl_xor_sync(0xffffffffu, h1, o), s, e);
      e1 += __shfl_xor_sync(0xffffffffu, e1, o) + e;
      h1 = s;
      two_sum(h2, __shfl_xor_sync(0xffffffffu, h2, o), s, e);
      e2 += __shfl_xor_sync(0xffffffffu, e2, o) + e;
      h2 = s;
    }
    if (lane == 0) {
      s_res[j * 3 + 0] = make_float2(h0, e0);
      s_res[j * 3 + 1] = make_float2(h1, e1);
      s_res[j * 3 + 2] = make_float2(h2, e2);
    }
  }
  __syncthreads();
  // Delta_l(q) in FP64, one (l, source) per thread: zero where nothing is integrated, the
  // Limber value where it replaces the lensing integral
  const int nout = C.nl * nsrc;
  double* D = C.delta + (size_t)q_ix * nout;
  for (int t = threadIdx.x; t < nout; t += blockDim.x) {
    const int j = t / nsrc, s = t - j * nsrc;
    const int flag = s_flag[j];
    double v = 0;
    if (s == 2 && (flag & F_LIMBER)) v = s_limb[j];
    else if (flag & F_INT) {
      const float2 r = s_res[j * 3 + s];
      v = (double)r.x + (double)r.y;
    }
    D[t] = v;
  }
}

__global__ void __launch_bounds__(LOS_THREADS) los_flat_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  if ((int)blockIdx.x >= C.nq || C.nl > kLosMaxL) return;
  extern __shared__ double smem[];
  los_flat_body(C, blockIdx.x, smem);
}

__global__ void __launch_bounds__(LOS_THREADS) los_flat_mixed_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  if ((int)blockIdx.x >= C.nq || C.nl > kLosMaxL) return;
  extern __shared__ double smem[];
  los_mixed_body(C, blockIdx.x, reinterpret_cast<float*>(smem));
}

constexpr int CLS_THREADS = 256;

// CalcScalCls' weight of integration wavenumber q: A_s P(q) dlnq (the primordial power of
// InitialPower.f90:121-144 times dq/q), the same for every sampled l, so formed once per
// (cosmology, q) instead of once per (l, q)
__global__ void pk_weight_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  for (int q_ix = blockIdx.x * blockDim.x + threadIdx.x; q_ix < C.nq; q_ix += gridDim.x * blockDim.x) {
    const double k = C.q_int[q_ix];
    const double dlnk = C.dq_int[q_ix] / k;
    const double lnrat = log(k / C.pivot_scalar);
    const double ap = C.As * exp(lnrat * (C.ns - 1 + lnrat * (C.nrun / 2)));
    C.pk_w[q_ix] = ap * dlnk;
  }
}

__global__ void __launch_bounds__(CLS_THREADS) scal_cls_kernel(const DevCosmo* __restrict__ cosmos) {
  const DevCosmo& C = cosmos[blockIdx.y];
  const int j = blockIdx.x;
  if (j >= C.nl) return;
  const int nsrc = C.nsrc, nl = C.nl;
  double c[6] = {0, 0, 0, 0, 0, 0};
  for (int q_ix = threadIdx.x; q_ix < C.nq; q_ix += blockDim.x) {
    const double* D = C.delta + ((size_t)q_ix * nl + j) * nsrc;
    const double w = C.pk_w[q_ix];
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
