// C ABI of libcambgpu: host tables, device residency, kernel orchestration.
// Declarations and the reference interfaces they replace: include/cambgpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cambgpu.h"
#include "device_tables.cuh"
#include "host/cosmo_host.hpp"

namespace cgdev {
int ode_blocks_per_sm(int team, int threads, int warp_stride);
cudaError_t launch_ode_kernel(int team, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                              const WorkItem* items, int nitems, int* counter, bool transfer, int warp_stride);
cudaError_t launch_sigma8(const DevCosmo* cosmos, int n, cudaStream_t s);
cudaError_t launch_fp64_probe(int blocks, int threads, int iters, double* out, cudaStream_t s);
cudaError_t launch_proj_tc(const DevCosmo* cosmos, int ncosmo, int nq, int nsrc, int nk, int nl, const double* chi,
                           const float* dchi_f, int nchi, float2* tsrc, int* err, cudaStream_t s);
cudaError_t launch_fp64_pipe_probe(int nsm, int warps, int lanes, int chains, int iters, long long* cyc, double* out,
                                   cudaStream_t s);
__global__ void source_spline_kernel(const DevCosmo*, const double* const*);
__global__ void source_spline_f32_kernel(const DevCosmo*, const double* const*);
__global__ void los_flat_kernel(const DevCosmo*);
__global__ void los_flat_mixed_kernel(const DevCosmo*);
__global__ void scal_cls_kernel(const DevCosmo*);
__global__ void pk_weight_kernel(const DevCosmo*);
}  // namespace cgdev

using namespace cgdev;

namespace {

thread_local std::string g_err;  // per calling thread, as errno
std::atomic<long long> g_launches{0};
double g_timings[6] = {0, 0, 0, 0, 0, 0};
double g_host_ms[4] = {0, 0, 0, 0};  // host tables, staging, device pipeline, fetch (wall ms)
double wall_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
int g_team = 0;
int g_precision = 0;  // 0: FP64 throughout; 1: mixed-precision line-of-sight projection
// autotuned ODE configuration per batch-size class: [0] small (< 24 modes/SM), [1] large
// (schedule 0: a static first item per thread, later ones from the atomic queue counter;
// 1: static stride, thread t takes items t, t + T, t + 2T, ... of the queue order)
struct OdeCfg { int team; int order; int cap; int sched; };
// untuned defaults: warp per mode (shared-memory rows) for few modes, where latency
// decides; thread per mode for large batches, where FP64 throughput does
OdeCfg g_tuned[2] = {{6, 0, 0, 0}, {7, 4, 0, 1}};
constexpr int kWarpStrideMax = 448;  // the shared-memory warp kernel's largest state row
int g_order = -1;  // forced queue order (-1: use the tuned one)
int g_blocks_cap = 0;  // resident ODE blocks per SM (0: as many as fit)
int g_sched = -1;      // forced ODE schedule (-1: use the tuned one)
long long g_last_evals = 0;
long long g_h2d = 0, g_d2h = 0;

int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(x)                                                                       \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) return set_err(CAMBGPU_ERROR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// grow-only device arena, reset per call
struct Arena {
  char* base = nullptr;
  size_t cap = 0, used = 0;
  bool overflow = false;  // a take() past cap: the caller fails before any device use
  int reserve(size_t bytes) {
    used = 0;
    overflow = false;
    if (bytes <= cap) return 0;
    if (base) cudaFree(base);
    base = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + (1 << 20);
    if (cudaMalloc(&base, want) != cudaSuccess) return CAMBGPU_ERROR_ALLOCATION;
    cap = want;
    return 0;
  }
  template <class T>
  T* take(size_t n) {
    size_t bytes = (n * sizeof(T) + 255) & ~size_t(255);
    if (used + bytes > cap) {
      overflow = true;
      return reinterpret_cast<T*>(base);
    }
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

struct Runtime {
  bool init = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8];
  int nsm = 0;
  Arena arena;
  // Bessel tables resident on the device, keyed by host table address and shape
  // tables stay while a staged batch may use them: only tables last used by an earlier
  // staging (an older epoch) are evicted
  struct DevBessel {
    const double* host;
    size_t n;
    double* dev;
    double* devx;
    int num_xx;
    float4* devf;
    unsigned long epoch;
    unsigned long long print;  // content fingerprint: host tables are freed and their addresses reused
    float* inv_dxf;            // 1/(x_{i+1}-x_i) in FP32
    int nseg;                  // runs of uniform spacing in x (0: more than kBessSegMax)
    double seg_x0[cgdev::kBessSegMax], seg_inv_h[cgdev::kBessSegMax];
    int seg_i0[cgdev::kBessSegMax], seg_n[cgdev::kBessSegMax];
  };
  unsigned long epoch = 0;
  std::vector<DevBessel> bessel;
  // pinned staging for uploads
  char* pinned = nullptr;
  size_t pinned_cap = 0;
  // high-L template on the device (uploaded once)
  double* d_tmpl = nullptr;
  // lensing theta-grid tables, keyed by their geometry
  struct DevLensGeom {
    int lmin, lmax, npoints, apw, interp_fac;
    double dtheta;
    double* tab;
    double* roots;
    double* sinth;
    int* lsj;
    int nj;
  };
  std::vector<DevLensGeom> lens;
};
Runtime g_rt;
std::mutex g_mu;

int rt_init() {
  if (g_rt.init) return 0;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&g_rt.nsm, cudaDevAttrMultiProcessorCount, dev));
  CUDA_TRY(cudaStreamCreateWithFlags(&g_rt.stream, cudaStreamNonBlocking));
  for (auto& e : g_rt.ev) CUDA_TRY(cudaEventCreate(&e));
  CUDA_TRY(cudaFuncSetAttribute(los_flat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  CUDA_TRY(cudaFuncSetAttribute(los_flat_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  g_rt.init = true;
  return 0;
}

// FNV-1a over the shape and 64 sampled words of the table and its x grid
unsigned long long bessel_print(const CambGpuTables& t, size_t n) {
  unsigned long long h = 1469598103934665603ULL;
  auto mix = [&](unsigned long long v) {
    for (int b = 0; b < 8; ++b) {
      h ^= (v >> (8 * b)) & 0xff;
      h *= 1099511628211ULL;
    }
  };
  mix(n);
  mix((unsigned long long)t.num_xx);
  for (int k = 0; k < 32; ++k) {
    double a = t.bessel_horner[(n - 1) * k / 31], x = t.bess_x[(size_t)(t.num_xx - 1) * k / 31];
    unsigned long long ua, ux;
    std::memcpy(&ua, &a, 8);
    std::memcpy(&ux, &x, 8);
    mix(ua);
    mix(ux);
  }
  return h;
}

int device_bessel(const CambGpuTables& t, double** dev_h, double** dev_x, float4** dev_f,
                  const Runtime::DevBessel** entry) {
  size_t n = (size_t)t.nl * (t.num_xx - 1) * 4;
  const unsigned long long print = bessel_print(t, n);
  for (auto& b : g_rt.bessel)
    if (b.host == t.bessel_horner && b.n == n && b.num_xx == t.num_xx && b.print == print) {
      b.epoch = g_rt.epoch;
      *dev_h = b.dev;
      *dev_x = b.devx;
      *dev_f = b.devf;
      *entry = &b;
      return 0;
    }
  Runtime::DevBessel b{t.bessel_horner, n, nullptr, nullptr, t.num_xx, nullptr, g_rt.epoch, print, nullptr, 0,
                       {}, {}, {}, {}};
  {
    // The x grid is a few runs of uniform spacing (bessels.f90:170-178): record them so
    // that the projection kernels find a point's interval arithmetically, not by bisection
    const int nx = t.num_xx;
    const double* x = t.bess_x;
    int k = 0;
    b.nseg = 0;
    while (k < nx - 1) {
      const double h = x[k + 1] - x[k];
      int e = k + 1;  // the run covers intervals [k, e)
      while (e < nx - 1 && std::fabs((x[e + 1] - x[e]) - h) <= 1e-6 * h) ++e;
      if (b.nseg == cgdev::kBessSegMax) {
        b.nseg = 0;
        break;
      }
      b.seg_x0[b.nseg] = x[k];
      b.seg_inv_h[b.nseg] = (e - k) / (x[e] - x[k]);
      b.seg_i0[b.nseg] = k;
      b.seg_n[b.nseg] = e - k;
      ++b.nseg;
      k = e;
    }
    std::vector<float> inv_dx(nx - 1);
    for (int i = 0; i < nx - 1; ++i) inv_dx[i] = (float)(1.0 / (x[i + 1] - x[i]));
    CUDA_TRY(cudaMalloc(&b.inv_dxf, (size_t)(nx - 1) * sizeof(float)));
    CUDA_TRY(cudaMemcpy(b.inv_dxf, inv_dx.data(), (size_t)(nx - 1) * sizeof(float), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(cudaMalloc(&b.dev, n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&b.devx, (size_t)t.num_xx * sizeof(double)));
  CUDA_TRY(cudaMalloc(&b.devf, n * sizeof(float)));
  CUDA_TRY(cudaMemcpy(b.dev, t.bessel_horner, n * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(b.devx, t.bess_x, (size_t)t.num_xx * sizeof(double), cudaMemcpyHostToDevice));
  {
    // the FP32 copy of the Horner coefficients for the mixed-precision projection
    std::vector<float> f(n);
    for (size_t i = 0; i < n; ++i) f[i] = (float)t.bessel_horner[i];
    CUDA_TRY(cudaMemcpy(b.devf, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (g_rt.bessel.size() >= 4) {
    for (size_t i = 0; i < g_rt.bessel.size(); ++i) {
      auto& o = g_rt.bessel[i];
      if (o.epoch == g_rt.epoch) continue;  // used by the batch being staged
      cudaFree(o.dev);
      cudaFree(o.devx);
      cudaFree(o.devf);
      cudaFree(o.inv_dxf);
      g_rt.bessel.erase(g_rt.bessel.begin() + i);
      break;
    }
  }
  g_rt.bessel.push_back(b);
  *dev_h = b.dev;
  *dev_x = b.devx;
  *dev_f = b.devf;
  *entry = &g_rt.bessel.back();
  return 0;
}

int device_template(double** out) {
  if (!g_rt.d_tmpl) {
    CUDA_TRY(cudaMalloc(&g_rt.d_tmpl, sizeof(double) * 8001 * 4));
    CUDA_TRY(cudaMemcpy(g_rt.d_tmpl, kHighLTemplate, sizeof(double) * 8001 * 4, cudaMemcpyHostToDevice));
  }
  *out = g_rt.d_tmpl;
  return 0;
}

// Lensing l range and theta grid of one cosmology: LensingExtrapLmax (lensing.f90:161-177),
// InitLensedClArrays (:230-247) and the sampling set-up of CorrFuncFullSkyApodized
// (:378-429) with AccurateBB off and the targeted-accuracy theta boost on.
struct HostLensGeom {
  int lmin = 2, lmax = 0, lmax_lensed = 0, npoints = 0, apw = 0, interp_fac = 1;
  double dtheta = 0;
  std::vector<int> lsj;
  bool same(const Runtime::DevLensGeom& g) const {
    return g.lmin == lmin && g.lmax == lmax && g.npoints == npoints && g.apw == apw && g.interp_fac == interp_fac &&
           g.dtheta == dtheta;
  }
};

int lens_geometry(const CambGpuTables& t, HostLensGeom& g) {
  const int margin = 200, gap = 50;  // lens_output_margin, lens_convolution_gap
  const double pi = 3.1415926535897932384626433832795;
  const int max_l = t.max_l;
  const double boost = t.lens_accuracy_boost;
  const int output_lmax = max_l - margin;
  const int extrap = std::max(750, (int)std::ceil((0.45 * output_lmax + 400.0) * boost));
  g.lmax = std::max(std::min(8000, output_lmax + gap + extrap), max_l);
  int ix = t.nl - 2;
  while (ix > 0 && t.ls[ix] > max_l - (margin - gap)) --ix;
  g.lmax_lensed = std::max(t.ls[ix], max_l - margin);
  double ramp = std::min(1.0, std::max(0.0, ((double)output_lmax - 2500.0) / 1000.0));
  ramp = ramp * ramp * (3.0 - 2.0 * ramp);
  const double theta_boost = boost * (1.6 + 0.6 * ramp);
  int npoints = (int)(max_l * 2 * theta_boost);
  if (npoints < 2) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lensing theta grid too small");
  g.dtheta = pi / npoints;
  g.apw = (int)std::lround(0.012 / g.dtheta);
  npoints = (int)(pi / g.dtheta);
  const double range_fac = std::max(1.0, 32 / boost);
  g.npoints = (int)(npoints / range_fac);
  g.interp_fac = std::max(1, std::min((int)std::lround(10 / boost), (int)(range_fac * 2) - 1));
  g.lsj.clear();
  for (int l = g.lmin; l <= g.lmax; ++l)
    if (l <= 15 || (l - 15) % g.interp_fac == g.interp_fac / 2) g.lsj.push_back(l);
  if (g.npoints < 2 || g.lmax_lensed < g.lmin || max_l < 10)
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lensing needs max_l >= 10");
  return 0;
}

// device d-table of a lensing geometry, built on first use and cached
int device_lens_geom(const HostLensGeom& h, LensGeomDev& G) {
  Runtime::DevLensGeom* found = nullptr;
  for (auto& g : g_rt.lens)
    if (h.same(g)) found = &g;
  if (!found) {
    if (g_rt.lens.size() >= 2) {
      auto& o = g_rt.lens.front();
      cudaFree(o.tab);
      cudaFree(o.roots);
      cudaFree(o.sinth);
      cudaFree(o.lsj);
      g_rt.lens.erase(g_rt.lens.begin());
    }
    Runtime::DevLensGeom g{h.lmin, h.lmax, h.npoints, h.apw, h.interp_fac, h.dtheta,
                           nullptr, nullptr, nullptr, nullptr, (int)h.lsj.size()};
    const int npts = h.npoints - 1;
    const size_t ntab = (size_t)7 * (h.lmax + 1) * npts;
    CUDA_TRY(cudaMalloc(&g.tab, ntab * 8));
    CUDA_TRY(cudaMalloc(&g.roots, (size_t)(h.lmax + 6) * 8));
    CUDA_TRY(cudaMalloc(&g.sinth, (size_t)npts * 8));
    CUDA_TRY(cudaMalloc(&g.lsj, h.lsj.size() * 4));
    std::vector<double> roots(h.lmax + 6), sinth(npts);
    roots[0] = 0;
    for (int l = 0; l <= h.lmax + 4; ++l) roots[l + 1] = std::sqrt((double)l);
    for (int ii = 0; ii < npts; ++ii) sinth[ii] = std::sin((ii + 1) * h.dtheta);
    CUDA_TRY(cudaMemcpy(g.roots, roots.data(), roots.size() * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(g.sinth, sinth.data(), sinth.size() * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(g.lsj, h.lsj.data(), h.lsj.size() * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemsetAsync(g.tab, 0, ntab * 8, g_rt.stream));
    CUDA_TRY(launch_lens_geom(g.tab, h.lmin, h.lmax, npts, h.dtheta, g_rt.stream));
    g_launches++;
    g_rt.lens.push_back(g);
    found = &g_rt.lens.back();
  }
  G.tab = found->tab;
  G.roots = found->roots;
  G.sinth = found->sinth;
  G.lsj = found->lsj;
  G.nj = found->nj;
  G.lmin = h.lmin;
  G.lmax = h.lmax;
  G.npts = h.npoints - 1;
  G.npoints = h.npoints;
  G.apodize_point_width = h.apw;
  G.interp_fac = h.interp_fac;
  G.dtheta = h.dtheta;
  return 0;
}

// per-cosmology upload plan
struct Upload {
  const CambGpuTables* t;
  const std::vector<double>* pre_tgrid = nullptr;  // inv_tgrid formed with the host tables, if any
  std::vector<double> spl;  // [5][nk]
  std::vector<double> inv_q;  // 1/nu_q
  std::vector<double> inv_tgrid;  // 1/tau_j of the thermal log grid
  std::vector<double> lfac;       // [3][nl] per sampled l: x_lim, sqrt(pi/2/(l+1/2)), doint threshold
  std::vector<double> tdist;      // [ntau] tau0 - tau_i
  std::vector<float> tdpf;        // [ntau] dtau_i in FP32
  DevCosmo d;
};

size_t bytes_for(const CambGpuTables& t) {
  auto r = [](size_t b) { return (b + 255) & ~size_t(255); };
  size_t s = 0;
  s += r((size_t)t.nthermo * 16 * 8) + 4 * r((size_t)t.nthermo * 8) + r(((size_t)t.nthermo + 1) * 8);
  s += 2 * r((size_t)t.ntau * 8) + r((size_t)t.nk * sizeof(CambGpuModeSpec)) + r((size_t)t.nk * 8);
  s += 2 * r((size_t)t.ntau * t.nsrc * t.nk * 8);
  s += r((size_t)t.nq * t.nl * t.nsrc * 8) + r((size_t)t.nl * 6 * 8);
  s += 2 * r((size_t)t.nq * 8) + r((size_t)t.nl * 4) + r(5 * (size_t)t.nk * 8) + r(256) + r((size_t)t.nl * 24);
  s += r((size_t)t.ntau * 8) + r((size_t)t.ntau * 4);  // tau0 - tau_i, FP32 dtau_i
  s += r((size_t)t.nq * 8);                            // C_l k-integral weights
  s += 3 * r((size_t)t.nqmax * 8) + r((size_t)t.nu_eig * t.nqmax * 8);  // neutrino momenta, weights, switch times
  s += r((size_t)(t.max_l + 1) * 6 * 8) + r((size_t)(t.max_l + 1) * 4 * 8);  // all-l C_l, lensed C_l
  if (t.transfer_only)
    s += r((size_t)t.num_transfer_times * 8) + r((size_t)t.num_transfer_times * t.nk * 13 * 4) +
         r((size_t)t.num_transfer_times * 16);
  return s;
}

// 1/tau_j on the thermal log grid tau_j = tauminn exp(j dlntau), j = 0..nthermo
void thermal_inverse_grid(int nthermo, double tauminn, double dlntau, std::vector<double>& out) {
  out.resize((size_t)nthermo + 1);
  for (int j = 0; j <= nthermo; ++j) out[j] = 1.0 / (tauminn * std::exp(j * dlntau));
}

void spline_factors(const CambGpuTables& t, std::vector<double>& spl) {
  int n = t.nk;
  const double* x = t.q_evolve;
  spl.assign(5 * (size_t)n, 0.0);
  double *inv_dx = &spl[0], *sig = &spl[n], *pinv = &spl[2 * n], *fac = &spl[3 * n], *c6 = &spl[4 * n];
  for (int i = 0; i < n - 1; ++i) inv_dx[i] = 1.0 / (x[i + 1] - x[i]);
  fac[0] = 0;
  for (int i = 1; i < n - 1; ++i) {
    sig[i] = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig[i] * fac[i - 1] + 2.0;
    pinv[i] = 1.0 / p;
    fac[i] = (sig[i] - 1.0) / p;
    c6[i] = 6.0 / (x[i + 1] - x[i - 1]);
  }
}

// copy host arrays into the arena and fill the device view; H2D on the runtime stream
int upload(Upload& u, int* status_dev, std::vector<std::pair<void*, std::pair<const void*, size_t>>>& copies) {
  const CambGpuTables& t = *u.t;
  DevCosmo& d = u.d;
  std::memset(&d, 0, sizeof(d));
  auto put = [&](const void* src, size_t bytes) {
    char* p = g_rt.arena.take<char>(bytes);
    copies.push_back({p, {src, bytes}});
    return p;
  };
  d.grhog = t.grhog; d.grhornomass = t.grhornomass; d.grhoc = t.grhoc; d.grhob = t.grhob; d.grhov = t.grhov;
  d.tau0 = t.tau0; d.taurend = t.taurend; d.tau_maxvis = t.tau_maxvis; d.matter_verydom_tau = t.matter_verydom_tau;
  d.photbar_a = t.grhog / t.grhob;
  d.nu_eig = t.nu_eig;
  d.nqmax = t.nqmax;
  for (int i = 0; i < 3; ++i) {
    d.nu_masses[i] = t.nu_masses[i];
    d.grhormass[i] = t.grhormass[i];
    d.nu_tau_nonrel[i] = t.nu_tau_nonrel[i];
  }
  d.photbar_fac = 0.75 / d.photbar_a;
  if (t.nu_eig > 0) {
    u.inv_q.resize(t.nqmax);
    for (int i = 0; i < t.nqmax; ++i) u.inv_q[i] = 1.0 / t.nu_q[i];
    d.nu_inv_q = (const double*)put(u.inv_q.data(), (size_t)t.nqmax * 8);
    d.nu_q = (const double*)put(t.nu_q, (size_t)t.nqmax * 8);
    d.nu_int_kernel = (const double*)put(t.nu_int_kernel, (size_t)t.nqmax * 8);
    d.nu_tau_notmassless = (const double*)put(t.nu_tau_notmassless, (size_t)t.nu_eig * t.nqmax * 8);
  }
  d.thermo_horner = (const double*)put(t.thermo_horner, (size_t)t.nthermo * 16 * 8);
  d.dddotmu = (const double*)put(t.dddotmu, (size_t)t.nthermo * 8);
  d.ddddotmu = (const double*)put(t.ddddotmu, (size_t)t.nthermo * 8);
  d.emmu = (const double*)put(t.emmu, (size_t)t.nthermo * 8);
  d.demmu = (const double*)put(t.demmu, (size_t)t.nthermo * 8);
  d.nthermo = t.nthermo;
  d.tauminn = t.tauminn; d.inv_tauminn = 1.0 / t.tauminn; d.dlntau = t.dlntau; d.dlntau_inv = t.dlntau_inv;
  d.dlntau_inv_log2 = (float)(0.69314718055994530942 * t.dlntau_inv);
  if (u.pre_tgrid && u.pre_tgrid->size() == (size_t)t.nthermo + 1) {
    d.inv_tgrid = (const double*)put(u.pre_tgrid->data(), u.pre_tgrid->size() * 8);
  } else {
    thermal_inverse_grid(t.nthermo, t.tauminn, t.dlntau, u.inv_tgrid);
    d.inv_tgrid = (const double*)put(u.inv_tgrid.data(), u.inv_tgrid.size() * 8);
  }
  int e = t.nthermo - 1;
  d.cs2_end = t.cs2[e]; d.dotmu_end = t.dotmu[e]; d.ddotmu_end = t.ddotmu[e]; d.dddotmu_end = t.dddotmu[e];
  d.emmu_end = t.emmu[e];
  d.tau_points = (const double*)put(t.tau_points, (size_t)t.ntau * 8);
  d.tau_dpoints = (const double*)put(t.tau_dpoints, (size_t)t.ntau * 8);
  d.ntau = t.ntau;
  // per time step of the mixed projection's staging: the distance to today and the step
  // width in FP32, formed here once instead of in every CTA
  u.tdist.resize(t.ntau);
  u.tdpf.resize(t.ntau);
  for (int i = 0; i < t.ntau; ++i) {
    u.tdist[i] = t.tau0 - t.tau_points[i];
    u.tdpf[i] = (float)t.tau_dpoints[i];
  }
  d.tau_dist = (const double*)put(u.tdist.data(), (size_t)t.ntau * 8);
  // the time grid's runs of uniform spacing (SetTimeSteps adds a few uniform ranges), for the
  // mixed projection's window ends
  {
    const double* x = t.tau_points;
    int k = 0;
    d.ntseg = 0;
    while (k < t.ntau - 1) {
      const double h = x[k + 1] - x[k];
      int e = k + 1;
      while (e < t.ntau - 1 && std::fabs((x[e + 1] - x[e]) - h) <= 1e-6 * h) ++e;
      if (d.ntseg == cgdev::kTimeSegMax) {
        d.ntseg = 0;
        break;
      }
      d.tseg_x0[d.ntseg] = x[k];
      d.tseg_inv_h[d.ntseg] = (e - k) / (x[e] - x[k]);
      d.tseg_i0[d.ntseg] = k;
      d.tseg_n[d.ntseg] = e - k;
      ++d.ntseg;
      k = e;
    }
  }
  d.tau_dpf = (const float*)put(u.tdpf.data(), (size_t)t.ntau * 4);
  d.modes = (const CambGpuModeSpec*)put(t.modes, (size_t)t.nk * sizeof(CambGpuModeSpec));
  d.q_evolve = (const double*)put(t.q_evolve, (size_t)t.nk * 8);
  d.nk = t.nk;
  d.status = status_dev;
  d.q_int = (const double*)put(t.q_int, (size_t)t.nq * 8);
  d.dq_int = (const double*)put(t.dq_int, (size_t)t.nq * 8);
  d.nq = t.nq;
  d.ls = (const int*)put(t.ls, (size_t)t.nl * 4);
  d.nl = t.nl;
  // l-only factors of the projection windows and the Limber value (DoFlatIntegration,
  // cmbmain.f90:1702-1716, 1821-1832), for the mixed-precision projection
  u.lfac.resize(3 * (size_t)t.nl);
  const double bib = t.AccuracyBoost * t.BessIntBoost;
  for (int j = 0; j < t.nl; ++j) {
    const double l = t.ls[j];
    u.lfac[j] = std::fmax(0.0, l - 4.2 * std::cbrt(l));
    u.lfac[t.nl + j] = std::sqrt(3.14159265358979323846 / 2 / (l + 0.5));
    // the lensed-run integration test's threshold on q, as the kernel's FP64 form forms it
    u.lfac[2 * (size_t)t.nl + j] = std::max(850, t.ls[j]) * 3 * bib / t.tau0 * 1.2;
  }
  d.l_xlim = (const double*)put(u.lfac.data(), u.lfac.size() * 8);
  d.l_limb = d.l_xlim + t.nl;
  d.l_doint = d.l_xlim + 2 * (size_t)t.nl;
  d.max_l = t.max_l;
  d.cl_template_scale = t.cl_template_scale;
  d.lensed = nullptr;
  d.lmax_lensed = 0;
  spline_factors(t, u.spl);
  double *bh = nullptr, *bx = nullptr;
  float4* bf = nullptr;
  if (t.bessel_horner) {  // transfer-function cosmologies have no Bessel table
    const Runtime::DevBessel* be = nullptr;
    int rc = device_bessel(t, &bh, &bx, &bf, &be);
    if (rc) return rc;
    d.bess_inv_dxf = be->inv_dxf;
    d.nseg = be->nseg;
    for (int r = 0; r < be->nseg; ++r) {
      d.seg_x0[r] = be->seg_x0[r];
      d.seg_inv_h[r] = be->seg_inv_h[r];
      d.seg_i0[r] = be->seg_i0[r];
      d.seg_n[r] = be->seg_n[r];
    }
  }
  d.bessel_horner = bh;
  d.bessel_f32 = bf;
  d.transfer_only = t.transfer_only;
  d.want_cls = t.want_cls;
  d.hubble_h = t.hubble_h;
  d.late_phot_boost_min = t.late_phot_switch_boost_min;
  d.n_tt = t.transfer_only ? t.num_transfer_times : 0;
  if (t.transfer_only) {
    d.transfer_times = (const double*)put(t.transfer_times, (size_t)t.num_transfer_times * 8);
  }
  // outputs and scratch after every uploaded array, so that the uploads are contiguous
  d.linear_src = g_rt.arena.take<double>((size_t)t.ntau * t.nsrc * t.nk);
  d.dd_src = g_rt.arena.take<double>((size_t)t.ntau * t.nsrc * t.nk);
  d.delta = g_rt.arena.take<double>((size_t)t.nq * t.nl * t.nsrc);
  d.icl = g_rt.arena.take<double>((size_t)t.nl * 6);
  d.pk_w = g_rt.arena.take<double>((size_t)t.nq);
  d.all_cl = g_rt.arena.take<double>((size_t)(t.max_l + 1) * 6);
  if (t.transfer_only) {
    d.transfer_out = g_rt.arena.take<float>((size_t)t.num_transfer_times * t.nk * 13);
    d.sigma8 = g_rt.arena.take<double>((size_t)t.num_transfer_times * 2);
  }
  d.bess_x = bx;
  d.num_xx = t.num_xx;
  d.src_keep_tau = t.src_keep_tau;
  d.tr_src_modes = t.transfer_source_modes;
  d.nsrc = t.nsrc; d.want_late_time = t.want_late_time; d.max_etak_scalar = t.max_etak_scalar; d.tol1 = t.tol1;
  d.AccuracyBoost = t.AccuracyBoost; d.IntTolBoost = t.IntTolBoost; d.TimeSwitchBoost = t.TimeSwitchBoost;
  d.BessIntBoost = t.BessIntBoost; d.LimberBoost = t.LimberBoost;
  d.As = t.As; d.ns = t.ns; d.nrun = t.nrun; d.pivot_scalar = t.pivot_scalar; d.Alens = t.Alens;
  return 0;
}

// A batch resident on the device
struct Batch {
  std::vector<const CambGpuTables*> views;
  std::vector<const std::vector<double>*> tgrid;  // per view: inv_tgrid built with its tables, or empty
  std::vector<Upload> ups;
  DevCosmo* d_cosmos = nullptr;
  const double** d_spl = nullptr;
  WorkItem* d_items = nullptr;
  WorkItem* d_items_rev = nullptr;
  std::vector<WorkItem> h_items_rev;
  WorkItem* d_items_grp = nullptr;  // q bands, cosmologies of similar neutrino mass together
  std::vector<WorkItem> h_items_grp;
  // queue order 3: decreasing measured cost (evaluations x system size) of the last run
  WorkItem* d_items_cost = nullptr;
  std::vector<WorkItem> h_items_cost;
  // queue order 4: the static-stride queue of a launch of bal_threads threads, balanced by
  // the last run's measured costs (build_balanced_order); bal_n entries incl. empty slots
  // shared grids (cambgpu_batch_prepare_shared): the comoving-distance nodes every
  // cosmology's time steps are taken from, for the tensor-core projection (precision 2)
  bool shared = false;
  std::vector<double> h_chi, h_dchi;
  std::vector<float> h_dchi_f;
  double *d_chi = nullptr, *d_dchi = nullptr;
  float* d_dchi_f = nullptr;
  float2* d_tsrc = nullptr;  // [nk][nsrc][nchi][n] FP32 {source, d2} pairs (tensor-core projection)
  int* d_tc_err = nullptr;
  WorkItem* d_items_bal = nullptr;
  size_t bal_cap = 0;
  int bal_threads = 0, bal_n = 0, bal_gen = 0, bal_tried = 0;
  bool bal_estimated = false;        // the balanced queue was built from the cost prior
  unsigned* d_mode_evals = nullptr;  // [nitems], cosmology-major
  std::vector<size_t> mode_base;     // first mode_evals entry of each cosmology
  bool costs_valid = false, cost_order = false;
  int nitems = 0;
  int* d_counter = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_evals = nullptr;
  int max_ntau = 0, max_nq = 0, max_nl = 0, max_rows = 0;
  bool massive_nu = false;  // some cosmology has massive neutrinos (thread-per-mode kernel only)
  bool transfer = false;    // transfer functions only (every cosmology of the batch)
  int warp_stride = 0;      // state-row length of the warp-per-mode kernel (largest system)
  // cosmologies to lens, grouped by lensing geometry
  struct LensGroup {
    HostLensGeom h;
    std::vector<int> cidx;
    int* d_cidx = nullptr;
    double *prep = nullptr, *sg = nullptr, *corr = nullptr;
    int lmax_lensed_max = 0;
  };
  std::vector<LensGroup> lens_groups;
  // packed outputs [n][out_lmax+1][4 | 4 | 3]
  int out_lmax = 0;
  double *d_unl = nullptr, *d_len = nullptr, *d_pot = nullptr;
  // repeated runs of a resident batch replay the stage sequence as a CUDA graph,
  // captured on the second run (the first one allocates the lazily built device tables)
  int runs = 0;
  unsigned long staged_epoch = 0;  // the arena holds this batch while no later staging happened
  long long graph_key = -1;
  cudaGraphExec_t graph = nullptr;
  long long graph_launches = 0;
};

int stage_batch(Batch& B, int lmax_out = 0) {
  int rc = rt_init();
  if (rc) return rc;
  ++g_rt.epoch;
  B.staged_epoch = g_rt.epoch;
  int n = (int)B.views.size();
  size_t total = 0;
  for (auto* v : B.views) total += bytes_for(*v);
  // lensing groups and their scratch
  B.lens_groups.clear();
  std::vector<int> lens_lmax_lensed(n, 0);
  for (int c = 0; c < n; ++c) {
    const CambGpuTables& v = *B.views[c];
    if (v.nl > 512) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "too many sampled l");
    if (!v.do_lensing) continue;
    HostLensGeom h;
    rc = lens_geometry(v, h);
    if (rc) return rc;
    lens_lmax_lensed[c] = h.lmax_lensed;
    Batch::LensGroup* grp = nullptr;
    for (auto& g : B.lens_groups)
      if (g.h.lmax == h.lmax && g.h.npoints == h.npoints && g.h.apw == h.apw && g.h.interp_fac == h.interp_fac &&
          g.h.dtheta == h.dtheta)
        grp = &g;
    if (!grp) {
      B.lens_groups.push_back(Batch::LensGroup{});
      grp = &B.lens_groups.back();
      grp->h = h;
    }
    grp->cidx.push_back(c);
    grp->lmax_lensed_max = std::max(grp->lmax_lensed_max, h.lmax_lensed);
  }
  auto rr = [](size_t b) { return (b + 255) & ~size_t(255); };
  for (auto& g : B.lens_groups) {
    size_t nc = g.cidx.size(), npts = (size_t)g.h.npoints - 1, L = (size_t)g.h.lmax + 1;
    total += rr(nc * 4) + rr(nc * 4 * L * 8) + rr(nc * npts * 2 * 8) + rr(4 * npts * nc * 8);
  }
  B.out_lmax = lmax_out;
  for (auto* v : B.views) B.out_lmax = std::max(B.out_lmax, v->max_l);
  total += 2 * rr((size_t)n * (B.out_lmax + 1) * 4 * 8) + rr((size_t)n * (B.out_lmax + 1) * 3 * 8);
  size_t nitems = 0;
  for (auto* v : B.views) nitems += v->nk;
  total += ((size_t)n * sizeof(DevCosmo) + 255) + ((size_t)n * 8 + 255) + 4 * (nitems * sizeof(WorkItem) + 255) +
           1024 + ((size_t)n * 4 + 255) + (nitems * 4 + 255);
  // balanced queue (order 4): the items plus the empty slots of partial rounds
  const size_t bal_cap = 2 * nitems + 2 * (size_t)g_rt.nsm * 2048;
  total += (bal_cap * sizeof(WorkItem) + 255);
  total += 2 * (B.h_chi.size() * 8 + 255) + 256;  // shared chi nodes and weights, error flag
  if (B.shared)  // FP32 weights, transposed FP32 source pairs
    total += (B.h_chi.size() * 4 + 255) +
             ((size_t)B.views[0]->nk * B.views[0]->nsrc * B.h_chi.size() * n * sizeof(float2) + 255);
  rc = g_rt.arena.reserve(total);
  if (rc) return set_err(rc, "device allocation failed");
  B.d_status = g_rt.arena.take<int>(n);
  B.d_counter = g_rt.arena.take<int>(1);
  B.d_evals = g_rt.arena.take<unsigned long long>(1);
  B.d_mode_evals = g_rt.arena.take<unsigned>(nitems);
  B.mode_base.assign(n, 0);
  for (int c = 1; c < n; ++c) B.mode_base[c] = B.mode_base[c - 1] + B.views[c - 1]->nk;
  std::vector<std::pair<void*, std::pair<const void*, size_t>>> copies;
  B.ups.resize(n);
  for (int c = 0; c < n; ++c) {
    B.ups[c].t = B.views[c];
    B.ups[c].pre_tgrid = c < (int)B.tgrid.size() ? B.tgrid[c] : nullptr;
    rc = upload(B.ups[c], B.d_status + c, copies);
    if (rc) return rc;
    B.ups[c].d.evals = B.d_evals;
    B.ups[c].d.mode_evals = B.d_mode_evals + B.mode_base[c];
    B.max_ntau = std::max(B.max_ntau, B.views[c]->ntau);
    B.max_nq = std::max(B.max_nq, B.views[c]->nq);
    B.max_nl = std::max(B.max_nl, B.views[c]->nl);
    B.max_rows = std::max(B.max_rows, B.views[c]->ntau * B.views[c]->nsrc);
    B.massive_nu |= B.views[c]->nu_eig > 0;
    {
      // largest packed system of GetNumEqns: photons, massless neutrinos, the massive
      // eigenstates' full momentum grids and the relativistic perturbation hierarchy
      const CambGpuTables& t = *B.views[c];
      for (int m = 0; m < t.nk; ++m) {
        const CambGpuModeSpec& ms = t.modes[m];
        int nv = 4 + (ms.lmaxg + 1) + (ms.lmaxnr + 1) + ms.lmaxgpol - 1;
        if (t.nu_eig > 0) nv += (ms.lmaxnu + 1) * (1 + t.nu_eig * t.nqmax);
        B.warp_stride = std::max(B.warp_stride, (nv + 1) & ~1);
      }
    }
    if (c == 0) B.transfer = B.views[c]->transfer_only != 0;
    else if (B.transfer != (B.views[c]->transfer_only != 0))
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "a batch is either all CMB or all transfer functions");
  }
  std::vector<DevCosmo> hc(n);
  std::vector<const double*> hspl(n);
  for (int c = 0; c < n; ++c) {
    hc[c] = B.ups[c].d;
    double* p = g_rt.arena.take<double>(B.ups[c].spl.size());
    copies.push_back({p, {B.ups[c].spl.data(), B.ups[c].spl.size() * 8}});
    hspl[c] = p;
  }
  for (int c = 0; c < n; ++c) {
    if (!B.views[c]->do_lensing) continue;
    B.ups[c].d.lmax_lensed = lens_lmax_lensed[c];
    B.ups[c].d.lensed = g_rt.arena.take<double>((size_t)(B.views[c]->max_l + 1) * 4);
    hc[c] = B.ups[c].d;
  }
  for (auto& g : B.lens_groups) {
    size_t nc = g.cidx.size(), npts = (size_t)g.h.npoints - 1, L = (size_t)g.h.lmax + 1;
    g.d_cidx = g_rt.arena.take<int>(nc);
    copies.push_back({g.d_cidx, {g.cidx.data(), nc * 4}});
    g.prep = g_rt.arena.take<double>(nc * 4 * L);
    g.sg = g_rt.arena.take<double>(nc * npts * 2);
    g.corr = g_rt.arena.take<double>(4 * npts * nc);
  }
  B.d_unl = g_rt.arena.take<double>((size_t)n * (B.out_lmax + 1) * 4);
  B.d_len = g_rt.arena.take<double>((size_t)n * (B.out_lmax + 1) * 4);
  B.d_pot = g_rt.arena.take<double>((size_t)n * (B.out_lmax + 1) * 3);
  B.d_cosmos = g_rt.arena.take<DevCosmo>(n);
  copies.push_back({B.d_cosmos, {hc.data(), (size_t)n * sizeof(DevCosmo)}});
  B.d_spl = g_rt.arena.take<const double*>(n);
  copies.push_back({(void*)B.d_spl, {hspl.data(), (size_t)n * 8}});
  // work items: all (cosmology, mode) pairs, highest q first (most expensive first)
  std::vector<WorkItem> items;
  items.reserve(nitems);
  for (int c = 0; c < n; ++c)
    for (int m = 0; m < B.views[c]->nk; ++m) items.push_back({c, m});
  std::stable_sort(items.begin(), items.end(), [&](const WorkItem& a, const WorkItem& b) {
    return B.views[a.cosmo]->q_evolve[a.mode] > B.views[b.cosmo]->q_evolve[b.mode];
  });
  B.nitems = (int)items.size();
  B.d_items = g_rt.arena.take<WorkItem>(items.size());
  copies.push_back({B.d_items, {items.data(), items.size() * sizeof(WorkItem)}});
  // the same items in increasing q (second queue order the autotuner tries)
  B.h_items_rev.assign(items.rbegin(), items.rend());
  B.d_items_rev = g_rt.arena.take<WorkItem>(items.size());
  copies.push_back({B.d_items_rev, {B.h_items_rev.data(), items.size() * sizeof(WorkItem)}});
  // third order: bands of 1.6% in q (high q first), and inside a band the cosmologies by
  // neutrino mass, so that a warp's 32 modes share hierarchy sizes and switch sequences
  B.h_items_grp = items;
  {
    // sort keys formed once per item (band of q, total neutrino mass, q), not per comparison
    struct Key {
      long band;
      double mass, q;
      WorkItem w;
    };
    std::vector<double> mass(n, 0.0);
    for (int c = 0; c < n; ++c)
      for (int i = 0; i < B.views[c]->nu_eig; ++i) mass[c] += B.views[c]->nu_masses[i];
    std::vector<Key> keys;
    keys.reserve(items.size());
    for (const WorkItem& w : items) {
      const double q = B.views[w.cosmo]->q_evolve[w.mode];
      keys.push_back({(long)std::floor(std::log(q) * 64), mass[w.cosmo], q, w});
    }
    std::stable_sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) {
      if (a.band != b.band) return a.band > b.band;
      if (a.mass != b.mass) return a.mass < b.mass;
      return a.q > b.q;
    });
    for (size_t i = 0; i < keys.size(); ++i) B.h_items_grp[i] = keys[i].w;
  }
  B.d_items_grp = g_rt.arena.take<WorkItem>(items.size());
  copies.push_back({B.d_items_grp, {B.h_items_grp.data(), items.size() * sizeof(WorkItem)}});
  // order 3 starts as order 2 and becomes the measured-cost order once a run has recorded
  // every mode's evaluations (build_cost_order)
  B.h_items_cost = B.h_items_grp;
  B.d_items_cost = g_rt.arena.take<WorkItem>(items.size());
  B.d_items_bal = g_rt.arena.take<WorkItem>(bal_cap);
  B.bal_cap = bal_cap;
  B.d_tc_err = g_rt.arena.take<int>(1);
  if (B.shared) {
    B.d_chi = g_rt.arena.take<double>(B.h_chi.size());
    B.d_dchi = g_rt.arena.take<double>(B.h_dchi.size());
    copies.push_back({B.d_chi, {B.h_chi.data(), B.h_chi.size() * 8}});
    copies.push_back({B.d_dchi, {B.h_dchi.data(), B.h_dchi.size() * 8}});
    B.h_dchi_f.assign(B.h_dchi.begin(), B.h_dchi.end());
    B.d_dchi_f = g_rt.arena.take<float>(B.h_dchi_f.size());
    copies.push_back({B.d_dchi_f, {B.h_dchi_f.data(), B.h_dchi_f.size() * 4}});
    B.d_tsrc = g_rt.arena.take<float2>((size_t)B.views[0]->nk * B.views[0]->nsrc * B.h_chi.size() * n);
  }
  copies.push_back({B.d_items_cost, {B.h_items_cost.data(), items.size() * sizeof(WorkItem)}});
  if (g_rt.arena.overflow) return set_err(CAMBGPU_ERROR_ALLOCATION, "device arena sized below its uses (internal)");
  // single pinned staging buffer for all uploads
  size_t stage = 0;
  for (auto& cp : copies) stage += (cp.second.second + 255) & ~size_t(255);
  if (stage > g_rt.pinned_cap) {
    if (g_rt.pinned) cudaFreeHost(g_rt.pinned);
    g_rt.pinned = nullptr;
    g_rt.pinned_cap = 0;
    CUDA_TRY(cudaMallocHost(&g_rt.pinned, stage + (1 << 20)));
    g_rt.pinned_cap = stage + (1 << 20);
  }
  CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
  g_h2d = 0;
  g_d2h = 0;
  // staging offsets, then the host copies into the pinned buffer on all cores
  std::vector<size_t> offs(copies.size());
  {
    size_t off = 0;
    for (size_t i = 0; i < copies.size(); ++i) {
      offs[i] = off;
      g_h2d += (long long)copies[i].second.second;
      off += (copies[i].second.second + 255) & ~size_t(255);
    }
    unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
      th.emplace_back([&]() {
        for (size_t i = next++; i < copies.size(); i = next++)
          std::memcpy(g_rt.pinned + offs[i], copies[i].second.first, copies[i].second.second);
      });
    for (auto& t : th) t.join();
  }
  // one device copy per run of copies that are contiguous on both sides (the arena and the
  // staging buffer use the same 256-byte rounding)
  for (size_t i = 0; i < copies.size();) {
    size_t j = i, bytes = copies[i].second.second;
    while (j + 1 < copies.size() && (char*)copies[j + 1].first == (char*)copies[j].first + (offs[j + 1] - offs[j]) &&
           copies[j + 1].first > copies[j].first) {
      ++j;
      bytes = offs[j] - offs[i] + copies[j].second.second;
    }
    CUDA_TRY(cudaMemcpyAsync(copies[i].first, g_rt.pinned + offs[i], bytes, cudaMemcpyHostToDevice, g_rt.stream));
    i = j + 1;
  }
  CUDA_TRY(cudaMemsetAsync(B.d_status, 0, (size_t)n * 4, g_rt.stream));
  CUDA_TRY(cudaMemsetAsync(B.d_mode_evals, 0, (size_t)B.nitems * 4, g_rt.stream));
  for (int c = 0; c < n; ++c) {
    const auto& v = *B.views[c];
    CUDA_TRY(cudaMemsetAsync(B.ups[c].d.linear_src, 0, (size_t)v.ntau * v.nsrc * v.nk * 8, g_rt.stream));
  }
  return 0;
}

// Lanes per k-mode for the ODE kernel.  The FP64 pipe binds: one thread per mode
// does no redundant scalar work and wins once there are enough modes to fill the
// GPU; a warp per mode has the shortest per-mode latency for small batches.
int size_class(const Batch& B) { return B.nitems >= 24 * g_rt.nsm ? 1 : 0; }

int pick_team(const Batch& B) {
  int t = g_team ? g_team : g_tuned[size_class(B)].team;
  // the register-resident warp kernels (8/16/32 lanes) evolve the massless-neutrino CMB
  // layout only; the shared-memory warp kernel (6) any layout up to kWarpStrideMax entries
  if ((B.massive_nu || B.transfer) && t >= 8) t = 6;
  // the register warp kernels hold at most 128 packed variables (higher lAccuracyBoost)
  if (t >= 8 && B.warp_stride > 128) t = 6;
  if (B.transfer && t > 3 && t != 6) t = 2;
  if (t == 6 && B.warp_stride > kWarpStrideMax) t = 2;
  return t;
}

int ode_order(const Batch& B) { return g_order >= 0 ? g_order : g_tuned[size_class(B)].order; }
int ode_cap(const Batch& B) { return g_blocks_cap > 0 ? g_blocks_cap : g_team ? 0 : g_tuned[size_class(B)].cap; }
int ode_sched(const Batch& B) { return g_sched >= 0 ? g_sched : g_team ? 0 : g_tuned[size_class(B)].sched; }

// blocks and threads per block of the ODE launch
void ode_launch_shape(const Batch& B, int team, int& blocks, int& tpb) {
  const int lanes = (team <= 5 || team == 7) ? 1 : team == 6 ? 32 : team;
  // Few modes (a single cosmology): one warp per block, so that the warps spread over the
  // SMs and none shares an SM's FP64 pipe; otherwise blocks of 128.  The shared-memory
  // warp kernel always runs one warp per block.
  const long threads_needed = (long)B.nitems * lanes;
  tpb = (team == 6 || threads_needed < 2L * 128 * g_rt.nsm) ? 32 : 128;
  int per_sm = std::max(1, ode_blocks_per_sm(team, tpb, B.warp_stride));
  // a cap below the occupancy limit leaves modes in the queue for threads that finish early
  // the cap counts resident threads in units of 128 (a 32-thread-block launch may keep
  // four times as many blocks)
  const int cap = ode_cap(B);
  if (cap > 0) per_sm = std::min(per_sm, cap * (128 / tpb));
  blocks = (int)std::min<long>((long)g_rt.nsm * per_sm, (threads_needed + tpb - 1) / tpb);
  if (blocks < 1) blocks = 1;
}

// the balanced queue applies to thread-per-mode launches with the static-stride schedule
bool balanced_applies(const Batch& B, int team) {
  return ode_order(B) == 4 && (team <= 5 || team == 7) && ode_sched(B) == 1;
}

int run_ode(Batch& B) {
  CUDA_TRY(cudaMemsetAsync(B.d_counter, 0, sizeof(int), g_rt.stream));
  CUDA_TRY(cudaMemsetAsync(B.d_evals, 0, sizeof(unsigned long long), g_rt.stream));
  int team = pick_team(B);
  int order = ode_order(B);
  int blocks, tpb;
  ode_launch_shape(B, team, blocks, tpb);
  const WorkItem* queue = order == 3 ? B.d_items_cost : order == 2 ? B.d_items_grp : order == 1 ? B.d_items_rev : B.d_items;
  int nq = B.nitems;
  if (order == 4) {
    queue = B.d_items_grp;  // until a run has measured the costs, or for other schedules
    if (balanced_applies(B, team) && B.bal_threads == blocks * tpb) {
      queue = B.d_items_bal;
      nq = B.bal_n;
    }
  }
  // static stride: no queue counter (the kernel derives every item from its thread index);
  // only the tpm kernels (teams 1-7) have that schedule, the register warp kernels (8, 16,
  // 32) always take their items from the counter
  int* counter = (ode_sched(B) == 1 && team <= 7) ? nullptr : B.d_counter;
  CUDA_TRY(launch_ode_kernel(team, blocks, tpb, g_rt.stream, B.d_cosmos, queue, nq, counter,
                             B.transfer, B.warp_stride));
  g_launches++;
  return 0;
}

int run_los(Batch& B) {
  int n = (int)B.views.size();
  dim3 g1((B.max_rows + 127) / 128, n);
  if (g_precision == 2) {
    // split hi/lo BF16 tensor-core projection of a batch on shared grids, on the FP64
    // source spline
    if (!B.shared) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "precision 2 needs a batch on shared grids");
    source_spline_kernel<<<g1, 128, 0, g_rt.stream>>>(B.d_cosmos, B.d_spl);
    g_launches++;
    CUDA_TRY(cudaMemsetAsync(B.d_tc_err, 0, sizeof(int), g_rt.stream));
    CUDA_TRY(launch_proj_tc(B.d_cosmos, n, B.max_nq, B.views[0]->nsrc, B.views[0]->nk, B.views[0]->nl, B.d_chi, B.d_dchi_f,
                            (int)B.h_chi.size(), B.d_tsrc, B.d_tc_err, g_rt.stream));
    g_launches += 2;
    return 0;
  }
  // mixed precision: the spline leaves FP32 {source, d2} pairs in dd_src for the FP32 staging
  if (g_precision == 1) source_spline_f32_kernel<<<g1, 128, 0, g_rt.stream>>>(B.d_cosmos, B.d_spl);
  else source_spline_kernel<<<g1, 128, 0, g_rt.stream>>>(B.d_cosmos, B.d_spl);
  g_launches++;
  // every Delta_p_l_k entry is written by the LOS kernel (zeros where it skips)
  dim3 g2(B.max_nq, n);
  if (g_precision == 1) {
    const size_t smem = (size_t)B.max_ntau * (3 + 1 + 1 + 1) * 4 + 64;
    los_flat_mixed_kernel<<<g2, 256, smem, g_rt.stream>>>(B.d_cosmos);
  } else {
    const size_t smem = (size_t)B.max_ntau * (3 + 1 + 1) * 8 + (size_t)B.max_ntau * 4 + 64;
    los_flat_kernel<<<g2, 256, smem, g_rt.stream>>>(B.d_cosmos);
  }
  g_launches++;
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int run_cls(Batch& B) {
  int n = (int)B.views.size();
  // the primordial-power weights once per (cosmology, q), then the k-integral per sampled l
  pk_weight_kernel<<<dim3((B.max_nq + 255) / 256, n), 256, 0, g_rt.stream>>>(B.d_cosmos);
  g_launches++;
  CUDA_TRY(cudaGetLastError());
  dim3 g(B.max_nl, n);
  scal_cls_kernel<<<g, 256, 0, g_rt.stream>>>(B.d_cosmos);
  g_launches++;
  CUDA_TRY(cudaGetLastError());
  // InterpolateCls to every l, then lens_Cls for the cosmologies that want lensing
  double* tmpl = nullptr;
  int rc = device_template(&tmpl);
  if (rc) return rc;
  CUDA_TRY(launch_interp_cls(B.d_cosmos, n, tmpl, g_rt.stream));
  g_launches++;
  for (auto& grp : B.lens_groups) {
    LensGeomDev G;
    rc = device_lens_geom(grp.h, G);
    if (rc) return rc;
    CUDA_TRY(launch_lensing(B.d_cosmos, grp.d_cidx, (int)grp.cidx.size(), tmpl, G, grp.lmax_lensed_max, grp.prep,
                            grp.sg, grp.corr, g_rt.stream));
    g_launches += 4;
  }
  return 0;
}

// packs the requested outputs on the device and copies them to the host
int fetch_spectra(Batch& B, int lmax_out, double* unl, double* len, double* pot) {
  int n = (int)B.views.size();
  if (lmax_out > B.out_lmax) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lmax_out above the staged outputs");
  CUDA_TRY(launch_pack_spectra(B.d_cosmos, n, lmax_out, unl ? B.d_unl : nullptr, len ? B.d_len : nullptr,
                               pot ? B.d_pot : nullptr, g_rt.stream));
  g_launches++;
  size_t m = (size_t)n * (lmax_out + 1);
  if (unl) CUDA_TRY(cudaMemcpyAsync(unl, B.d_unl, m * 4 * 8, cudaMemcpyDeviceToHost, g_rt.stream));
  if (len) CUDA_TRY(cudaMemcpyAsync(len, B.d_len, m * 4 * 8, cudaMemcpyDeviceToHost, g_rt.stream));
  if (pot) CUDA_TRY(cudaMemcpyAsync(pot, B.d_pot, m * 3 * 8, cudaMemcpyDeviceToHost, g_rt.stream));
  CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
  g_d2h += (long long)m * 8 * ((unl ? 4 : 0) + (len ? 4 : 0) + (pot ? 3 : 0));
  return 0;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// runs every stage on a staged batch, with events between stages
// Queue order 3 (longest processing time first): the modes in decreasing order of the
// last run's evaluations times their largest packed system, so that the expensive modes
// start first and cheap ones fill the tail; built once per batch from the first ODE run.
int build_cost_order(Batch& B) {
  std::vector<unsigned> ev(B.nitems);
  CUDA_TRY(cudaMemcpy(ev.data(), B.d_mode_evals, ev.size() * 4, cudaMemcpyDeviceToHost));
  std::vector<std::pair<double, WorkItem>> key;
  key.reserve(B.nitems);
  for (const WorkItem& w : B.h_items_grp) {
    const CambGpuTables& t = *B.views[w.cosmo];
    const CambGpuModeSpec& ms = t.modes[w.mode];
    double nv = 4 + (ms.lmaxg + 1) + (ms.lmaxnr + 1) + ms.lmaxgpol - 1;
    if (t.nu_eig > 0) nv += (ms.lmaxnu + 1) * (1 + t.nu_eig * t.nqmax);
    key.push_back({(double)ev[B.mode_base[w.cosmo] + w.mode] * nv, w});
  }
  std::stable_sort(key.begin(), key.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  for (int i = 0; i < B.nitems; ++i) B.h_items_cost[i] = key[i].second;
  CUDA_TRY(cudaMemcpy(B.d_items_cost, B.h_items_cost.data(), (size_t)B.nitems * sizeof(WorkItem),
                      cudaMemcpyHostToDevice));
  B.cost_order = true;
  return 0;
}

// Evaluations per mode as a function of ln q, recorded from the first run of the last batch
// whose costs were measured, for batches of the same kind (l range, sources, massive
// neutrinos, transfer functions): a fresh batch's first run then starts on a balanced queue
// built from these estimates instead of the q-band order.  Any queue holds every mode once,
// so the estimates change the schedule only, never the results.
struct CostPrior {
  long long sig = -1;
  double lq0 = 0, dlq = 1;
  std::vector<double> ev;  // mean evaluations per ln q bin (interpolated over empty bins)
};
CostPrior g_cost_prior;

long long cost_signature(const Batch& B) {
  const CambGpuTables& t = *B.views[0];
  return ((long long)t.max_l * 8 + t.nsrc) * 4 + (B.massive_nu ? 2 : 0) + (B.transfer ? 1 : 0);
}

int record_cost_prior(Batch& B) {
  std::vector<unsigned> ev(B.nitems);
  CUDA_TRY(cudaMemcpy(ev.data(), B.d_mode_evals, ev.size() * 4, cudaMemcpyDeviceToHost));
  double lo = 1e300, hi = -1e300;
  for (const WorkItem& w : B.h_items_grp) {
    const double lq = std::log(B.views[w.cosmo]->modes[w.mode].q);
    lo = std::min(lo, lq);
    hi = std::max(hi, lq);
  }
  const int nb = 128;
  CostPrior P;
  P.sig = cost_signature(B);
  P.lq0 = lo;
  P.dlq = std::max(hi - lo, 1e-12) / (nb - 1);
  std::vector<double> sum(nb, 0.0), cnt(nb, 0.0);
  for (const WorkItem& w : B.h_items_grp) {
    const double lq = std::log(B.views[w.cosmo]->modes[w.mode].q);
    const int b = std::min(nb - 1, std::max(0, (int)std::lround((lq - lo) / P.dlq)));
    sum[b] += ev[B.mode_base[w.cosmo] + w.mode];
    cnt[b] += 1;
  }
  P.ev.assign(nb, 0.0);
  int last = -1;
  for (int b = 0; b < nb; ++b) {
    if (cnt[b] == 0) continue;
    P.ev[b] = sum[b] / cnt[b];
    for (int e = last + 1; e < b; ++e)  // empty bins: linear between filled neighbours
      P.ev[e] = last < 0 ? P.ev[b] : P.ev[last] + (P.ev[b] - P.ev[last]) * (e - last) / (b - last);
    last = b;
  }
  for (int e = last + 1; e < nb && last >= 0; ++e) P.ev[e] = P.ev[last];
  g_cost_prior = std::move(P);
  return 0;
}

// estimated evaluations of every mode (cosmology-major, as d_mode_evals) from the prior
std::vector<unsigned> estimated_evals(const Batch& B) {
  const CostPrior& P = g_cost_prior;
  std::vector<unsigned> ev(B.nitems, 0);
  const int nb = (int)P.ev.size();
  for (const WorkItem& w : B.h_items_grp) {
    const double x = (std::log(B.views[w.cosmo]->modes[w.mode].q) - P.lq0) / P.dlq;
    const int b = std::min(nb - 2, std::max(0, (int)std::floor(x)));
    const double f = std::min(1.0, std::max(0.0, x - b));
    ev[B.mode_base[w.cosmo] + w.mode] = (unsigned)(P.ev[b] + f * (P.ev[b + 1] - P.ev[b]) + 0.5);
  }
  return ev;
}

bool cost_prior_applies(const Batch& B) {
  return g_cost_prior.ev.size() >= 2 && g_cost_prior.sig == cost_signature(B);
}

// Queue order 4 for a static-stride launch of T threads (thread t takes entries t, t + T,
// t + 2T, ...): the q-band order (2) cut into bundles of 32 neighbouring modes -- one warp's
// lanes, which share hierarchy sizes and switch sequences -- and the bundles dealt to the
// T/32 warps longest first, each to the warp with the least work so far (LPT), the cost of a
// bundle being its costliest mode's evaluations x system size in the last run.  Warps are
// then ranked by their number of bundles so that round k of the stride holds the k-th
// bundles of the warps that have one; the few slots left over are empty (cosmo = -1).
// The costs are the last run's measured evaluations, or, before the batch has run, the
// cost prior's estimates (estimated = true).
int build_balanced_order(Batch& B, int T, bool estimated = false) {
  B.bal_tried = T;
  B.bal_estimated = estimated;
  std::vector<unsigned> ev(B.nitems);
  if (estimated) ev = estimated_evals(B);
  else CUDA_TRY(cudaMemcpy(ev.data(), B.d_mode_evals, ev.size() * 4, cudaMemcpyDeviceToHost));
  const int nw = std::max(1, T / 32);
  const int nb = (B.nitems + 31) / 32;
  std::vector<double> bcost(nb, 0.0);
  for (int i = 0; i < B.nitems; ++i) {
    const WorkItem& w = B.h_items_grp[i];
    const CambGpuTables& t = *B.views[w.cosmo];
    const CambGpuModeSpec& ms = t.modes[w.mode];
    double nv = 4 + (ms.lmaxg + 1) + (ms.lmaxnr + 1) + ms.lmaxgpol - 1;
    if (t.nu_eig > 0) nv += (ms.lmaxnu + 1) * (1 + t.nu_eig * t.nqmax);
    bcost[i / 32] = std::max(bcost[i / 32], (double)ev[B.mode_base[w.cosmo] + w.mode] * nv);
  }
  std::vector<int> border(nb);
  for (int b = 0; b < nb; ++b) border[b] = b;
  std::stable_sort(border.begin(), border.end(), [&](int a, int b) { return bcost[a] > bcost[b]; });
  std::vector<double> load(nw, 0.0);
  std::vector<std::vector<int>> wb(nw);
  // min-heap of (load, warp)
  std::vector<std::pair<double, int>> heap;
  for (int w = 0; w < nw; ++w) heap.push_back({0.0, w});
  auto cmp = [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
    return a.first > b.first || (a.first == b.first && a.second > b.second);
  };
  std::make_heap(heap.begin(), heap.end(), cmp);
  for (int b : border) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto top = heap.back();
    heap.pop_back();
    wb[top.second].push_back(b);
    top.first += bcost[b];
    heap.push_back(top);
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  std::vector<int> rank(nw);
  for (int w = 0; w < nw; ++w) rank[w] = w;
  std::stable_sort(rank.begin(), rank.end(), [&](int a, int b) { return wb[a].size() > wb[b].size(); });
  const WorkItem empty{-1, 0};
  std::vector<WorkItem> q;
  size_t rounds = wb[rank[0]].size();
  for (size_t k = 0; k < rounds; ++k) {
    for (int r = 0; r < nw; ++r) {
      const std::vector<int>& bl = wb[rank[r]];
      if (k >= bl.size()) break;  // ranked by bundle count: no later warp has round k
      for (int l = 0; l < 32; ++l) {
        const int i = bl[k] * 32 + l;
        q.push_back(i < B.nitems ? B.h_items_grp[i] : empty);
      }
    }
    // threads beyond the ranked warps (T not a multiple of 32) and the rest of the round
    if (k + 1 < rounds) {
      size_t full = (size_t)(k + 1) * T;
      while (q.size() < full) q.push_back(empty);
    }
  }
  B.bal_gen++;
  if (q.size() > B.bal_cap) {  // too many partial rounds: keep the q-band order
    B.bal_threads = -1;
    B.bal_n = 0;
    return 0;
  }
  CUDA_TRY(cudaMemcpy(B.d_items_bal, q.data(), q.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
  B.bal_n = (int)q.size();
  B.bal_threads = T;
  return 0;
}

// under stream capture the stage boundaries are external event records, so that in the
// graph they stay event-record nodes the host can time and wait on
int enqueue_all(Batch& B, bool do_ode, bool do_los, bool do_cls, bool capturing) {
  cudaStream_t s = g_rt.stream;
  const unsigned fl = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  CUDA_TRY(cudaEventRecordWithFlags(g_rt.ev[0], s, fl));
  if (do_ode) { int rc = run_ode(B); if (rc) return rc; }
  CUDA_TRY(cudaEventRecordWithFlags(g_rt.ev[1], s, fl));
  if (do_los) { int rc = run_los(B); if (rc) return rc; }
  CUDA_TRY(cudaEventRecordWithFlags(g_rt.ev[2], s, fl));
  if (do_cls) { int rc = run_cls(B); if (rc) return rc; }
  CUDA_TRY(cudaEventRecordWithFlags(g_rt.ev[3], s, fl));
  return 0;
}

// everything the enqueued sequence depends on besides the batch itself
long long run_key(const Batch& B, bool do_ode, bool do_los, bool do_cls) {
  long long k = pick_team(B);
  k = k * 8 + (ode_order(B) + 1);
  k = k * 64 + ode_cap(B);
  k = k * 2 + ode_sched(B);
  k = k * 4 + g_precision;
  k = k * 4096 + (B.bal_gen & 4095);  // each build of the balanced queue is a new graph
  return k * 8 + (do_ode ? 4 : 0) + (do_los ? 2 : 0) + (do_cls ? 1 : 0);
}

int capture_graph(Batch& B, bool do_ode, bool do_los, bool do_cls, long long key) {
  cudaStream_t s = g_rt.stream;
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
    B.graph_key = -1;
  }
  const long long l0 = g_launches.load();
  CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_all(B, do_ode, do_los, do_cls, true);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);  // always leave capture mode
  B.graph_launches = g_launches.load() - l0;
  g_launches = l0;
  if (rc || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return rc ? rc : set_err(CAMBGPU_ERROR_CUDA, cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&B.graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    B.graph = nullptr;
    return set_err(CAMBGPU_ERROR_CUDA, cudaGetErrorString(e));
  }
  B.graph_key = key;
  return 0;
}

int run_all(Batch& B, bool do_ode, bool do_los, bool do_cls) {
  cudaStream_t s = g_rt.stream;
  if (do_ode && B.costs_valid && !B.cost_order && ode_order(B) == 3) {
    int rc = build_cost_order(B);  // outside any capture: a synchronous copy each way
    if (rc) return rc;
  }
  if (do_ode) {
    const int team = pick_team(B);
    int blocks, tpb;
    ode_launch_shape(B, team, blocks, tpb);
    if (balanced_applies(B, team)) {
      int rc = 0;  // outside any capture
      if (B.costs_valid && (B.bal_tried != blocks * tpb || B.bal_estimated))
        rc = build_balanced_order(B, blocks * tpb);
      else if (!B.costs_valid && B.bal_tried != blocks * tpb && cost_prior_applies(B))
        rc = build_balanced_order(B, blocks * tpb, true);
      if (rc) return rc;
    }
  }
  if (B.runs == 0) {
    int rc = enqueue_all(B, do_ode, do_los, do_cls, false);
    if (rc) return rc;
  } else {
    const long long key = run_key(B, do_ode, do_los, do_cls);
    if (key != B.graph_key) {
      int rc = capture_graph(B, do_ode, do_los, do_cls, key);
      if (rc) return rc;
    }
    CUDA_TRY(cudaGraphLaunch(B.graph, s));
    g_launches += B.graph_launches;
  }
  B.runs++;
  CUDA_TRY(cudaEventSynchronize(g_rt.ev[3]));
  if (do_ode && !B.costs_valid) {
    B.costs_valid = true;
    int rc = record_cost_prior(B);  // the first measured costs of this batch
    if (rc) return rc;
  }
  g_timings[0] = elapsed(g_rt.ev[0], g_rt.ev[1]);
  g_timings[1] = 0;
  g_timings[2] = elapsed(g_rt.ev[1], g_rt.ev[2]);
  g_timings[3] = elapsed(g_rt.ev[2], g_rt.ev[3]);
  if (do_ode) {
    unsigned long long ev = 0;
    CUDA_TRY(cudaMemcpy(&ev, B.d_evals, sizeof(ev), cudaMemcpyDeviceToHost));
    g_last_evals = (long long)ev;
  }
  if (do_los && g_precision == 2) {
    int terr = 0;
    CUDA_TRY(cudaMemcpy(&terr, B.d_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (terr) return set_err(CAMBGPU_ERROR_CUDA, "tensor-core projection: a completion wait ran out");
  }
  return 0;
}

int check_status(const Batch& B, int* status_out) {
  std::vector<int> st(B.views.size());
  CUDA_TRY(cudaMemcpy(st.data(), B.d_status, st.size() * 4, cudaMemcpyDeviceToHost));
  int worst = 0;
  for (size_t i = 0; i < st.size(); ++i) {
    if (status_out) status_out[i] = st[i];
    if (st[i]) worst = st[i];
  }
  if (worst) set_err(worst, "evolution failed for at least one k-mode");
  return worst;
}

struct Handle {
  cg::Cosmology c;
  std::shared_ptr<const cg::BesselTable> bt;
  CambGpuTables view;
  std::vector<double> inv_tgrid;  // 1/tau_j of the thermal log grid, formed with the tables
  bool combined = false;          // wants the CMB and transfer functions: tview is the latter
  CambGpuTables tview;
};

// a handle's tables (and the thermal inverse grid built with them) into a batch; its
// transfer-function half for a transfer batch of a run that wants the CMB too
void add_handle(Batch& B, Handle* h, bool transfer_half = false) {
  B.views.push_back(transfer_half && h->combined ? &h->tview : &h->view);
  B.tgrid.push_back(&h->inv_tgrid);
}

// transfer functions and sigma8 of a transfer batch staged from hs (each its transfer half
// when it wants the CMB too) into the caller's arrays; synchronises the stream
int fetch_transfers(Batch& B, const std::vector<Handle*>& hs, int nz, int nq_max, float* transfer, int* nq,
                    double* sigma8, double* sigma2_vdelta_8) {
  std::vector<double> s8(2 * (size_t)nz);
  for (size_t c = 0; c < hs.size(); ++c) {
    const CambGpuTables& v = hs[c]->combined ? hs[c]->tview : hs[c]->view;
    if (nq) nq[c] = v.nk;
    if (transfer) {
      for (int z = 0; z < v.num_transfer_times; ++z) {
        float* dst = transfer + (((size_t)c * nz + z) * nq_max) * 13;
        CUDA_TRY(cudaMemcpyAsync(dst, B.ups[c].d.transfer_out + (size_t)z * v.nk * 13, (size_t)v.nk * 13 * 4,
                                 cudaMemcpyDeviceToHost, g_rt.stream));
      }
    }
    if (sigma8 || sigma2_vdelta_8) {
      CUDA_TRY(cudaMemcpyAsync(s8.data(), B.ups[c].d.sigma8, s8.size() * 8, cudaMemcpyDeviceToHost, g_rt.stream));
      CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
      for (int z = 0; z < nz; ++z) {
        if (sigma8) sigma8[c * nz + z] = s8[2 * z];
        if (sigma2_vdelta_8) sigma2_vdelta_8[c * nz + z] = s8[2 * z + 1];
      }
    }
  }
  CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
  return 0;
}

// the transfer-function half of a run that wants the CMB and transfer functions
void fill_transfer_half(Handle* h, const CambGpuParams& p) {
  h->combined = p.want_transfer && p.want_cls;
  if (h->combined) cg::fill_transfer_view(h->c, h->tview);
}

int make_handle(const CambGpuParams* p, Handle*& h) {
  h = new Handle();
  std::string err;
  int rc;
  try {
    rc = cg::build_cosmology(*p, h->c, err);
  } catch (const std::exception& e) {
    rc = CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
    err = e.what();
  }
  if (rc) {
    delete h;
    h = nullptr;
    return set_err(rc, err);
  }
  if (p->want_cls || !p->want_transfer) {
    try {
      h->bt = cg::get_bessel_table(h->c.ls, h->c.maximum_qeta, p->BesselBoost, p->AccuracyBoost);
    } catch (const std::exception& e) {
      delete h;
      h = nullptr;
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, e.what());
    }
    cg::fill_view(h->c, *h->bt, h->view);
    fill_transfer_half(h, *p);
  } else {
    static const cg::BesselTable empty;  // transfer functions need no Bessel table
    cg::fill_view(h->c, empty, h->view);
  }
  return 0;
}

// resident batch for the bench path
struct Resident {
  std::vector<Handle*> handles;
  Batch B;
  ~Resident() {
    if (B.graph) cudaGraphExecDestroy(B.graph);
    for (auto* h : handles) delete h;
  }
};
std::unique_ptr<Resident> g_res;

int build_handles(const CambGpuParams* p, int n, std::vector<Handle*>& hs, int* status) {
  hs.assign(n, nullptr);
  std::vector<int> rcs(n, 0);
  std::vector<std::string> errs(n);
  unsigned nth = std::max(1u, std::min((unsigned)n, std::thread::hardware_concurrency()));
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nth; ++t)
    th.emplace_back([&]() {
      for (;;) {
        int i = next++;
        if (i >= n) break;
        Handle* h = new Handle();
        std::string err;
        int rc;
        try {
          rc = cg::build_cosmology(p[i], h->c, err);
        } catch (const std::exception& e) {
          rc = CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
          err = e.what();
        }
        if (rc) { delete h; h = nullptr; }
        // the per-step thermal inverse grid of the upload, formed here on the building
        // thread (in a stream of batches, while the device runs the previous batch)
        else thermal_inverse_grid(h->c.nthermo, h->c.tauminn, h->c.dlntau, h->inv_tgrid);
        hs[i] = h;
        rcs[i] = rc;
        errs[i] = err;
      }
    });
  for (auto& t : th) t.join();
  int worst = 0;
  for (int i = 0; i < n; ++i) {
    if (status) status[i] = rcs[i];
    if (rcs[i]) { worst = rcs[i]; g_err = errs[i]; }
  }
  for (int i = 0; i < n; ++i) {
    if (!hs[i]) continue;
    if (p[i].want_transfer && !p[i].want_cls) {  // transfer functions need no Bessel table
      static const cg::BesselTable empty;
      cg::fill_view(hs[i]->c, empty, hs[i]->view);
      continue;
    }
    try {
      hs[i]->bt = cg::get_bessel_table(hs[i]->c.ls, hs[i]->c.maximum_qeta, p[i].BesselBoost, p[i].AccuracyBoost);
    } catch (const std::exception& e) {
      g_err = e.what();
      if (status) status[i] = CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
      worst = CAMBGPU_ERROR_UNSUPPORTED_PARAMS;
      delete hs[i];
      hs[i] = nullptr;
      continue;
    }
    cg::fill_view(hs[i]->c, *hs[i]->bt, hs[i]->view);
    fill_transfer_half(hs[i], p[i]);
  }
  return worst;
}


}  // namespace

namespace cgdev {
// the calling thread's error message (cambgpu_last_error), for entry points defined in
// other translation units; returns code
int set_last_error(int code, const char* msg) { return set_err(code, msg); }
}  // namespace cgdev

extern "C" {

void cambgpu_default_params(CambGpuParams* p) {
  std::memset(p, 0, sizeof(*p));
  p->H0 = 67.5; p->ombh2 = 0.022; p->omch2 = 0.122; p->omk = 0; p->TCMB = 2.7255; p->YHe = 0.2454;
  p->nnu = 3.044; p->mnu = 0; p->num_massive_neutrinos = 1; p->optical_depth = 0.06; p->reion_delta_redshift = 0.5;
  p->As = 2.1e-9; p->ns = 0.965; p->nrun = 0; p->pivot_scalar = 0.05; p->Alens = 1;
  p->max_l = 2500; p->max_eta_k = 6250; p->do_lensing = 0;
  p->AccuracyBoost = p->lAccuracyBoost = p->lSampleBoost = p->IntTolBoost = p->TimeStepBoost = 1;
  p->SourcekAccuracyBoost = p->IntkAccuracyBoost = p->BesselBoost = p->BessIntBoost = 1;
  p->TimeSwitchBoost = p->LimberBoost = p->BackgroundTimeStepBoost = 1;
  p->accurate_polarization = 1;
  p->accurate_reionization = 1;
  p->LensingBoost = 1;
  p->want_cls = 1;
  p->want_transfer = 0;
  p->transfer_high_precision = 1;
  p->transfer_kmax = 1.2;  // set_matter_power default kmax
  p->num_transfer_redshifts = 1;
  p->transfer_redshifts[0] = 0;
  p->reion_use_optical_depth = 1;
  p->reion_redshift = 10;
}

int cambgpu_tables_create(const CambGpuParams* p, void** handle) {
  Handle* h = nullptr;
  int rc = make_handle(p, h);
  *handle = h;
  return rc;
}

int cambgpu_tables_view(void* handle, CambGpuTables* view) {
  if (!handle) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "null handle");
  *view = static_cast<Handle*>(handle)->view;
  return 0;
}

int cambgpu_tables_transfer_view(void* handle, CambGpuTables* view) {
  if (!handle) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "null handle");
  const Handle* h = static_cast<Handle*>(handle);
  if (!h->combined) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "not a run that wants the CMB and transfers");
  *view = h->tview;
  return 0;
}

void cambgpu_tables_destroy(void* handle) { delete static_cast<Handle*>(handle); }

int cambgpu_tables_derived(void* handle, double* o) {
  if (!handle) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "null handle");
  const cg::Cosmology& c = static_cast<Handle*>(handle)->c;
  o[0] = c.tau0; o[1] = c.DMt0; o[2] = c.taurst; o[3] = c.taurend; o[4] = c.tau_maxvis;
  o[5] = c.reion.redshift; o[6] = c.z_drag; o[7] = c.scale;
  return 0;
}

int cambgpu_recfast_xe(void* handle, const double* z, int n, double* xe) {
  if (!handle) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "null handle");
  const cg::Cosmology& c = static_cast<Handle*>(handle)->c;
  for (int i = 0; i < n; ++i) xe[i] = c.recfast.x_e(1 / (1 + z[i]));
  return 0;
}

int cambgpu_conformal_time(void* handle, const double* z, int n, double* eta) {
  if (!handle) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "null handle");
  const cg::Cosmology& c = static_cast<Handle*>(handle)->c;
  for (int i = 0; i < n; ++i) eta[i] = c.time_of_z(z[i]);
  return 0;
}

int cambgpu_evolve_scalar_sources(const CambGpuTables* t, double* linear_src) {
  std::lock_guard<std::mutex> lk(g_mu);
  Batch B;
  B.views = {t};
  int rc = stage_batch(B);
  if (rc) return rc;
  rc = run_all(B, true, false, false);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(linear_src, B.ups[0].d.linear_src, (size_t)t->ntau * t->nsrc * t->nk * 8, cudaMemcpyDeviceToHost));
  return check_status(B, nullptr);
}

int cambgpu_los_flat(const CambGpuTables* t, const double* linear_src, double* delta) {
  std::lock_guard<std::mutex> lk(g_mu);
  Batch B;
  B.views = {t};
  int rc = stage_batch(B);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(B.ups[0].d.linear_src, linear_src, (size_t)t->ntau * t->nsrc * t->nk * 8,
                           cudaMemcpyHostToDevice, g_rt.stream));
  rc = run_all(B, false, true, false);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(delta, B.ups[0].d.delta, (size_t)t->nq * t->nl * t->nsrc * 8, cudaMemcpyDeviceToHost));
  return 0;
}

int cambgpu_calc_scal_cls(const CambGpuTables* t, const double* delta, double* icl) {
  std::lock_guard<std::mutex> lk(g_mu);
  Batch B;
  B.views = {t};
  int rc = stage_batch(B);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(B.ups[0].d.delta, delta, (size_t)t->nq * t->nl * t->nsrc * 8, cudaMemcpyHostToDevice,
                           g_rt.stream));
  rc = run_all(B, false, false, true);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(icl, B.ups[0].d.icl, (size_t)t->nl * 6 * 8, cudaMemcpyDeviceToHost));
  return 0;
}

}  // extern "C"

// host tables of a batch built ahead of its device run
struct CambGpuPrepared {
  std::vector<Handle*> hs;
  double host_ms = 0;
  ~CambGpuPrepared() {
    for (auto* h : hs) delete h;
  }
};

extern "C" {

int cambgpu_prepare_tables(const CambGpuParams* p, int n, CambGpuPrepared** out, int* status) {
  if (!out) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "no output handle");
  *out = nullptr;
  if (n < 1) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "empty batch");
  const double t0 = wall_ms();
  auto* t = new CambGpuPrepared();
  int rc = build_handles(p, n, t->hs, status);
  if (rc) {
    delete t;
    return rc;
  }
  t->host_ms = wall_ms() - t0;
  *out = t;
  return 0;
}

void cambgpu_free_prepared(CambGpuPrepared* t) { delete t; }

int cambgpu_get_spectra_prepared(const CambGpuPrepared* t, int lmax_out, double* unlensed, double* lensed,
                                 double* lens_potential, int* lmax_lensed, int* status) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!t || t->hs.empty()) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "no prepared tables");
  if (lmax_out < 0 || lmax_out > 8000) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lmax_out out of range");
  const int n = (int)t->hs.size();
  int rc = 0;
  const double t1 = wall_ms();
  Batch B;
  for (auto* h : t->hs) add_handle(B, h);
  rc = stage_batch(B, lmax_out);
  if (rc) return rc;
  if (B.transfer) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "want_cls = 0: use cambgpu_get_transfer_batch");
  const double t2 = wall_ms();
  rc = run_all(B, true, true, true);
  if (rc) return rc;
  rc = check_status(B, status);
  if (rc) return rc;
  const double t3 = wall_ms();
  if (lmax_lensed)
    for (int c = 0; c < n; ++c) lmax_lensed[c] = B.ups[c].d.lensed ? B.ups[c].d.lmax_lensed : 0;
  rc = fetch_spectra(B, lmax_out, unlensed, lensed, lens_potential);
  const double t4 = wall_ms();
  g_host_ms[0] = t->host_ms;
  g_host_ms[1] = t2 - t1;
  g_host_ms[2] = t3 - t2;
  g_host_ms[3] = t4 - t3;
  return rc;
}

int cambgpu_get_spectra_batch(const CambGpuParams* p, int n, int lmax_out, double* unlensed, double* lensed,
                              double* lens_potential, int* lmax_lensed, int* status) {
  if (lmax_out < 0 || lmax_out > 8000) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lmax_out out of range");
  CambGpuPrepared* t = nullptr;
  int rc = cambgpu_prepare_tables(p, n, &t, status);
  if (rc) return rc;
  rc = cambgpu_get_spectra_prepared(t, lmax_out, unlensed, lensed, lens_potential, lmax_lensed, status);
  cambgpu_free_prepared(t);
  return rc;
}

int cambgpu_last_host_timings(double* out4) {
  for (int i = 0; i < 4; ++i) out4[i] = g_host_ms[i];
  return 0;
}

int cambgpu_get_results_batch(const CambGpuParams* p, int n, int lmax_out, double* cl_out, int* status) {
  return cambgpu_get_spectra_batch(p, n, lmax_out, cl_out, nullptr, nullptr, nullptr, status);
}

int cambgpu_get_transfer_batch(const CambGpuParams* p, int n, int nq_max, float* transfer, int* nq, double* sigma8,
                               double* sigma2_vdelta_8, int* status) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n < 1) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "empty batch");
  for (int c = 0; c < n; ++c) {
    if (!p[c].want_transfer) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "transfer batches need want_transfer = 1");
    if (p[c].num_transfer_redshifts != p[0].num_transfer_redshifts)
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "every cosmology of a transfer batch needs the same redshift count");
  }
  std::vector<Handle*> hs;
  int rc = build_handles(p, n, hs, status);
  struct Guard { std::vector<Handle*>& h; ~Guard() { for (auto* x : h) delete x; } } guard{hs};
  if (rc) return rc;
  // a run that wants the CMB too contributes its transfer-function half
  auto half = [](const Handle* h) -> const CambGpuTables& { return h->combined ? h->tview : h->view; };
  for (auto* h : hs)
    if (transfer && half(h).nk > nq_max) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "nq_max too small");
  Batch B;
  for (auto* h : hs) add_handle(B, h, true);
  rc = stage_batch(B);
  if (rc) return rc;
  rc = run_all(B, true, false, false);
  if (rc) return rc;
  CUDA_TRY(launch_sigma8(B.d_cosmos, n, g_rt.stream));
  g_launches++;
  rc = check_status(B, status);
  if (rc) return rc;
  return fetch_transfers(B, hs, p[0].num_transfer_redshifts, nq_max, transfer, nq, sigma8, sigma2_vdelta_8);
}

int cambgpu_get_results_with_transfers(const CambGpuParams* p, int n, int lmax_out, double* unlensed, double* lensed,
                                       double* lens_potential, int* lmax_lensed, int nq_max, float* transfer, int* nq,
                                       double* sigma8, double* sigma2_vdelta_8, int* status) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n < 1) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "empty batch");
  if (lmax_out < 0 || lmax_out > 8000) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "lmax_out out of range");
  for (int c = 0; c < n; ++c) {
    if (!p[c].want_transfer || !p[c].want_cls)
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "this call needs want_cls = want_transfer = 1");
    if (p[c].num_transfer_redshifts != p[0].num_transfer_redshifts)
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "every cosmology of a transfer batch needs the same redshift count");
  }
  std::vector<Handle*> hs;
  int rc = build_handles(p, n, hs, status);
  struct Guard { std::vector<Handle*>& h; ~Guard() { for (auto* x : h) delete x; } } guard{hs};
  if (rc) return rc;
  for (auto* h : hs)
    if (transfer && h->tview.nk > nq_max) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "nq_max too small");
  // the CMB sources, stored by the transfer half's launch and read by the CMB half: outside
  // the arena, which the CMB half stages again
  std::vector<size_t> off(n + 1, 0);
  for (int c = 0; c < n; ++c)
    off[c + 1] = off[c] + (size_t)hs[c]->view.ntau * hs[c]->view.nsrc * hs[c]->view.nk;
  struct DevBuf { double* p = nullptr; ~DevBuf() { if (p) cudaFree(p); } } src;
  rc = rt_init();
  if (rc) return rc;
  CUDA_TRY(cudaMalloc(&src.p, off[n] * 8));
  CUDA_TRY(cudaMemsetAsync(src.p, 0, off[n] * 8, g_rt.stream));
  {
    // transfer half: the source modes evolved once, CMB sources at the source times and
    // transfer variables at the transfer times; the transfer grid's modes above them
    Batch B;
    for (auto* h : hs) add_handle(B, h, true);
    rc = stage_batch(B);
    if (rc) return rc;
    std::vector<DevCosmo> hc(n);
    for (int c = 0; c < n; ++c) {
      B.ups[c].d.src_out = src.p + off[c];
      B.ups[c].d.src_nk = hs[c]->view.nk;
      hc[c] = B.ups[c].d;
    }
    CUDA_TRY(cudaMemcpyAsync(B.d_cosmos, hc.data(), (size_t)n * sizeof(DevCosmo), cudaMemcpyHostToDevice, g_rt.stream));
    rc = run_all(B, true, false, false);
    if (rc) return rc;
    CUDA_TRY(launch_sigma8(B.d_cosmos, n, g_rt.stream));
    g_launches++;
    rc = check_status(B, status);
    if (rc) return rc;
    rc = fetch_transfers(B, hs, p[0].num_transfer_redshifts, nq_max, transfer, nq, sigma8, sigma2_vdelta_8);
    if (rc) return rc;
  }
  // CMB half: the sources copied in, then spline, projection, C_l, interpolation, lensing
  Batch B;
  for (auto* h : hs) add_handle(B, h);
  rc = stage_batch(B, lmax_out);
  if (rc) return rc;
  for (int c = 0; c < n; ++c)
    CUDA_TRY(cudaMemcpyAsync(B.ups[c].d.linear_src, src.p + off[c], (off[c + 1] - off[c]) * 8, cudaMemcpyDeviceToDevice,
                             g_rt.stream));
  rc = run_all(B, false, true, true);
  if (rc) return rc;
  rc = check_status(B, status);
  if (rc) return rc;
  if (lmax_lensed)
    for (int c = 0; c < n; ++c) lmax_lensed[c] = B.ups[c].d.lensed ? B.ups[c].d.lmax_lensed : 0;
  return fetch_spectra(B, lmax_out, unlensed, lensed, lens_potential);
}

int cambgpu_lensing_range(const CambGpuTables* t, int* out3) {
  HostLensGeom h;
  int rc = lens_geometry(*t, h);
  if (rc) return rc;
  out3[0] = h.lmax;
  out3[1] = h.lmax_lensed;
  out3[2] = h.npoints - 1;
  return 0;
}

int cambgpu_get_results(const CambGpuParams* p, int lmax_out, double* cl_out) {
  int st = 0;
  return cambgpu_get_results_batch(p, 1, lmax_out, cl_out, &st);
}

// ---- resident batch (bench path: inputs staged in HBM before timing) ----
// Any later staging (a one-shot call, a transfer batch) reuses the device arena, so the
// resident batch is only usable while it is the last one staged.
int resident_check() {
  if (!g_res) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "no resident batch");
  if (g_res->B.staged_epoch != g_rt.epoch)
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "the resident batch was replaced by a later staging");
  return 0;
}

int cambgpu_batch_prepare(const CambGpuParams* p, int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_res.reset(new Resident());
  int rc = build_handles(p, n, g_res->handles, nullptr);
  if (rc) return rc;
  for (auto* h : g_res->handles) add_handle(g_res->B, h);
  rc = stage_batch(g_res->B);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
  return 0;
}

// Puts host tables on grids shared by all of them (cg::build_shared_grid): the members'
// time steps, source k grid, integration q grid and Bessel table are made common, so that
// the projection of the whole batch at one q is one matrix product.  Host only.
static int share_grids(const std::vector<Handle*>& hs, cg::SharedGrid& sg) {
  if (hs.empty()) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "shared grids: empty batch");
  std::vector<const cg::Cosmology*> cs;
  const cg::Cosmology& c0 = hs[0]->c;
  for (auto* h : hs) {
    if (!h || !h->c.P.want_cls || (h->c.P.want_transfer && !h->c.P.want_cls) || h->c.ls != c0.ls ||
        h->c.nsrc != c0.nsrc || h->c.P.BesselBoost != c0.P.BesselBoost || h->c.P.AccuracyBoost != c0.P.AccuracyBoost)
      return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS,
                     "shared grids need CMB runs with one l sampling, one set of sources and one accuracy");
    cs.push_back(&h->c);
  }
  std::string err;
  int rc = cg::build_shared_grid(cs, sg, err);
  if (rc) return set_err(rc, err);
  if (sg.chi.size() > 4096) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "shared grid: more than 4096 time nodes");
  // the Bessel table covers every argument q chi of the shared grids: the members with
  // tau0 above the grid member's see q chi beyond their own q_max tau0
  double xmax = sg.q_int.back() * sg.chi.front() * 1.0001;
  for (auto* h : hs) xmax = std::max(xmax, h->c.maximum_qeta);
  std::shared_ptr<const cg::BesselTable> bt;
  try {
    bt = cg::get_bessel_table(c0.ls, xmax, c0.P.BesselBoost, c0.P.AccuracyBoost);
  } catch (const std::exception& e) {
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, e.what());
  }
  for (auto* h : hs) {
    cg::apply_shared_grid(h->c, sg);
    h->bt = bt;
    cg::fill_view(h->c, *bt, h->view);
  }
  return 0;
}

int cambgpu_tables_share_grids(void** handles, int n, int* nchi_out) {
  if (!handles || n < 1) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "share_grids: no handles");
  std::vector<Handle*> hs(n);
  for (int i = 0; i < n; ++i) hs[i] = static_cast<Handle*>(handles[i]);
  cg::SharedGrid sg;
  int rc = share_grids(hs, sg);
  if (rc) return rc;
  if (nchi_out) *nchi_out = (int)sg.chi.size();
  return 0;
}

int cambgpu_batch_prepare_shared(const CambGpuParams* p, int n, int* nchi_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_res.reset(new Resident());
  int rc = build_handles(p, n, g_res->handles, nullptr);
  if (rc) return rc;
  cg::SharedGrid sg;
  rc = share_grids(g_res->handles, sg);
  if (rc) return rc;
  for (auto* h : g_res->handles) add_handle(g_res->B, h);
  g_res->B.shared = true;
  g_res->B.h_chi = sg.chi;
  g_res->B.h_dchi = sg.dchi;
  rc = stage_batch(g_res->B);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(g_rt.stream));
  if (nchi_out) *nchi_out = (int)sg.chi.size();
  return 0;
}

int cambgpu_batch_run(double* ms3) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (int rc = resident_check()) return rc;
  int rc = run_all(g_res->B, true, true, true);
  if (rc) return rc;
  if (ms3) { ms3[0] = g_timings[0]; ms3[1] = g_timings[2]; ms3[2] = g_timings[3]; }
  return check_status(g_res->B, nullptr);
}

int cambgpu_batch_fetch(int lmax_out, double* cl_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (int rc = resident_check()) return rc;
  return fetch_spectra(g_res->B, lmax_out, cl_out, nullptr, nullptr);
}

int cambgpu_batch_spectra_from_transfer(const double* As, const double* ns, const double* nrun,
                                        const double* pivot_scalar, int lmax_out, double* unlensed, double* lensed,
                                        double* lens_potential, int* lmax_lensed) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (int rc = resident_check()) return rc;
  Batch& B = g_res->B;
  const int n = (int)B.views.size();
  if (As || ns || nrun || pivot_scalar) {
    std::vector<DevCosmo> hc(n);
    for (int c = 0; c < n; ++c) {
      DevCosmo& d = B.ups[c].d;
      if (As) d.As = As[c];
      if (ns) d.ns = ns[c];
      if (nrun) d.nrun = nrun[c];
      if (pivot_scalar) d.pivot_scalar = pivot_scalar[c];
      if (!(d.As > 0) || !(d.pivot_scalar > 0))
        return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "As and pivot_scalar must be positive");
      hc[c] = d;
    }
    CUDA_TRY(cudaMemcpyAsync(B.d_cosmos, hc.data(), (size_t)n * sizeof(DevCosmo), cudaMemcpyHostToDevice,
                             g_rt.stream));
  }
  // CalcScalCls, InterpolateCls and lens_Cls from the resident transfer functions
  int rc = run_all(B, false, false, true);
  if (rc) return rc;
  if (lmax_lensed)
    for (int c = 0; c < n; ++c) lmax_lensed[c] = B.ups[c].d.lensed ? B.ups[c].d.lmax_lensed : 0;
  return fetch_spectra(B, lmax_out, unlensed, lensed, lens_potential);
}

void cambgpu_batch_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_res.reset();
}

int cambgpu_set_precision(int mode) {
  if (mode < 0 || mode > 2) return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "precision mode must be 0, 1 or 2");
  std::lock_guard<std::mutex> lk(g_mu);
  g_precision = mode;
  return 0;
}

int cambgpu_get_precision(void) { return g_precision; }

int cambgpu_set_ode_team(int lanes) {
  if (lanes < 0 || (lanes > 8 && lanes != 16 && lanes != 32))
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "team code must be 0-8, 16 or 32");
  g_team = lanes;
  return 0;
}

int cambgpu_set_ode_schedule(int schedule) {
  if (schedule < -1 || schedule > 1)
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "schedule must be -1 (tuned), 0 (queue) or 1 (static stride)");
  g_sched = schedule;
  return 0;
}

int cambgpu_set_ode_launch(int queue_order, int blocks_per_sm) {
  if (queue_order < -1 || queue_order > 4 || blocks_per_sm < 0)
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "queue order must be -1..4 and blocks per SM >= 0");
  g_order = queue_order;
  g_blocks_cap = blocks_per_sm;
  return 0;
}

int cambgpu_last_timings(double* out6) {
  for (int i = 0; i < 6; ++i) out6[i] = g_timings[i];
  return 0;
}

long long cambgpu_last_ode_evals(void) { return g_last_evals; }

int cambgpu_autotune_ode(const CambGpuParams* p, int n, int* best, double* times) {
  // candidates: (team code, queue order, resident-block cap); team 32 = warp per mode with
  // registers (massless layout), 6 = warp per mode with shared-memory rows, 1/2/3 = thread
  // per mode compiled for 3/4/5 resident blocks per SM (cap 0: that many; 2: two, so that
  // threads finishing early take the queue's remaining modes), 7 = thread per mode compiled
  // for 2 resident blocks (more registers per thread, CMB sources only)
  // 4th column: schedule (0 = queue counter, 1 = static stride)
  static const int cand[][4] = {{32, 0, 0, 0}, {1, 0, 0, 0}, {1, 2, 0, 0}, {2, 2, 0, 0}, {1, 3, 2, 0},
                                {1, 2, 2, 0},  {2, 2, 2, 0}, {1, 1, 2, 0}, {6, 0, 0, 0}, {7, 2, 0, 0},
                                {7, 3, 0, 0},  {7, 2, 0, 1}, {7, 3, 0, 1}, {7, 4, 0, 1}, {1, 4, 0, 1},
                                {2, 4, 0, 1}};
  const int nc = (int)(sizeof(cand) / sizeof(cand[0]));
  int rc = cambgpu_batch_prepare(p, n);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_mu);
  Batch& B = g_res->B;
  int saved_team = g_team, saved_order = g_order, saved_cap = g_blocks_cap, saved_sched = g_sched;
  double best_ms = 1e30;
  int bi = 0;
  for (int c = 0; c < nc; ++c) {
    if (times) times[c] = 0;
    if ((B.massive_nu || B.transfer) && cand[c][0] >= 8) continue;  // massless-only warp kernel
    // the shared-memory warp kernel is the latency choice for few modes; on large batches
    // its redundant per-lane scalar work loses to thread per mode several times over
    if (cand[c][0] == 6 && (B.warp_stride > kWarpStrideMax || size_class(B) == 1)) continue;
    if (cand[c][0] == 7 && B.transfer) continue;  // compiled for CMB sources only
    g_team = cand[c][0];
    g_order = cand[c][1];
    g_blocks_cap = cand[c][2];
    g_sched = cand[c][3];
    rc = run_all(B, true, false, false);  // warm-up
    if (rc) break;
    rc = run_all(B, true, false, false);
    if (rc) break;
    if (times) times[c] = g_timings[0];
    if (g_timings[0] < best_ms) { best_ms = g_timings[0]; bi = c; }
  }
  g_team = saved_team;
  g_order = saved_order;
  g_blocks_cap = saved_cap;
  g_sched = saved_sched;
  if (rc) return rc;
  g_tuned[size_class(B)] = {cand[bi][0], cand[bi][1], cand[bi][2], cand[bi][3]};
  if (best) {
    best[0] = cand[bi][0];
    best[1] = cand[bi][1];
    best[2] = size_class(B);
    best[3] = cand[bi][2];
  }
  return 0;
}

int cambgpu_last_transfer_bytes(long long* out2) {
  out2[0] = g_h2d;
  out2[1] = g_d2h;
  return 0;
}

int cambgpu_probe_fp64_tflops(double* tflops) {
  std::lock_guard<std::mutex> lk(g_mu);
  int rc = rt_init();
  if (rc) return rc;
  double* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, 8));
  const int threads = 256, iters = 4096;
  const int blocks = g_rt.nsm * 8;
  CUDA_TRY(launch_fp64_probe(blocks, threads, 64, d, g_rt.stream));  // warm-up
  CUDA_TRY(cudaEventRecord(g_rt.ev[4], g_rt.stream));
  CUDA_TRY(launch_fp64_probe(blocks, threads, iters, d, g_rt.stream));
  CUDA_TRY(cudaEventRecord(g_rt.ev[5], g_rt.stream));
  CUDA_TRY(cudaEventSynchronize(g_rt.ev[5]));
  g_launches += 2;
  double ms = elapsed(g_rt.ev[4], g_rt.ev[5]);
  cudaFree(d);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return 0;
}

int cambgpu_probe_fp64_pipe(int warps_per_sm, int active_lanes, int chains, double* lane_fma_per_sm_cycle) {
  if (warps_per_sm < 1 || warps_per_sm > 32 || active_lanes < 1 || active_lanes > 32 ||
      (chains != 1 && chains != 4 && chains != 8) || !lane_fma_per_sm_cycle)
    return set_err(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "probe: warps 1-32, lanes 1-32, chains 1, 4 or 8");
  std::lock_guard<std::mutex> lk(g_mu);
  int rc = rt_init();
  if (rc) return rc;
  const int nsm = g_rt.nsm, iters = 4096;
  long long* d_cyc = nullptr;
  double* d_out = nullptr;
  CUDA_TRY(cudaMalloc(&d_cyc, sizeof(long long) * nsm));
  CUDA_TRY(cudaMalloc(&d_out, 8));
  cudaError_t e = launch_fp64_pipe_probe(nsm, warps_per_sm, active_lanes, chains, 64, d_cyc, d_out, g_rt.stream);
  if (e == cudaSuccess) e = launch_fp64_pipe_probe(nsm, warps_per_sm, active_lanes, chains, iters, d_cyc, d_out,
                                                   g_rt.stream);
  std::vector<long long> cyc(nsm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cyc.data(), d_cyc, sizeof(long long) * nsm, cudaMemcpyDeviceToHost,
                                            g_rt.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_rt.stream);
  cudaFree(d_cyc);
  cudaFree(d_out);
  if (e != cudaSuccess) return set_err(CAMBGPU_ERROR_CUDA, cudaGetErrorString(e));
  g_launches += 2;
  double mean = 0;
  for (long long c : cyc) mean += (double)c;
  mean /= nsm;
  *lane_fma_per_sm_cycle = (double)warps_per_sm * active_lanes * chains * iters / mean;
  return 0;
}

long long cambgpu_kernel_launches(int reset) {
  long long v = g_launches.load();
  if (reset) g_launches = 0;
  return v;
}

const char* cambgpu_last_error(void) { return g_err.c_str(); }

}  // extern "C"
