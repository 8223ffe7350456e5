// Allocation-free variant of the line-of-sight stage (source k-spline + flat LOS).
//
// For callers that cannot allocate device memory themselves or through this library:
// code running where cudaMalloc is unavailable or forbidden (inside a framework
// that owns all device memory through its own pool, a process with a fixed memory
// budget that must not grow after start-up, or a long-running service that keeps a
// strict no-allocation rule on its serving path).  Such a caller passes device
// pointers for every input and output; the only scratch the stage needs -- the
// k-spline second derivatives of the sources, the spline factors of the k grid and
// the device copy of the per-cosmology view -- lives in the file-scope array below.
//
// Limits and sharing rules:
//   - the scratch is kNoAllocScratchDoubles doubles (16 MiB); a problem whose
//     5*nk + ntau*nsrc*nk + view words exceed it, or whose time grid needs more than the
//     projection kernel's 160 KiB of dynamic shared memory (ntau*44 + 64 bytes, i.e.
//     ntau above 3722), is rejected with error code 2 and a message
//     (cambgpu_last_error) before any device call;
//   - every array in the tables and both buffers must be device (or managed) memory:
//     a host pointer is rejected with code 2 before anything is launched;
//   - every GPU that loads the library holds this array until the process exits;
//   - all calls share the array and it keeps the last call's contents, so calls that
//     overlap on the GPU (different streams, or host threads racing) corrupt each
//     other: serialise them;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and sets the kernel's shared-memory limit, under a lock,
//     so two host threads making their first calls together do it once; make that
//     first call before any stream capture;
//   - a call returns after the work it queued on `stream` has finished (it
//     synchronises that stream), so the caller's buffers are complete on return.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/cambgpu.h"
#include "device_tables.cuh"

namespace cgdev {
__global__ void source_spline_kernel(const DevCosmo*, const double* const*);
__global__ void los_flat_kernel(const DevCosmo*);
int set_last_error(int code, const char* msg);
}  // namespace cgdev

using namespace cgdev;

namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 21;  // 16 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mu;  // guards the one-time per-device set-up below
constexpr size_t kLosSmemMax = 160 * 1024;  // dynamic shared memory the projection kernel may use

// device (or managed) memory only: the kernels dereference every pointer of the view
bool on_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the (non-sticky) error left by an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// spline factors of the k grid (same quantities the host computes for the batched path)
__global__ void noalloc_spline_factors(const double* __restrict__ x, int n, double* __restrict__ spl) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double *inv_dx = spl, *sig = spl + n, *pinv = spl + 2 * n, *fac = spl + 3 * n, *c6 = spl + 4 * n;
  for (int i = 0; i < n - 1; ++i) inv_dx[i] = 1.0 / (x[i + 1] - x[i]);
  inv_dx[n - 1] = 0;
  sig[0] = pinv[0] = c6[0] = 0;
  fac[0] = 0;
  for (int i = 1; i < n - 1; ++i) {
    sig[i] = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig[i] * fac[i - 1] + 2.0;
    pinv[i] = 1.0 / p;
    fac[i] = (sig[i] - 1.0) / p;
    c6[i] = 6.0 / (x[i + 1] - x[i - 1]);
  }
  sig[n - 1] = pinv[n - 1] = fac[n - 1] = c6[n - 1] = 0;
}

}  // namespace

extern "C" int cambgpu_los_flat_noalloc(const CambGpuTables* t, const double* linear_src_dev, double* delta_dev,
                                        void* stream) {
  if (!t || !linear_src_dev || !delta_dev)
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "los_flat_noalloc: null tables or buffer");
  if (t->nk < 3 || t->ntau < 3 || t->nq < 1 || t->nl < 1 || t->nl > 512 || t->nsrc < 2 || t->nsrc > 3 ||
      t->num_xx < 2)
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "los_flat_noalloc: grid sizes out of range");
  // scratch layout: [view | spline-factor pointer | spline factors 5*nk | dd_src ntau*nsrc*nk];
  // the size check comes before any device call
  const size_t view_words = (sizeof(DevCosmo) + 255) / 256 * 32;
  const size_t ptr_words = 32;
  const size_t spl_words = ((size_t)5 * t->nk + 31) / 32 * 32;
  const size_t dd_words = (size_t)t->ntau * t->nsrc * t->nk;
  if (view_words + ptr_words + spl_words + dd_words > kNoAllocScratchDoubles) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "los_flat_noalloc: problem needs %zu doubles of scratch (5*nk + ntau*nsrc*nk with nk=%d, "
                  "ntau=%d, nsrc=%d), above the %zu of the static scratch array",
                  view_words + ptr_words + spl_words + dd_words, t->nk, t->ntau, t->nsrc, kNoAllocScratchDoubles);
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, msg);
  }
  // the projection stages the time grid in shared memory: sources x3, two weights, an index
  const size_t smem = (size_t)t->ntau * (3 + 1 + 1) * 8 + (size_t)t->ntau * 4 + 64;
  if (smem > kLosSmemMax) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "los_flat_noalloc: ntau=%d needs %zu bytes of shared memory (ntau*44 + 64), above the %zu "
                  "the projection kernel is set up for",
                  t->ntau, smem, kLosSmemMax);
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, msg);
  }
  if (!t->q_evolve || !t->tau_points || !t->tau_dpoints || !t->q_int || !t->ls || !t->bess_x || !t->bessel_horner)
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "los_flat_noalloc: null array in the tables");
  {
    const void* ptrs[] = {linear_src_dev, delta_dev, t->q_evolve, t->tau_points, t->tau_dpoints, t->q_int,
                          t->ls, t->bess_x, t->bessel_horner};
    const char* names[] = {"linear_src_dev", "delta_dev", "q_evolve", "tau_points", "tau_dpoints", "q_int",
                           "ls", "bess_x", "bessel_horner"};
    for (int i = 0; i < 9; ++i)
      if (!on_device(ptrs[i])) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "los_flat_noalloc: %s is not device memory", names[i]);
        return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, msg);
      }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: no current CUDA device");
  std::unique_lock<std::mutex> setup_lock(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    // one-time set-up on this device (call before any stream capture)
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
      return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: cudaGetSymbolAddress of the scratch failed");
    if (cudaFuncSetAttribute(los_flat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLosSmemMax) !=
        cudaSuccess)
      return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: cudaFuncSetAttribute failed");
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  double* base = g_scratch_addr[dev];
  setup_lock.unlock();
  DevCosmo* d_view = reinterpret_cast<DevCosmo*>(base);
  const double** d_splp = reinterpret_cast<const double**>(base + view_words);
  double* d_spl = base + view_words + ptr_words;
  double* d_dd = d_spl + spl_words;

  DevCosmo h;
  std::memset(&h, 0, sizeof(h));
  h.tau0 = t->tau0;
  h.tau_points = t->tau_points;
  h.tau_dpoints = t->tau_dpoints;
  h.ntau = t->ntau;
  h.q_evolve = t->q_evolve;
  h.nk = t->nk;
  h.linear_src = const_cast<double*>(linear_src_dev);
  h.dd_src = d_dd;
  h.delta = delta_dev;
  h.q_int = t->q_int;
  h.nq = t->nq;
  h.ls = t->ls;
  h.nl = t->nl;
  h.bess_x = t->bess_x;
  h.bessel_horner = t->bessel_horner;
  h.num_xx = t->num_xx;
  h.nsrc = t->nsrc;
  h.want_late_time = t->want_late_time;
  h.max_etak_scalar = t->max_etak_scalar;
  h.AccuracyBoost = t->AccuracyBoost;
  h.BessIntBoost = t->BessIntBoost;
  h.LimberBoost = t->LimberBoost;
  // the view and the factor pointer are small pageable copies on the caller's stream;
  // the stream is synchronised before returning so the host structs can go out of scope
  if (cudaMemcpyAsync(d_view, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: copy of the view failed");
  const double* spl_ptr = d_spl;
  if (cudaMemcpyAsync(d_splp, &spl_ptr, sizeof(spl_ptr), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: copy of the spline-factor pointer failed");
  noalloc_spline_factors<<<1, 1, 0, s>>>(t->q_evolve, t->nk, d_spl);
  const int rows = t->ntau * t->nsrc;
  source_spline_kernel<<<dim3((rows + 127) / 128, 1), 128, 0, s>>>(d_view, d_splp);
  // the projection leaves l above the last integrated multipole untouched: clear the output
  if (cudaMemsetAsync(delta_dev, 0, (size_t)t->nq * t->nl * t->nsrc * sizeof(double), s) != cudaSuccess)
    return set_last_error(CAMBGPU_ERROR_CUDA, "los_flat_noalloc: clearing the output failed");
  los_flat_kernel<<<dim3(t->nq, 1), 256, smem, s>>>(d_view);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_last_error(CAMBGPU_ERROR_CUDA, cudaGetErrorString(e));
  return CAMBGPU_OK;
}
