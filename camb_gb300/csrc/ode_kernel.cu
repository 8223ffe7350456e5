// ODE kernel dispatch (team code -> compiled variant) and the FP64 throughput probe.  The
// variants are instantiated in ode_thread_*.cu and ode_warp.cu from ode_device.cuh.
#include <cuda_runtime.h>

#include "device_tables.cuh"

namespace cgdev {

int occ_thread2(bool transfer, int threads);
int occ_thread3(bool transfer, int threads);
int occ_thread4(bool transfer, int threads);
int occ_thread5(bool transfer, int threads);
int occ_thread6(bool transfer, int threads);
int occ_thread8(bool transfer, int threads);
int occ_warp(int team, int threads, int warp_stride);
cudaError_t launch_thread2(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_thread3(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_thread4(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_thread5(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_thread6(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_thread8(bool, int, int, cudaStream_t, const DevCosmo*, const WorkItem*, int, int*);
cudaError_t launch_warp(int team, bool transfer, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                        const WorkItem* items, int nitems, int* counter, int warp_stride);

// DFMA throughput probe: 8 independent FMA chains per thread
__global__ void fp64_probe_kernel(double* out, int iters) {
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = 1.0 + 1e-7 * (threadIdx.x + j);
  const double m = 0.999999, c = 1e-9;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fma(a[j], m, c);
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 12345.0) out[0] = s;  // keeps the chains live
}

cudaError_t launch_fp64_probe(int blocks, int threads, int iters, double* out, cudaStream_t s) {
  fp64_probe_kernel<<<blocks, threads, 0, s>>>(out, iters);
  return cudaGetLastError();
}

// FP64 issue model: one block per SM (held there by its dynamic shared memory), `lanes`
// active lanes in each of its warps, NC independent DFMA chains per lane.  Each block
// records the SM cycles (clock64) of its timed loop.
template <int NC>
__global__ void fp64_pipe_probe_kernel(long long* cyc, double* out, int iters, int lanes) {
  double a[NC];
#pragma unroll
  for (int j = 0; j < NC; ++j) a[j] = 1.0 + 1e-7 * (threadIdx.x + j);
  const double m = 0.999999, c = 1e-9;
  __syncthreads();
  const long long t0 = clock64();
  if ((int)(threadIdx.x & 31) < lanes) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int j = 0; j < NC; ++j) a[j] = fma(a[j], m, c);
    }
  }
  __syncthreads();
  const long long t1 = clock64();
  double s = 0;
#pragma unroll
  for (int j = 0; j < NC; ++j) s += a[j];
  if (s == 12345.0) out[0] = s;  // keeps the chains live
  if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

cudaError_t launch_fp64_pipe_probe(int nsm, int warps, int lanes, int chains, int iters, long long* cyc, double* out,
                                   cudaStream_t s) {
  const int smem = 150 * 1024;  // more than half an SM's shared memory: one block per SM
  const int threads = 32 * warps;
  cudaError_t e = cudaSuccess;
  if (chains == 1) {
    e = cudaFuncSetAttribute(fp64_pipe_probe_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) fp64_pipe_probe_kernel<1><<<nsm, threads, smem, s>>>(cyc, out, iters, lanes);
  } else if (chains == 4) {
    e = cudaFuncSetAttribute(fp64_pipe_probe_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) fp64_pipe_probe_kernel<4><<<nsm, threads, smem, s>>>(cyc, out, iters, lanes);
  } else {
    e = cudaFuncSetAttribute(fp64_pipe_probe_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) fp64_pipe_probe_kernel<8><<<nsm, threads, smem, s>>>(cyc, out, iters, lanes);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

// team 1..5 = thread per mode compiled for 3/4/5/6/8 resident blocks of 128 per SM, 7 =
// the same for 2 blocks; 6 = warp per mode with shared-memory rows; 8/16/32 =
// register-resident warp teams
int ode_blocks_per_sm(int team, int threads, int warp_stride) {
  switch (team) {
    case 1: return occ_thread3(false, threads);
    case 2: return occ_thread4(false, threads);
    case 3: return occ_thread5(false, threads);
    case 4: return occ_thread6(false, threads);
    case 5: return occ_thread8(false, threads);
    case 7: return occ_thread2(false, threads);
    default: return occ_warp(team, threads, warp_stride);
  }
}

cudaError_t launch_ode_kernel(int team, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                              const WorkItem* items, int nitems, int* counter, bool transfer, int warp_stride) {
  // transfer functions are compiled for 3/4/5 resident blocks only: other thread teams use 4
  if (transfer && team != 1 && team != 3 && (team <= 5 || team == 7)) team = 2;
  switch (team) {
    case 1: return launch_thread3(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    case 2: return launch_thread4(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    case 3: return launch_thread5(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    case 4: return launch_thread6(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    case 5: return launch_thread8(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    case 7: return launch_thread2(transfer, blocks, threads, s, cosmos, items, nitems, counter);
    default: return launch_warp(team, transfer, blocks, threads, s, cosmos, items, nitems, counter, warp_stride);
  }
}

}  // namespace cgdev
