// Instantiates the thread-per-mode ODE kernel compiled for 2 resident blocks of 128 per SM
// (see ode_device.cuh).  The batched workload runs best at two resident blocks per SM
// (the stage rows of more resident modes overflow L2); compiled for that occupancy the
// kernel may use up to 255 registers per thread instead of 168, which leaves the compiler
// room to keep more loads in flight.  CMB sources only: transfer-function runs use the
// 4-block variant.
#include "ode_device.cuh"

namespace cgdev {

int occ_thread2(bool transfer, int threads) {
  int per_sm = 0;
  if (transfer) return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tpm::ode_thread_kernel<2, false>, threads, 0);
  return per_sm;
}

cudaError_t launch_thread2(bool transfer, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                           const WorkItem* items, int nitems, int* counter) {
  // no shared memory: the whole of the SM's L1/shared array goes to L1, which caches the
  // stage rows held in local memory (a hint; a refusal leaves the default split)
  static const bool carve = [] {
    cudaFuncSetAttribute(tpm::ode_thread_kernel<2, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxL1);
    cudaGetLastError();
    return true;
  }();
  (void)carve;
  if (transfer) return cudaErrorInvalidValue;
  tpm::ode_thread_kernel<2, false><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  return cudaGetLastError();
}

}  // namespace cgdev
