// Instantiates thread-per-mode ODE kernel variants (see ode_device.cuh); one translation
// unit per few variants so that the library compiles in parallel.
#include "ode_device.cuh"

namespace cgdev {

int occ_thread6(bool transfer, int threads) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tpm::ode_thread_kernel<6, false>, threads, 0);
  return per_sm;
}

cudaError_t launch_thread6(bool transfer, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                       const WorkItem* items, int nitems, int* counter) {
  // no shared memory: the whole of the SM's L1/shared array goes to L1, which caches the
  // stage rows held in local memory (a hint; a refusal leaves the default split)
  static const bool carve = [] {
    cudaFuncSetAttribute(tpm::ode_thread_kernel<6, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxL1);
    cudaGetLastError();
    return true;
  }();
  (void)carve;
  if (transfer) return cudaErrorInvalidValue;
  tpm::ode_thread_kernel<6, false><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  return cudaGetLastError();
}

int occ_thread8(bool transfer, int threads) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tpm::ode_thread_kernel<8, false>, threads, 0);
  return per_sm;
}

cudaError_t launch_thread8(bool transfer, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                       const WorkItem* items, int nitems, int* counter) {
  // no shared memory: the whole of the SM's L1/shared array goes to L1, which caches the
  // stage rows held in local memory (a hint; a refusal leaves the default split)
  static const bool carve = [] {
    cudaFuncSetAttribute(tpm::ode_thread_kernel<8, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxL1);
    cudaGetLastError();
    return true;
  }();
  (void)carve;
  if (transfer) return cudaErrorInvalidValue;
  tpm::ode_thread_kernel<8, false><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  return cudaGetLastError();
}

}  // namespace cgdev
