// Instantiates the warp-per-mode ODE kernels (see ode_device.cuh): shared-memory rows for
// any layout (team 6) and the register-resident massless kernels (teams 8, 16, 32).
#include "ode_device.cuh"

namespace cgdev {

int occ_warp(int team, int threads, int warp_stride) {
  int per_sm = 0;
  if (team == 6) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tpm::ode_warp_kernel<false>, 32,
                                                                tpm::warp_smem_bytes(warp_stride));
  else if (team == 32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ode_persistent_kernel<32>, threads, 0);
  else if (team == 16) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ode_persistent_kernel<16>, threads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ode_persistent_kernel<8>, threads, 0);
  return per_sm;
}

cudaError_t launch_warp(int team, bool transfer, int blocks, int threads, cudaStream_t s, const DevCosmo* cosmos,
                        const WorkItem* items, int nitems, int* counter, int warp_stride) {
  if (team == 6) {  // warp per mode (any layout), one warp per block
    const size_t smem = tpm::warp_smem_bytes(warp_stride);
    if (transfer) tpm::ode_warp_kernel<true><<<blocks, 32, smem, s>>>(cosmos, items, nitems, counter, warp_stride);
    else tpm::ode_warp_kernel<false><<<blocks, 32, smem, s>>>(cosmos, items, nitems, counter, warp_stride);
  } else if (transfer) {
    return cudaErrorInvalidValue;  // the register kernels evolve the massless CMB layout only
  } else if (team == 32) {
    ode_persistent_kernel<32><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  } else if (team == 16) {
    ode_persistent_kernel<16><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  } else {
    ode_persistent_kernel<8><<<blocks, threads, 0, s>>>(cosmos, items, nitems, counter);
  }
  return cudaGetLastError();
}

}  // namespace cgdev
