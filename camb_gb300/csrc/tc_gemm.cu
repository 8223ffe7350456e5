// Split hi/lo BF16 matrix product on the fifth-generation tensor cores:
//   D[m][n] = sum_k A[m][k] B[n][k]   (FP32 in, FP32 out)
// with A = A_hi + A_lo and B = B_hi + B_lo split into BF16 pairs and D accumulated in FP32
// in tensor memory as A_hi B_hi + A_hi B_lo + A_lo B_hi (the A_lo B_lo term is below the
// FP32 accumulation's resolution).  One CTA of four warps computes a 128 x 128 tile: the
// 128 threads split and stage 64-deep K tiles of both operands in shared memory, one
// thread issues the twelve tcgen05.mma of each tile (4 K slices x 3 products) and commits
// them to an mbarrier, every wait is bounded, and the four warps read the accumulator
// back from their tensor-memory lane quarters.  This is the primitive of the shared-grid
// line-of-sight projection; cambgpu_gemm_bf16x3 exposes it for testing.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/cambgpu.h"
#include "tc_gemm.cuh"

namespace cgdev {
int set_last_error(int code, const char* msg);

namespace tc {

constexpr long long kWaitLimit = 1LL << 26;  // try_wait polls before a wait gives up
constexpr int kTileBytes = 128 * kChunk * 2;   // 128 rows x 64 K values in BF16
constexpr size_t kGemmSmem = 4 * (size_t)kTileBytes + 2048;

__global__ void __launch_bounds__(128, 1) gemm_bf16x3_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                             float* __restrict__ D, int M, int N, int K,
                                                             int* __restrict__ err) {
  extern __shared__ unsigned char tc_smem_raw[];
  // 1024-byte aligned tiles: A_hi, A_lo, B_hi, B_lo, then the mbarrier and the TMEM slot
  unsigned char* base =
      tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
  unsigned char* a_hi = base;
  unsigned char* a_lo = base + kTileBytes;
  unsigned char* b_hi = base + 2 * kTileBytes;
  unsigned char* b_lo = base + 3 * kTileBytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + 4 * kTileBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(base + 4 * kTileBytes + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
  if (tid == 0) mbar_init(bar, 1);
  if (warp == 0) tmem_alloc(tslot, 128);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = *tslot;
  constexpr uint32_t idesc = idesc_bf16_f32(128, 128);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kChunk) {
    for (int idx = tid; idx < 128 * kChunk; idx += 128) {
      const int r = idx / kChunk, k = idx % kChunk;
      const bool kin = k0 + k < K;
      const float a = (kin && m0 + r < M) ? A[(size_t)(m0 + r) * K + k0 + k] : 0.0f;
      const float b = (kin && n0 + r < N) ? B[(size_t)(n0 + r) * K + k0 + k] : 0.0f;
      __nv_bfloat16 h, l;
      const uint32_t off = tile_offset(r, k);
      split_bf16(a, h, l);
      *reinterpret_cast<__nv_bfloat16*>(a_hi + off) = h;
      *reinterpret_cast<__nv_bfloat16*>(a_lo + off) = l;
      split_bf16(b, h, l);
      *reinterpret_cast<__nv_bfloat16*>(b_hi + off) = h;
      *reinterpret_cast<__nv_bfloat16*>(b_lo + off) = l;
    }
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int s = 0; s < kChunk / 16; ++s) {
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const unsigned char* a = p == 2 ? a_lo : a_hi;
          const unsigned char* b = p == 1 ? b_lo : b_hi;
          const uint64_t ad = smem_desc(smem_u32(a) + s * 256, 128, 1024);
          const uint64_t bd = smem_desc(smem_u32(b) + s * 256, 128, 1024);
          mma_bf16(tbase, ad, bd, idesc, (k0 > 0 || s > 0 || p > 0) ? 1u : 0u);
        }
      }
      mma_commit(bar);
    }
    // the tiles are rewritten only after the tensor core has read them
    const bool done = mbar_wait(bar, phase, kWaitLimit);
    phase ^= 1;
    ok = __syncthreads_and(done) != 0;
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    mbar_wait(bar, phase ^ 1, kWaitLimit);  // once more for the MMAs still in flight
  } else {
    fence_after_sync();
    const int m = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < 128; c0 += 32) {
      float v[32];
      tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (m < M) {
#pragma unroll
        for (int i = 0; i < 32; ++i)
          if (n0 + c0 + i < N) D[(size_t)m * N + n0 + c0 + i] = v[i];
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 128);
}

}  // namespace tc
}  // namespace cgdev

using namespace cgdev;

extern "C" int cambgpu_gemm_bf16x3(const float* A, const float* B, int M, int N, int K, float* D) {
  if (!A || !B || !D || M < 1 || N < 1 || K < 1 || M > 65536 || N > 65536 || K > 65536)
    return set_last_error(CAMBGPU_ERROR_UNSUPPORTED_PARAMS, "gemm_bf16x3: sizes 1-65536 and non-null buffers");
  static const bool attr = [] {
    cudaFuncSetAttribute(tc::gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kGemmSmem);
    cudaGetLastError();
    return true;
  }();
  (void)attr;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* derr = nullptr;
  const size_t sa = (size_t)M * K * 4, sb = (size_t)N * K * 4, sd = (size_t)M * N * 4;
  cudaError_t e = cudaMalloc(&dA, sa);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sb);
  if (e == cudaSuccess) e = cudaMalloc(&dD, sd);
  if (e == cudaSuccess) e = cudaMalloc(&derr, 4);
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, sa, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, 4);
  int herr = 0;
  if (e == cudaSuccess) {
    dim3 grid((N + 127) / 128, (M + 127) / 128);
    tc::gemm_bf16x3_kernel<<<grid, 128, tc::kGemmSmem>>>(dA, dB, dD, M, N, K, derr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(D, dD, sd, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(derr);
  if (e != cudaSuccess) return set_last_error(CAMBGPU_ERROR_CUDA, cudaGetErrorString(e));
  if (herr) return set_last_error(CAMBGPU_ERROR_CUDA, "gemm_bf16x3: a tensor-core completion wait ran out");
  return CAMBGPU_OK;
}
