// Flat line-of-sight projection of a batch on shared grids as split hi/lo BF16 products on
// the fifth-generation tensor cores (DoFlatIntegration, cmbmain.f90:1639-1862, restated as
// a matrix product).
//
// With one comoving-distance grid chi_n for every cosmology of the batch (tau_n = tau0_c -
// chi_n) and one integration q grid, the projection of source s at wavenumber q is
//     Delta_s[l][c] = sum_n J_q[l][n] S_q,s[n][c],   J_q[l][n] = j_l(q chi_n) dchi_n,
// one Bessel matrix per q for the whole batch.  One CTA of eight warps computes a 128
// (sampled l) x 128 (cosmologies) tile of one (q, source), l tiles and cosmology tiles
// along the grid's x: it stages 64-deep K tiles of J (from the FP32 Horner
// table, zero outside each l's integration window) and of S (the source k-spline of each
// cosmology evaluated at q, zero outside the cosmology's time range and its q*tau < max_etak
// prefix), split into BF16 pairs, in shared memory; one thread issues the twelve
// tcgen05.mma per tile into an FP32 accumulator in tensor memory; the epilogue applies the
// per-cosmology cuts of the FP64 kernel (l above q tau0, the lensed-run integration test),
// the Limber value of the lensing source, and writes Delta_p_l_k in FP64.
#include <cuda_runtime.h>

#include "device_tables.cuh"
#include "tc_gemm.cuh"

namespace cgdev {
namespace tc {

constexpr int kProjMaxChi = 4096;  // shared chi nodes staged per CTA
constexpr int kTileBytesP = 128 * kChunk * 2;
constexpr size_t kProjSmem = 4 * (size_t)kTileBytesP + (size_t)kProjMaxChi * 8 + 2048;

__device__ __forceinline__ int bsearch_lo_d(const double* x, int n, double v) {
  int lo = 0, hi = n - 1;  // largest i with x[i] <= v, for x increasing
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (x[m] <= v) lo = m;
    else hi = m;
  }
  return lo;
}

// number of shared nodes with chi_n >= v (chi decreasing)
__device__ __forceinline__ int count_ge(const double* chi, int n, double v) {
  int lo = 0, hi = n;  // chi[0..lo) >= v, chi[hi..n) < v
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (chi[m] >= v) lo = m + 1;
    else hi = m;
  }
  return lo;
}

// the k-spline weights of q on the shared source k grid (InterpolateSources)
struct KW {
  int klo, khi;
  double a0, b0, a03, b03, ho2o6;
};

// The batch's sources and their k-spline second derivatives as FP32 pairs, laid out
// [k][source][shared node][cosmology] so that the 128 cosmologies of a tile read one
// contiguous kilobyte per (k, source, node); zero where a cosmology has no row.
__global__ void proj_src_transpose_kernel(const DevCosmo* __restrict__ cosmos, int ncos, int nchi, int nk, int nsrc,
                                          float2* __restrict__ T) {
  __shared__ float2 tile[32][33];
  const int n = blockIdx.z / nsrc, s = blockIdx.z % nsrc;
  const int k0 = blockIdx.x * 32, c0 = blockIdx.y * 32, tx = threadIdx.x, ty = threadIdx.y;
  for (int cy = ty; cy < 32; cy += 8) {  // read 32 consecutive k of one cosmology
    const int c = c0 + cy, k = k0 + tx;
    float2 v = make_float2(0.0f, 0.0f);
    if (c < ncos && k < nk) {
      const DevCosmo& C = cosmos[c];
      const int i = n - (nchi - C.ntau);
      if (i >= 0 && i < C.ntau) {
        const size_t idx = ((size_t)i * nsrc + s) * nk + k;
        v = make_float2((float)C.linear_src[idx], (float)C.dd_src[idx]);
      }
    }
    tile[cy][tx] = v;
  }
  __syncthreads();
  for (int ky = ty; ky < 32; ky += 8) {  // write 32 consecutive cosmologies of one k
    const int k = k0 + ky, c = c0 + tx;
    if (k < nk && c < ncos) T[(((size_t)k * nsrc + s) * nchi + n) * ncos + c] = tile[tx][ky];
  }
}

// FP32 spline weights of q (the operand is split into BF16 pairs afterwards)
struct KWf {
  int klo, khi;
  float a0, b0, a03h, b03h;  // a03, b03 times ho^2/6
};
// source s of cosmology c at shared node n, from the transposed pairs
__device__ __forceinline__ float src_t(const float2* __restrict__ T, int ncos, int nchi, int nsrc, const KWf& K, int s,
                                       int n, int c) {
  const float2 p0 = __ldg(T + (((size_t)K.klo * nsrc + s) * nchi + n) * ncos + c);
  const float2 p1 = __ldg(T + (((size_t)K.khi * nsrc + s) * nchi + n) * ncos + c);
  return fmaf(K.a0, p0.x, fmaf(K.b0, p1.x, fmaf(K.a03h, p0.y, K.b03h * p1.y)));
}

// row i of cosmology C holds a source at q: 1 <= i and the prefix test of source_row_count
__device__ __forceinline__ bool row_valid(const DevCosmo& C, double q, int i) {
  if (i < 1 || i >= C.ntau) return false;
  const double tau = C.tau_points[i];
  const bool etak_ok = C.want_late_time || q * tau < C.max_etak_scalar;
  return etak_ok && q * (C.tau0 - tau) > 1e-8;
}

// end of the valid rows [1, end): the prefix test holds on an initial run of rows
__device__ __forceinline__ int valid_row_end(const DevCosmo& C, double q) {
  int lo = 1, hi = C.ntau;  // rows below lo pass; the first failing row is in [lo, hi]
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (row_valid(C, q, m)) lo = m + 1;
    else hi = m;
  }
  return lo;
}

__global__ void __launch_bounds__(256, 1)
    proj_tc_kernel(const DevCosmo* __restrict__ cosmos, int ncosmo, const double* __restrict__ chi,
                   const float* __restrict__ dchi_f, int nchi, const float2* __restrict__ T, int* __restrict__ err) {
  extern __shared__ unsigned char tp_smem_raw[];
  unsigned char* base = tp_smem_raw + ((1024 - (smem_u32(tp_smem_raw) & 1023)) & 1023);
  unsigned char* a_hi = base;
  unsigned char* a_lo = base + kTileBytesP;
  unsigned char* b_hi = base + 2 * kTileBytesP;
  unsigned char* b_lo = base + 3 * kTileBytesP;
  int* s_bix = reinterpret_cast<int*>(base + 4 * kTileBytesP);             // [nchi]
  float* s_a2 = reinterpret_cast<float*>(s_bix + kProjMaxChi);            // [nchi]
  uint64_t* bar = reinterpret_cast<uint64_t*>(s_a2 + kProjMaxChi);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  __shared__ int s_kbeg, s_kend;
  // per cosmology of the tile: first shared node, l cut, the node of its second row
  // (window test), lensed integration test for l <= 850, tau0
  __shared__ int s_off[128], s_llmax[128];
  __shared__ int s_nlo[128], s_nhi[128];  // integration window of each sampled l, in shared nodes
  __shared__ double s_chi1[128], s_tau0[128];
  __shared__ unsigned char s_doint850[128];
  // 256 threads: warps 0-3 stage the J rows (sampled l; warp w rows 32 w .. 32 w + 31, the
  // lanes along the nodes, so that a warp's table gathers fall on one row), threads
  // 128-255 the S rows (cosmologies; one thread per cosmology) of each tile; all eight
  // warps read the accumulator back, warp w from tensor-memory lane quarter w % 4 and
  // column half w / 4
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = tid & 127, side = tid >> 7;
  // blockIdx.x = (tile of 128 sampled l) x (tile of 128 cosmologies)
  const int ctiles = (ncosmo + 127) / 128;
  const int ctile = blockIdx.x % ctiles, l0 = (blockIdx.x / ctiles) * 128;
  const int src = blockIdx.y, q_ix = blockIdx.z;
  const DevCosmo& G = cosmos[0];  // shared grids: q, k, l sampling, Bessel table
  const double q = G.q_int[q_ix];
  const int nl = G.nl, nbx = G.num_xx, nsrc = G.nsrc;
  if (tid == 0) {
    mbar_init(bar, 1);
    s_kbeg = nchi;
    s_kend = 0;
  }
  if (warp == 0) tmem_alloc(tslot, 128);
  __syncthreads();  // s_kbeg / s_kend initialised before the atomics below
  // Bessel-table interval and Horner variable of every shared node at this q
  for (int n = tid; n < nchi; n += 256) {
    const double xx = fabs(q * chi[n]);
    const int bi = min(bsearch_lo_d(G.bess_x, nbx, xx), nbx - 2);
    const double xh = G.bess_x[bi + 1], dx = xh - G.bess_x[bi];
    s_bix[n] = bi;
    s_a2[n] = (float)((xh - xx) / dx);
  }
  // integration window of each sampled l in shared nodes (window_setup in chi): the last
  // node with chi >= 80 l BessIntBoost / q through the last node with chi >= xlim / q
  const double bib = G.AccuracyBoost * G.BessIntBoost;
  int nlo = nchi, nhi = -1;
  if (side == 0 && l0 + row < nl) {
    const int l = G.ls[l0 + row];
    const double xlim = fmax(0.0, l - 4.2 * cbrt((double)l));
    nlo = count_ge(chi, nchi, 80.0 * l * bib / q) - 1;
    nhi = count_ge(chi, nchi, xlim / q) - 1;
    if (nlo < 0) nlo = 0;
    atomicMin(&s_kbeg, nlo);
    atomicMax(&s_kend, nhi);
  }
  if (side == 0) {  // rows past the sampled l keep an empty window
    s_nlo[row] = nlo;
    s_nhi[row] = nhi;
  }
  // the k-spline weights of q on the shared source k grid
  KW K;
  {
    const int nk = G.nk;
    if (q <= G.q_evolve[0]) K.klo = 0;
    else if (q >= G.q_evolve[nk - 1]) K.klo = nk - 2;
    else K.klo = bsearch_lo_d(G.q_evolve, nk, q);
    K.khi = K.klo + 1;
    const double ho = G.q_evolve[K.khi] - G.q_evolve[K.klo];
    K.a0 = (G.q_evolve[K.khi] - q) / ho;
    K.b0 = (q - G.q_evolve[K.klo]) / ho;
    K.ho2o6 = ho * ho / 6.0;
    K.a03 = K.a0 * K.a0 * K.a0 - K.a0;
    K.b03 = K.b0 * K.b0 * K.b0 - K.b0;
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = *tslot;
  const int c = ctile * 128 + row;  // the cosmology column of an S-side thread
  const bool has_c = side == 1 && c < ncosmo;
  const DevCosmo* Cc = has_c ? &cosmos[c] : nullptr;
  const int c_off = has_c ? nchi - Cc->ntau : 0;  // shared node of the cosmology's row 0
  const int c_rend = has_c ? valid_row_end(*Cc, q) : 0;
  KWf Kf;
  Kf.klo = K.klo;
  Kf.khi = K.khi;
  Kf.a0 = (float)K.a0;
  Kf.b0 = (float)K.b0;
  Kf.a03h = (float)(K.a03 * K.ho2o6);
  Kf.b03h = (float)(K.b03 * K.ho2o6);
  if (has_c) {
    const double tau0 = Cc->tau0;
    int llmax = (int)llrint(q * tau0);
    if (llmax < 15) llmax = 17;
    else llmax = (int)llrint(q * (tau0 + 6 * 3.14159265358979323846 / q));
    s_off[row] = c_off;
    s_llmax[row] = llmax;
    s_chi1[row] = c_off + 1 < nchi ? chi[c_off + 1] : -1.0;
    s_tau0[row] = tau0;
    s_doint850[row] = q < 850 * 3 * (G.AccuracyBoost * G.BessIntBoost) / tau0 * 1.2;
  }
  __syncthreads();  // the per-cosmology arrays, read by the epilogue's threads
  constexpr uint32_t idesc = idesc_bf16_f32(128, 128);
  const int kbeg = (s_kbeg / kChunk) * kChunk, kend = s_kend;
  uint32_t phase = 0;
  bool ok = true, any = false;
  for (int k0 = kbeg; k0 <= kend && ok; k0 += kChunk) {
    if (side == 0) {
      // J: warp w fills rows 32 w .. 32 w + 31, each lane two nodes (k = lane, lane + 32);
      // the nodes' table intervals, Horner variables and weights are the same for every row
      int nn[2], bix[2];
      float a2[2], dc[2];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        nn[hh] = k0 + 32 * hh + lane;
        const bool in = nn[hh] < nchi;
        bix[hh] = in ? s_bix[nn[hh]] : 0;
        a2[hh] = in ? s_a2[nn[hh]] : 0.0f;
        dc[hh] = in ? dchi_f[nn[hh]] : 0.0f;
      }
#pragma unroll 4
      for (int r = 0; r < 32; ++r) {
        const int jrow = (warp & 3) * 32 + r;
        const int lo = s_nlo[jrow], hi = s_nhi[jrow];
        const float4* __restrict__ H = G.bessel_f32 + (size_t)min(l0 + jrow, nl - 1) * (nbx - 1);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          float v = 0.0f;
          if (nn[hh] < nchi && nn[hh] >= lo && nn[hh] <= hi) {
            const float4 h = __ldg(H + bix[hh]);
            v = (h.x + a2[hh] * (h.y + a2[hh] * (h.z + a2[hh] * h.w))) * dc[hh];
          }
          __nv_bfloat16 vh, vl;
          const uint32_t off = tile_offset(jrow, 32 * hh + lane);
          split_bf16(v, vh, vl);
          *reinterpret_cast<__nv_bfloat16*>(a_hi + off) = vh;
          *reinterpret_cast<__nv_bfloat16*>(a_lo + off) = vl;
        }
      }
    } else {
      // S: row = cosmology, 64 nodes
#pragma unroll 8
      for (int k = 0; k < kChunk; ++k) {
        const int n = k0 + k;
        float v = 0.0f;
        if (has_c && n < nchi) {
          const int i = n - c_off;
          if (i >= 1 && i < c_rend) v = src_t(T, ncosmo, nchi, nsrc, Kf, src, n, c);
        }
        __nv_bfloat16 vh, vl;
        const uint32_t off = tile_offset(row, k);
        split_bf16(v, vh, vl);
        *reinterpret_cast<__nv_bfloat16*>(b_hi + off) = vh;
        *reinterpret_cast<__nv_bfloat16*>(b_lo + off) = vl;
      }
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
          mma_bf16(tbase, smem_desc(smem_u32(a) + s * 256, 128, 1024), smem_desc(smem_u32(b) + s * 256, 128, 1024),
                   idesc, (any || s > 0 || p > 0) ? 1u : 0u);
        }
      }
      mma_commit(bar);
    }
    any = true;
    const bool done = mbar_wait(bar, phase, 1LL << 26);
    phase ^= 1;
    ok = __syncthreads_and(done) != 0;
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    mbar_wait(bar, phase ^ 1, 1LL << 26);
  } else {
    fence_after_sync();
    // epilogue: thread (warp w, lane) holds sampled l j = l0 + 32 (w % 4) + lane for the 64
    // cosmology columns of half w / 4, 32 at a time
    const int j = l0 + (warp & 3) * 32 + lane;
    const bool has_j = j < nl;
    const int l = has_j ? G.ls[j] : 0;
    const double limber_l = 400 * sqrt(G.AccuracyBoost * G.LimberBoost);
    const double xlim = has_j ? fmax(0.0, l - 4.2 * cbrt((double)l)) : 0.0;
    // Limber node pair of the lensing source in shared nodes (cmbmain.f90:1821-1832)
    const double chif = (l + 0.5) / q;
    const int mlim = count_ge(chi, nchi, chif);  // nodes with chi >= chif
#pragma unroll 1
    for (int c0 = (warp >> 2) * 64; c0 < (warp >> 2) * 64 + 64; c0 += 32) {
      float v[32];
      if (any) tmem_ld32(tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0, v);
      else
        for (int i = 0; i < 32; ++i) v[i] = 0.0f;
      if (!has_j) continue;
      const double xq = xlim / q;
      for (int i = 0; i < 32; ++i) {
        const int ct = c0 + i, cc = ctile * 128 + ct;
        if (cc >= ncosmo) break;
        const DevCosmo& C = cosmos[cc];
        const int off = s_off[ct];
        const double tau0 = s_tau0[ct];
        double out = v[i];
        // F_SKIP: above the cut, or the window ends before the cosmology's first source row
        const bool skip = l > s_llmax[ct] || (s_chi1[ct] >= 0.0 && xq > s_chi1[ct]);
        if (skip) out = 0.0;
        else if (C.nsrc > 2) {
          const bool doint = l <= 850 ? s_doint850[ct] != 0 : q < max(850, l) * 3 * bib / tau0 * 1.2;
          if (!doint && src < 2) out = 0.0;
          if (src == 2 && (!doint || l > limber_l)) {
            double limb = 0.0;
            // xf = tau0 - (l + 1/2)/q inside (tp[0], tp[ntau-1]): chif below chi[off], above 0
            if (chif > 0 && chif < chi[off] && mlim >= 1 && mlim < nchi) {
              const int ia = mlim - 1 - off, ib = mlim - off;  // rows n - 1 and n of the cosmology
              const double f = (chi[mlim - 1] - chif) / (chi[mlim - 1] - chi[mlim]);
              const double slo = row_valid(C, q, ia) ? (double)src_t(T, ncosmo, nchi, nsrc, Kf, 2, ia + off, cc) : 0.0;
              const double shi = row_valid(C, q, ib) ? (double)src_t(T, ncosmo, nchi, nsrc, Kf, 2, ib + off, cc) : 0.0;
              limb = (slo * (1 - f) + f * shi) * sqrt(3.14159265358979323846 / 2 / (l + 0.5)) / q;
            }
            out = limb;
          }
        }
        C.delta[((size_t)q_ix * nl + j) * C.nsrc + src] = out;
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 128);
}

}  // namespace tc

cudaError_t launch_proj_tc(const DevCosmo* cosmos, int ncosmo, int nq, int nsrc, int nk, int nl, const double* chi,
                           const float* dchi_f, int nchi, float2* tsrc, int* err, cudaStream_t s) {
  static const bool attr = [] {
    cudaFuncSetAttribute(tc::proj_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kProjSmem);
    cudaGetLastError();
    return true;
  }();
  (void)attr;
  if (nchi > tc::kProjMaxChi) return cudaErrorInvalidValue;
  dim3 gt((nk + 31) / 32, (ncosmo + 31) / 32, nchi * nsrc);
  tc::proj_src_transpose_kernel<<<gt, dim3(32, 8), 0, s>>>(cosmos, ncosmo, nchi, nk, nsrc, tsrc);
  dim3 grid(((ncosmo + 127) / 128) * ((nl + 127) / 128), nsrc, nq);
  tc::proj_tc_kernel<<<grid, 256, tc::kProjSmem, s>>>(cosmos, ncosmo, chi, dchi_f, nchi, tsrc, err);
  return cudaGetLastError();
}

}  // namespace cgdev
