// Tensor-core kernels of the blocked FP32 LU (the 300-species factorization). The Schur-complement
// tile update: for each tile,
// D[128][N] -= A[128][32] * B[32][N] with TF32 operands and FP32 accumulation, the trailing-matrix
// update of a blocked LU with 32-column panels (four kind::tf32 MMAs of K = 8 into one TMEM
// accumulator). One CTA of four warps per tile: the operands are written into the K-major
// no-swizzle canonical layout in shared memory, the D tile is moved into TMEM (thread = row), one
// elected thread issues the MMAs with A negated and commits them to an mbarrier, and the warps
// read D back. Every wait is bounded; on expiry the kernel records kErrBarrierTimeout in the
// device error word, waits one more bounded window for the MMAs in flight, frees its TMEM and
// returns without writing D.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/tchem_gb.h"
#include "capi_internal.hpp"
#include "engine.cuh"
#include "tc_tile.cuh"

namespace tchem_gb {
namespace {

constexpr int kTcRows = 128;  // M of the MMA (one TMEM lane per row)
constexpr int kTcK = 32;      // panel width

__global__ void __launch_bounds__(128, 1) tc_tile_update_kernel(int N, uint32_t ncols, const float* A, const float* B,
                                                                float* D, int32_t* error_word) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* sa = smem;                              // A operand: 128 x 32, 16 KB
  unsigned char* sb = smem + kTcRows * kTcK * 4;         // B operand: N x 32 (K-major), N * 128 B
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sb + static_cast<size_t>(N) * kTcK * 4);
  uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t t = blockIdx.x;
  const float* At = A + t * kTcRows * kTcK;
  const float* Bt = B + t * static_cast<size_t>(kTcK) * N;
  float* Dt = D + t * static_cast<size_t>(kTcRows) * N;

  if (warp == 0) tc::tmem_alloc(slot, ncols);
  if (tid == 0) tc::mbar_init(mbar, 1);
  for (int e = tid; e < kTcRows * kTcK; e += 128) {
    const int r = e / kTcK, k = e - r * kTcK;
    *reinterpret_cast<float*>(sa + tc::kmajor_offset(r, k, kTcK)) = At[e];
  }
  for (int e = tid; e < kTcK * N; e += 128) {
    const int k = e / N, n = e - k * N;
    *reinterpret_cast<float*>(sb + tc::kmajor_offset(n, k, kTcK)) = Bt[e];
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *slot;
  const int row = 32 * warp + lane;
  for (int c = 0; c < N; c += 16) {
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = Dt[static_cast<size_t>(row) * N + c + i];
    tc::tmem_st16(tbase, warp, c, v);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    const uint32_t id = tc::idesc_tf32(kTcRows, N, true);
    const uint32_t a0 = tc::smem_addr(sa), b0 = tc::smem_addr(sb);
#pragma unroll
    for (int s = 0; s < kTcK / 8; ++s)
      tc::mma_tf32(tbase, tc::smem_desc(a0 + 256 * s, 128, 32 * kTcK), tc::smem_desc(b0 + 256 * s, 128, 32 * kTcK), id,
                   true);
    tc::commit(mbar);
  }
  bool ok = tc::mbar_wait(mbar, 0, kSpinLimit);
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  if (!ok) {
    if (tid == 0) atomicOr(error_word, kErrBarrierTimeout);
    // a second bounded window for the MMAs in flight; if it also expires, the TMEM below is freed
    // while MMAs may still write it, which the error word records
    const bool drained = __syncthreads_and(tc::mbar_wait(mbar, 0, kSpinLimit) ? 1 : 0) != 0;
    if (!drained && tid == 0) atomicOr(error_word, kErrMmaInFlight);
  }
  tc::fence_after_sync();
  if (ok) {
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(tbase, warp, c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) Dt[static_cast<size_t>(row) * N + c + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

// Blocked right-looking LU with partial pivoting of one FP32 matrix per CTA (four warps), in place
// in global memory (L2-resident): 32-column panels factored on the CUDA cores (pivot = first
// largest magnitude in the current row order, whole-row swaps), U12 = L11^-1 A12 on the CUDA
// cores, and the trailing update A22 -= L21 U12 on the tensor cores in tiles of 128 rows x up to
// 256 columns (TF32 operands, FP32 accumulation in TMEM) -- the algorithm of the oracle's
// factor_blocked with TF32 tiles. info[b]: 0, k + 1 when column k has no usable pivot, -1 when a
// bounded wait expired (the factors are then incomplete).
__global__ void __launch_bounds__(128, 1) tc_lu_kernel(int m, int lda, float* A, int32_t* piv, int32_t* info,
                                                       int32_t* error_word) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* sa = smem;                       // A operand: 128 x 32 (16 KB)
  unsigned char* sb = smem + kTcRows * kTcK * 4;  // B operand: up to 256 x 32 (32 KB)
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sb + 256 * kTcK * 4);
  uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 1);
  float* red_v = reinterpret_cast<float*>(mbar + 2);  // [4] per-warp pivot candidates
  int* red_i = reinterpret_cast<int*>(red_v + 4);     // [4]
  int* s_piv = red_i + 4;                             // the chosen pivot row (-1: none)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* M = A + static_cast<size_t>(blockIdx.x) * m * lda;
  int32_t* pv = piv + static_cast<size_t>(blockIdx.x) * m;
  auto at = [&](int i, int j) -> float& { return M[static_cast<size_t>(i) * lda + j]; };

  if (warp == 0) tc::tmem_alloc(slot, 256);
  if (tid == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *slot;
  uint32_t phase = 0;
  int status = 0;
  for (int k0 = 0; k0 < m && status == 0; k0 += kTcK) {
    const int p1 = min(m, k0 + kTcK);
    for (int k = k0; k < p1; ++k) {
      float best = -1.f;
      int bi = m;
      for (int i = k + tid; i < m; i += 128) {
        const float v = fabsf(at(i, k));
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(kFullMask, best, o);
        const int oi = __shfl_xor_sync(kFullMask, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        red_v[warp] = best;
        red_i[warp] = bi;
      }
      __syncthreads();
      if (tid == 0) {
        float b = red_v[0];
        int ii = red_i[0];
        for (int w = 1; w < 4; ++w)
          if (red_v[w] > b || (red_v[w] == b && red_i[w] < ii)) {
            b = red_v[w];
            ii = red_i[w];
          }
        *s_piv = (b > 0.f && isfinite(b) && ii < m) ? ii : -1;
      }
      __syncthreads();
      const int p = *s_piv;
      if (p < 0) {
        status = k + 1;
        break;
      }
      if (tid == 0) pv[k] = p;
      if (p != k)
        for (int j = tid; j < m; j += 128) {
          const float a = at(k, j);
          at(k, j) = at(p, j);
          at(p, j) = a;
        }
      __syncthreads();
      const float inv = 1.f / at(k, k);
      for (int i = k + 1 + tid; i < m; i += 128) at(i, k) *= inv;
      __syncthreads();
      const int w = p1 - k - 1;
      if (w > 0) {
        const int total = (m - k - 1) * w;
        for (int e = tid; e < total; e += 128) {
          const int i = k + 1 + e / w, j = k + 1 + e % w;
          at(i, j) -= at(i, k) * at(k, j);
        }
      }
      __syncthreads();
    }
    if (status != 0) break;
    // U12 = L11^-1 A12 (unit lower L11), one column per thread
    for (int j = p1 + tid; j < m; j += 128)
      for (int k = k0; k < p1; ++k) {
        const float u = at(k, j);
        for (int i = k + 1; i < p1; ++i) at(i, j) -= at(i, k) * u;
      }
    __syncthreads();
    const int kb = p1 - k0;
    for (int r0 = p1; r0 < m && status == 0; r0 += kTcRows) {
      for (int c0 = p1; c0 < m && status == 0; c0 += 256) {
        const int N = (min(256, m - c0) + 15) & ~15;
        for (int e = tid; e < kTcRows * kTcK; e += 128) {
          const int r = e / kTcK, kk = e - r * kTcK, i = r0 + r;
          *reinterpret_cast<float*>(sa + tc::kmajor_offset(r, kk, kTcK)) = (i < m && kk < kb) ? at(i, k0 + kk) : 0.f;
        }
        for (int e = tid; e < N * kTcK; e += 128) {
          const int n = e / kTcK, kk = e - n * kTcK, j = c0 + n;
          *reinterpret_cast<float*>(sb + tc::kmajor_offset(n, kk, kTcK)) = (j < m && kk < kb) ? at(k0 + kk, j) : 0.f;
        }
        const int i = r0 + tid;
        for (int c = 0; c < N; c += 16) {
          float v[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int j = c0 + c + q;
            v[q] = (i < m && j < m) ? at(i, j) : 0.f;
          }
          tc::tmem_st16(tbase, warp, c, v);
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
          const uint32_t id = tc::idesc_tf32(kTcRows, N, true);
          const uint32_t a0 = tc::smem_addr(sa), b0 = tc::smem_addr(sb);
#pragma unroll
          for (int s4 = 0; s4 < kTcK / 8; ++s4)
            tc::mma_tf32(tbase, tc::smem_desc(a0 + 256 * s4, 128, 32 * kTcK),
                         tc::smem_desc(b0 + 256 * s4, 128, 32 * kTcK), id, true);
          tc::commit(mbar);
        }
        const uint32_t ph = phase;
        phase ^= 1u;
        bool done = tc::mbar_wait(mbar, ph, kSpinLimit);
        done = __syncthreads_and(done ? 1 : 0) != 0;
        if (!done) {
          if (tid == 0) atomicOr(error_word, kErrBarrierTimeout);
          // a second bounded window for the MMAs in flight (expired too: TMEM is freed while MMAs
          // may still write it, recorded in the error word)
          const bool drained = __syncthreads_and(tc::mbar_wait(mbar, ph, kSpinLimit) ? 1 : 0) != 0;
          if (!drained && tid == 0) atomicOr(error_word, kErrMmaInFlight);
          status = -1;
        }
        tc::fence_after_sync();
        if (done) {
          for (int c = 0; c < N; c += 16) {
            float v[16];
            tc::tmem_ld16(tbase, warp, c, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int j = c0 + c + q;
              if (i < m && j < m) at(i, j) = v[q];
            }
          }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
      }
    }
  }
  if (tid == 0) info[blockIdx.x] = status;
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

}  // namespace
}  // namespace tchem_gb

using namespace tchem_gb;

extern "C" int tchem_gb_tc_lu_factor_tf32(int nbatch, int m, int lda, float* A, int32_t* piv, int32_t* info,
                                          void* stream) {
  if (nbatch < 0 || m < 1 || lda < m)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_tc_lu_factor_tf32: need nbatch >= 0, m >= 1 and lda >= m");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!A || !piv || !info) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_tc_lu_factor_tf32: null array");
  int dev = 0;
  cudaGetDevice(&dev);
  unsigned char* ws = nullptr;
  try {
    ws = static_cast<unsigned char*>(owned_workspace(dev, kHeaderBytes));
  } catch (...) {
    return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_tc_lu_factor_tf32: workspace allocation failed");
  }
  // at most two CTAs per SM (each holds 256 of the SM's 512 TMEM columns)
  const size_t smem = 100 * 1024;
  cudaError_t e = cudaFuncSetAttribute(tc_lu_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(tc_lu_kernel)");
  tc_lu_kernel<<<nbatch, 128, smem, static_cast<cudaStream_t>(stream)>>>(m, lda, A, piv, info,
                                                                         reinterpret_cast<int32_t*>(ws + 64));
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tc_lu_kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}

extern "C" int tchem_gb_tc_tile_update_tf32(int ntiles, int N, const float* A, const float* B, float* D,
                                            void* stream) {
  if (ntiles < 0 || N < 16 || N > 256 || N % 16 != 0)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_tc_tile_update_tf32: N must be a multiple of 16 in [16, 256]");
  if (ntiles == 0) return TCHEM_GB_OK;
  if (!A || !B || !D) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_tc_tile_update_tf32: null array");
  int dev = 0;
  cudaGetDevice(&dev);
  unsigned char* ws = nullptr;
  try {
    ws = static_cast<unsigned char*>(owned_workspace(dev, kHeaderBytes));
  } catch (...) {
    return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_tc_tile_update_tf32: workspace allocation failed");
  }
  uint32_t ncols = 32;
  while (ncols < static_cast<uint32_t>(N)) ncols <<= 1;
  // at most two CTAs per SM (each holds up to 256 of the SM's 512 TMEM columns)
  const size_t need = static_cast<size_t>(kTcRows) * kTcK * 4 + static_cast<size_t>(N) * kTcK * 4 + 16;
  const size_t smem = std::max<size_t>(need, 100 * 1024);
  cudaError_t e = cudaFuncSetAttribute(tc_tile_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(tc_tile_update_kernel)");
  tc_tile_update_kernel<<<ntiles, 128, smem, static_cast<cudaStream_t>(stream)>>>(
      N, ncols, A, B, D, reinterpret_cast<int32_t*>(ws + 64));
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tc_tile_update_kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}
