// Schur-complement tile update on the 5th-generation tensor cores: for each tile,
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
    tc::mbar_wait(mbar, 0, kSpinLimit);  // a second bounded window for the MMAs in flight
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

}  // namespace
}  // namespace tchem_gb

using namespace tchem_gb;

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
  return TCHEM_GB_OK;
}
