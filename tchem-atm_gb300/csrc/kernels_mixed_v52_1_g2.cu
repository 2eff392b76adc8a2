// Instantiation of the FP32-LU (with FP64-residual refinement) mixed-precision kernel with one
// sample per 2 warps: MC=52 columns, one row per thread (one translation unit per kernel so the
// kernels compile in parallel).
#include "kernels_mixed_impl.cuh"

namespace tchem_gb {

cudaError_t launch_mixed_52_1_g2(const AdvanceParams& P, int grid, int threads, size_t smem, cudaStream_t stream) {
  auto k = mixed::trbdf2_mixed_kernel<52, 1, false, 2>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, threads, smem, stream>>>(P);
  return cudaGetLastError();
}

const void* kernel_mixed_52_1_g2() {
  return reinterpret_cast<const void*>(mixed::trbdf2_mixed_kernel<52, 1, false, 2>);
}

}  // namespace tchem_gb
