// Instantiation of the full-Newton FP32 form with the static-order sparse LU, one warp per sample,
// 4 rows per lane (up to 128 species; one translation unit per kernel so the kernels compile in
// parallel).
#include "kernels_mixed_impl.cuh"

namespace tchem_gb {

cudaError_t launch_mixsp_128_4(const AdvanceParams& P, int grid, int threads, size_t smem, cudaStream_t stream) {
  auto k = mixed::trbdf2_mixed_kernel<128, 4, true, 1, true, false, true>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, threads, smem, stream>>>(P);
  return cudaGetLastError();
}

const void* kernel_mixsp_128_4() {
  return reinterpret_cast<const void*>(mixed::trbdf2_mixed_kernel<128, 4, true, 1, true, false, true>);
}

}  // namespace tchem_gb
