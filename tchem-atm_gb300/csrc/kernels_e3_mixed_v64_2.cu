// Instantiation of the E3SM variant (per-sample rate constants and external sources) of the
// FP32-LU mixed-precision kernel for MC=64 columns and 2 rows per lane (one translation unit per
// kernel so the kernels compile in parallel).
#include "kernels_mixed_impl.cuh"

namespace tchem_gb {

cudaError_t launch_e3mixed_64_2(const AdvanceParams& P, int grid, int threads, size_t smem, cudaStream_t stream) {
  auto k = mixed::trbdf2_mixed_kernel<64, 2, false, 1, false, true>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, threads, smem, stream>>>(P);
  return cudaGetLastError();
}

const void* kernel_e3mixed_64_2() {
  return reinterpret_cast<const void*>(mixed::trbdf2_mixed_kernel<64, 2, false, 1, false, true>);
}

}  // namespace tchem_gb
