// Instantiation of the FP32 mixed-precision form with the Gauss-Jordan inverse and full Newton
// (one FP64-residual refinement sweep per solve), one sample per 2 warps: MC=64 columns, one row
// per thread (one translation unit per kernel so the kernels compile in parallel).
#include "kernels_mixed_impl.cuh"

namespace tchem_gb {

cudaError_t launch_mixgj_64_1_g2(const AdvanceParams& P, int grid, int threads, size_t smem, cudaStream_t stream) {
  auto k = mixed::trbdf2_mixed_kernel<64, 1, true, 2, true>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, threads, smem, stream>>>(P);
  return cudaGetLastError();
}

const void* kernel_mixgj_64_1_g2() {
  return reinterpret_cast<const void*>(mixed::trbdf2_mixed_kernel<64, 1, true, 2, true>);
}

}  // namespace tchem_gb
