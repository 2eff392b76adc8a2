// FMA-throughput probe of the benchmark (libtchem_gb_probe.so, not part of the engine library):
// the roofline denominators of the time-advance kernels.
//
// The time advance is bound by arithmetic, not memory: the plain form by the FP64 pipe, the
// mixed form by FP32 FMA, and the measured GPU peaks list only HBM and BF16 tensor figures. The
// probe runs 8 independent FMA chains per thread on a grid that fills every SM and reports
// FLOP/s (2 per FMA). Return codes: 0 ok, 1 bad argument, 3 CUDA error, 5 allocation failed.
#include <cuda_runtime.h>

#include <cstdint>


namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == T(-12345.678)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
int measure(int blocks_per_sm, int iters, double* flops_per_s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * blocks_per_sm, block = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * grid * block) != cudaSuccess) return 5;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain_kernel<T><<<grid, block>>>(out, iters / 4, T(0.999999), T(1e-7));  // warm-up
  cudaEventRecord(e0);
  fma_chain_kernel<T><<<grid, block>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return 3;
  const double flops = 2.0 * 8.0 * 16.0 * static_cast<double>(iters) * grid * block;
  *flops_per_s = flops / (ms * 1e-3);
  return 0;
}

}  // namespace

extern "C" int tchem_gb_probe_fma_peak(int fp64, int blocks_per_sm, int iters, double* flops_per_s) {
  if (!flops_per_s || blocks_per_sm <= 0 || iters <= 0) return 1;
  return fp64 ? measure<double>(blocks_per_sm, iters, flops_per_s) : measure<float>(blocks_per_sm, iters, flops_per_s);
}
