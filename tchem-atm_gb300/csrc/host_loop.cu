// The carry-over step of the reference's host time loop, on the device.
//
// The reference's box-model driver (src/examples/TChem_AtmosphericChemistry.cpp:312-352) calls
// runDeviceBatch repeatedly; each call advances every sample by at most
// num_time_iterations_per_interval steps, and between calls a parallel_reduce copies each
// sample's returned time and step size into its time-advance record (tadv(i)._tbeg = t(i),
// tadv(i)._dt = dt(i)) and sums t for the loop's stopping test (mean t >= 0.9999 tend).
// tchem_gb_time_advance_carry_over is that step: one launch, no host round trip.
#include <cuda_runtime.h>

#include "capi_internal.hpp"

namespace tchem_gb {
namespace {

constexpr int kCarryThreads = 256;

__global__ void __launch_bounds__(kCarryThreads) carry_over_kernel(tchem_gb_tadv* tadv, const double* t,
                                                                   const double* dt, int n, int iters_per_interval,
                                                                   double* t_sum) {
  __shared__ double part[kCarryThreads / 32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ti = t[i];
    tadv[i].tbeg = ti;
    tadv[i].dt = dt[i];
    if (iters_per_interval > 0) tadv[i].num_time_iterations_per_interval = iters_per_interval;
    acc += ti;
  }
  if (!t_sum) return;
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kCarryThreads / 32; ++w) s += part[w];
    atomicAdd(t_sum, s);
  }
}

}  // namespace
}  // namespace tchem_gb

using namespace tchem_gb;

extern "C" int tchem_gb_time_advance_carry_over(tchem_gb_tadv* tadv, const double* t_out, const double* dt_out,
                                                int nbatch, int iters_per_interval, double* t_sum,
                                                void* stream_v) {
  if (nbatch < 0) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_carry_over: negative batch size");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  if (t_sum) {
    const cudaError_t e = cudaMemsetAsync(t_sum, 0, sizeof(double), stream);
    if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_time_advance_carry_over: cudaMemsetAsync");
  }
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!tadv || !t_out || !dt_out) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_carry_over: null argument");
  int dev = 0;
  cudaGetDevice(&dev);
  const int sms = device_info(dev).sm_count > 0 ? device_info(dev).sm_count : 1;
  const int need = (nbatch + kCarryThreads - 1) / kCarryThreads;
  const int grid = need < 4 * sms ? need : 4 * sms;
  carry_over_kernel<<<grid, kCarryThreads, 0, stream>>>(tadv, t_out, dt_out, nbatch, iters_per_interval, t_sum);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_time_advance_carry_over: kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}
