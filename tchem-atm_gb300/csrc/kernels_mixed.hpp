// Mixed-precision form: FP32 Newton LU and solves held in registers, FP64 residual, state and
// error control.
#pragma once

#include <cuda_runtime.h>

#include "advance.hpp"

namespace tchem_gb {

struct MixedConfig {
  const void* kernel = nullptr;
  int warps_per_block = 0;
  int grid = 0;
  size_t smem = 0;
  int threads_per_sample = 32;
  MixedLayout ml{};
};

// e3: the E3SM instantiations (per-sample rate constants and source terms); lu_nnz: entries of
// the mechanism's static-order sparse LU (0: no program, the sparse-LU shapes are not used).
MixedConfig mixed_config(const MechLayout& L, int threads_per_sample, int sm_count, int max_smem_optin, int nbatch,
                         bool simplified, bool e3 = false, int lu_nnz = 0);
cudaError_t launch_trbdf2_mixed(const AdvanceParams& P, const MechLayout& L, int grid, int warps_per_block,
                                size_t smem, int threads_per_sample, cudaStream_t stream);

}  // namespace tchem_gb
