// Launch parameters of the time-advance kernels (shared by host launch code and kernels).
#pragma once

#include <cstdint>

#include "../../include/tchem_gb.h"
#include "device_tables.hpp"

namespace tchem_gb {

constexpr int kMaxMechs = 64;       // mechanisms per time-advance call
constexpr int kMaxGroupSlots = 8;   // structure-compatible mechanisms sharing one launch
constexpr int kTapeSegment = 32;    // steps between trajectory checkpoints (adjoint)

// Byte offsets of the sections of one warp's shared-memory region (mixed form). Kept in the
// kernel parameters (constant bank) so section addresses cost no registers.
struct MixedLayout {
  uint32_t warp_bytes;
  uint32_t x, keff, q, x32, keff32, d32, ustage, lrow, pinv, piv, ybuf, vec, stats, red, item;
  uint32_t lu;   // [nnz] FP32 factors of the sparse-LU shape (else 0)
  uint32_t src;  // [m] the sample's E3SM source term (E3SM instantiations only; else 0)
  int32_t LDU, LDL;
  int32_t simplified;  // 1: simplified-Newton form; 2: full Newton on the Gauss-Jordan inverse; 0: LU
};

struct AdvanceParams {
  MechDev mech;                                 // tables of the group (shared structure)
  const double* rate_param[kMaxGroupSlots];     // per slot: [R][8] rate parameters
  int32_t slot_of_mech[kMaxMechs];              // global mechanism index -> slot (-1: other group)
  const int32_t* mech_of_sample;                // [B] or null (all samples use mechanism 0)
  const int32_t* items;                         // samples of this launch, or null (identity over n_items)
  const int32_t* n_items_dev;                   // device-side item count, or null (use n_items)
  int32_t n_items;
  int32_t* queue;                               // work-queue head, 0 at launch
  const double* tol_newton;                     // [2]
  const double* tol_time;                       // [m][2]
  const tchem_gb_tadv* tadv;                    // [B]
  const double* state;                          // [B][state_dim]
  double* state_out;                            // [B][state_dim] (may alias state)
  double* t_out;                                // [B] in/out
  double* dt_out;                               // [B]
  int32_t* status;                              // [B]
  tchem_gb_sample_stats* stats;                 // [B] or null
  int32_t state_dim;
  double* gmat;                                 // per-warp matrix slots in global memory (when not in smem)
  int64_t gmat_stride;                          // elements per slot
  int32_t lda;
  int32_t matrix_in_smem;
  uint32_t warp_smem_bytes;
  int32_t* error_word;                          // device-side error report (bounded waits)
  MixedLayout ml;                               // mixed form only
  // Trajectory record of the plain form for the discrete adjoint (tape_dt null: none): the
  // accepted step sizes and the state at the start of every kTapeSegment-th step, per sample.
  double* tape_dt;                              // [B][tape_cap]
  double* tape_ckpt;                            // [B][tape_cap / kTapeSegment + 1][m]
  int32_t* tape_nsteps;                         // [B]
  int32_t tape_cap;
  const double* k_scale;                        // [R] rate-constant multipliers (null: none)
  // E3SM inputs (null: the mechanism's rate constants and emissions): per-sample effective rate
  // constants (constant-species factors included) and source terms, row s at src_in + s * src_stride.
  const double* keff_in;                        // [B][R]
  const double* src_in;                         // [B][m] (src_stride m) or one zero row (src_stride 0)
  int64_t src_stride;
};

}  // namespace tchem_gb
