// Host-callable launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include "advance.hpp"

namespace tchem_gb {

// Plain FP64 form (kernels_fp64.cu).
size_t fp64_warp_smem_bytes(const MechLayout& L, int lda, bool matrix_in_smem, bool src_section = false);
cudaError_t launch_trbdf2_fp64(const AdvanceParams& P, int grid, int warps_per_block, size_t smem,
                               cudaStream_t stream);
const void* trbdf2_fp64_kernel_ptr(int m);

// Tensor-core full-Newton form for mechanisms of 129 to tc_advance_max_species() active species
// (kernels_tc_advance.cu): one CTA of 128 threads per sample, one CTA per SM, the FP32 Newton
// matrix in a global slot of tc_advance_matrix_floats() floats per CTA (AdvanceParams::gmat,
// gmat_stride in floats).
size_t tc_advance_smem_bytes(const MechLayout& L);
size_t tc_advance_matrix_floats();
int tc_advance_max_species();
cudaError_t launch_trbdf2_tc(const AdvanceParams& P, int grid, size_t smem, cudaStream_t stream);

// Discrete adjoint of the plain form (kernels_adjoint.cu): one warp per sample, one mechanism.
struct AdjointParams {
  MechDev mech;
  const double* rate_param;
  const double* k_scale;         // [R] rate-constant multipliers of the forward run, or null
  int32_t B;
  const double* state;           // [B][state_dim] initial states of the forward run
  int32_t state_dim;
  const tchem_gb_tadv* tadv;     // [B] (Newton settings)
  const double* tol_newton;      // [2]
  const double* tape_dt;         // [B][tape_cap]
  const double* tape_ckpt;       // [B][tape_cap / kTapeSegment + 1][m]
  const int32_t* tape_nsteps;    // [B]
  int32_t tape_cap;
  const double* lambda;          // [B][m] dL/dy(t_end)
  double* grad_x0;               // [B][m] dL/dy(t_0)
  double* grad_k;                // [B][R] dL/dtheta_r (k_r scaled by exp(theta_r))
  int32_t* status;               // [B]
  double* seg;                   // per warp: [kTapeSegment][2][m]
  int64_t seg_stride;
  double* gmat;                  // per-warp matrix slots when not in shared memory
  int64_t gmat_stride;
  int32_t lda;
  int32_t matrix_in_smem;
  uint32_t warp_smem_bytes;
  int32_t* queue;
  int32_t* error_word;
};
size_t adjoint_warp_smem_bytes(const MechLayout& L, int lda, bool matrix_in_smem);
const void* adjoint_kernel_ptr(int m);
cudaError_t launch_adjoint(const AdjointParams& P, int grid, int warps, size_t smem, cudaStream_t stream);

// Unit kernels on the same tables (kernels_fp64.cu): one warp per sample.
struct UnitParams {
  MechDev mech;
  const double* rate_param[kMaxGroupSlots];
  int32_t slot_of_mech[kMaxMechs];
  const int32_t* mech_of_sample;
  int32_t B;
  const double* state;  // [B][state_dim]
  int32_t state_dim;
  double* out;          // kforward [B][R], rhs [B][m], jacobian [B][m][m]
  int32_t* error_word;
  int32_t* status;      // [B] or null: TCHEM_GB_SAMPLE_BAD_MECH for samples with no mechanism
};
enum UnitKind { UNIT_KFORWARD = 0, UNIT_RHS = 1, UNIT_JACOBIAN = 2 };
cudaError_t launch_unit(const UnitParams& P, UnitKind kind, cudaStream_t stream);

// E3SM gas-chemistry rates (kernels_e3sm.cu): one warp per sample, grid-stride over samples.
enum E3smOut { E3SM_KFOR = 0, E3SM_ROP = 1, E3SM_OMEGA = 2, E3SM_KEFF = 3 };
struct E3smParams {
  MechDev mech;            // plain-form tables (CSR net-production program) and e3_* tables
  int32_t B;
  const double* state;     // [B][state_dim]
  int32_t state_dim;
  const double* photo;     // [B][n_photo] or null
  int32_t n_photo;
  const double* ext;       // [B][m] or null (E3SM_OMEGA)
  double* out;             // kfor, rop, keff [B][R]; omega [B][m]
};
cudaError_t launch_e3sm(const E3smParams& P, E3smOut kind, int sm_count, cudaStream_t stream);

// Gas-aerosol problem (SIMPOL.1 phase transfer) of the plain form (kernels_aero.cu): one warp per
// sample, one gas mechanism and one aerosol model per call. The ODE vector is [active gas species,
// particle 0's aerosol species, particle 1's, ...], M = m_gas + nP * nA entries.
struct AeroDev {
  int32_t nA, nP, nS, m_gas, M;  // aerosol species per particle, particles, SIMPOL entries, active gas, ODEs
  const int32_t* sim_idx;        // [nS][3]: aerosol ODE index (particle 0), gas index, alpha from N*
  const double* sim_par;         // [nS][7]: B1..B4, diffusion coefficient, N*, gas molecular weight
  const double* density;         // [nA] kg/m3
  const double* mw;              // [nA] kg/mol
  double vol0, mass0, moles0;    // particle volume, mass and moles floors
};
// Byte offsets of one warp's shared-memory sections (computed on the host, read by the kernel).
struct AeroWarpLayout {
  uint32_t x, f, keff, q, w, piv, simc, part, dsim, nc, A, bytes;
};
AeroWarpLayout aero_warp_layout(const MechLayout& L, const AeroDev& A, int lda, bool matrix_in_smem);
struct AeroParams {
  MechDev mech;                   // gas tables (plain form)
  AeroDev aero;
  AeroWarpLayout wl;
  int32_t B, n_gas, state_dim;    // samples, gas species (active + constant), state row width
  const double* number_conc;      // [B][nP]
  const double* tol_newton;       // [2]
  const double* tol_time;         // [M][2]
  const tchem_gb_tadv* tadv;      // [B]
  const double* state;            // [B][state_dim]: rho, p, T, gas species, particles
  double* state_out;              // [B][state_dim] (may alias state)
  double* t_out;                  // [B] in/out
  double* dt_out;                 // [B]
  int32_t* status;                // [B]
  tchem_gb_sample_stats* stats;   // [B] or null
  double* omega;                  // right-hand-side mode: [B][M]
  double* gmat;                   // per-warp matrix slots in global memory (when not in smem)
  int64_t gmat_stride;
  int32_t lda;
  int32_t matrix_in_smem;
  int32_t* queue;
  int32_t* error_word;
};
constexpr int kAeroMaxOde = 320;  // largest ODE system of the aerosol kernel (10 entries per lane)
const void* aero_kernel_ptr(int M, bool rhs_only);
cudaError_t launch_aero(const AeroParams& P, bool rhs_only, int grid, int warps_per_block, size_t smem,
                        cudaStream_t stream);

// Groups samples by mechanism group: items[g * B + k], counts[g] (kernels_fp64.cu).
struct GroupMap {
  int32_t group_of_mech[kMaxMechs];
};
cudaError_t launch_bucket(const int32_t* mech_of_sample, int B, const GroupMap& G, int n_mechs,
                          int32_t* counts, int32_t* items, int32_t* status, cudaStream_t stream);

}  // namespace tchem_gb
