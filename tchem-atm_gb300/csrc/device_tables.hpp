// Packed per-mechanism tables for the device kernels.
//
// The reference keeps the mechanism as arrays-of-structs read from global memory on every
// RHS call (KineticModelNCAR_ConstData, src/core/TChem_KineticModelNCAR_ConstData.hpp:30-113)
// and recomputes every rate constant inside every RHS call
// (src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:96). Here the mechanism is compiled once
// into three small sparse programs that a CTA stages into shared memory with one bulk copy:
//
//  * rate of progress: for reaction r, q_r = keff_r * prod_{f in [rf_ptr[r], rf_ptr[r+1])} x[rf_sp[f]]
//    where every active reactant appears |nu| times and keff_r folds the rate constant and the
//    (per-sample constant) concentrations of constant species;
//  * net production (CSR over active species k): omega_k = emis_k + sum_e pr_nu[e] * q[pr_r[e]];
//  * analytic Jacobian: for each factor slot f, d_f = keff_r * prod_{g != f} x[rf_sp[g]] is
//    dq_r/dx along that slot; Jacobian nonzero z = (jz_row[z], jz_col[z]) accumulates
//    J_z = sum_{c in [jz_ptr[z], jz_ptr[z+1])} jc_nu[c] * d[jc_f[c]].
//
// Rate-constant parameters stay in global memory: they are read once per sample.
#pragma once

#include <cstdint>
#include <vector>

#include "kinetic_model.hpp"
#include "sparse_lu.hpp"

namespace tchem_gb {

enum DevRateType : int32_t { RATE_ARRHENIUS = 0, RATE_TROE = 1, RATE_CMAQ_H2O2 = 2, RATE_ZERO = 3 };

// Rate forms of the E3SM gas chemistry (kernels_e3sm.cu); E3_NONE reactions take the photolysis
// input or 0.
enum E3smRateType : int32_t { E3_NONE = 0, E3_ARRHENIUS = 1, E3_TROE = 2, E3_CMAQ_H2O2 = 3, E3_JPL = 4, E3_RJPL = 5 };
constexpr int kE3smParams = 10;  // parameters per reaction in MechDev::e3_param

// Byte offsets of each section inside the staged blob (16-byte aligned sections).
struct MechLayout {
  int32_t m, n, nconst, R, NF, NP, NZ, NC;
  int32_t off_rf_ptr, off_rf_sp;            // int32[R+1], int16[NF]
  int32_t off_pr_ptr, off_pr_r, off_pr_nu;  // int32[m+1], int16[NP], double[NP]
  int32_t off_jz_rc, off_jz_ptr;            // int32[NZ] (row<<16 | col), int32[NZ+1]
  int32_t off_jc_f, off_jc_nu, off_jc_nu32;  // int16[NC], double[NC], float[NC]
  int32_t off_emis;                         // double[m]
  int32_t blob_bytes;                       // multiple of 16
  int32_t max_factors;                      // max factor slots of one reaction
  // Sliced-ELL programs of the mixed form (blob_x): items sorted by entry count, 32 per slice,
  // entries stored [slice][entry][lane] and padded within the slice with a dummy index whose
  // value is 0 (d32[NF] for the Jacobian, q[R] for the net production), so every lane of a
  // slice runs the same trip count with independent loads.
  int32_t NJS, NJE, NWS, NWE;
  int32_t off_js_rc, off_js_cnt, off_js_off, off_jse_f, off_jse_nu32;  // Jacobian nonzeros
  int32_t off_ws_sp, off_ws_cnt, off_ws_off, off_wse_r, off_wse_nu;    // net production per species
  // Sparse-LU shape (m <= kSparseLuMaxSpecies, else -1): per Jacobian slot of the sliced-ELL
  // program (off_js_rc), the entry of (row, col) in the static-order filled pattern (int16).
  int32_t off_js_e;
};

// Device pointers of one mechanism on one device (passed by value to kernels).
struct MechDev {
  MechLayout L;
  const unsigned char* blob;  // staged tables (global copy, 256-byte aligned)
  const int32_t* rate_type;   // [R]
  const double* rate_param;   // [R][8]
  const int32_t* conv_exp;    // [R]
  const int32_t* cf_ptr;      // [R+1] constant-species factors of reaction r
  const int32_t* cf_idx;      // constant-species slot (0..nconst-1), one entry per unit of |nu|
  double conv_ppm;
  // Stoichiometry by reaction in the reference's layout (KineticModelNCAR_ConstData reacSidx,
  // reacNuki, reacNreac, reacNprod): read by the adjoint for nu_r . mu.
  const int32_t* rx_sidx;  // [R][rx_S]
  const double* rx_nu;     // [R][rx_S], reactants signed negative, products from rx_S / 2
  const int32_t* rx_n;     // [R][2]: number of reactants, products
  int32_t rx_S;
  // E3SM rate tables. e3_param per form: ARRHENIUS A, B, C, D, E; TROE the 8 reacPpar values;
  // CMAQ_H2O2 A1, B1, C1, A2, B2, C2; JPL k0_A, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc; R_JPL the
  // JPL values then A, B, C.
  const int32_t* e3_type;     // [R] E3smRateType
  const double* e3_param;     // [R][kE3smParams]
  const int32_t* e3_adj_ptr;  // [R+1] adjust factors of reaction r: e3_adj_sp[e3_adj_ptr[r] ..), file order
  const int32_t* e3_adj_sp;   // species whose concentration multiplies the rate constant
  const int32_t* e3_o1d;      // [e3_no1d][7]: reactions 1..3, photolysis reaction, species 1..3
  const double* e3_o1d_par;   // [e3_no1d][6]: A1, C1, A2, C2, A3, C3
  int32_t e3_no1d, M_index;
  // Static-order sparse LU program (sparse_lu.hpp), or null when the mechanism is too large.
  const int32_t* lu_prog;
  SparseLuLayout lu;
};

// Host-side packed tables, built from a parsed kinetic model.
struct HostTables {
  MechLayout L{};                  // plain form (CSR programs)
  std::vector<unsigned char> blob;
  MechLayout Lx{};                 // mixed form (sliced-ELL programs)
  std::vector<unsigned char> blob_x;
  SparseLuHost slu;                // sparse-LU program (slu.lay.m == 0: none)
  std::vector<int32_t> rate_type, conv_exp, cf_ptr, cf_idx;
  std::vector<double> rate_param;
  std::vector<int32_t> rx_sidx, rx_n;  // stoichiometry by reaction (MechDev::rx_*)
  std::vector<double> rx_nu;
  int32_t rx_S = 0;
  // Structural signature: mechanisms with equal signatures share one kernel launch.
  std::vector<int64_t> signature;
  bool supported = true;     // false when the mechanism has rate types outside the box path
  std::string unsupported_reason;
  // E3SM tables (MechDev::e3_*); e3sm_state_free: no active species scales a rate constant, so
  // the E3SM time advance may evaluate them once per sample.
  std::vector<int32_t> e3_type, e3_adj_ptr, e3_adj_sp, e3_o1d;
  std::vector<double> e3_param, e3_o1d_par;
  int32_t M_index = -1;
  bool e3sm_valid = true;  // false: the tables cannot drive the E3SM kernels (reason below)
  std::string e3sm_invalid_reason;
  bool e3sm_state_free = true;
  std::string e3sm_reason;
};

HostTables build_host_tables(const KineticModel& km);

struct DeviceTables {
  int device = -1;
  MechDev dev{};    // plain-form tables
  MechDev dev_x{};  // mixed-form tables (same rate parameters, sliced-ELL blob)
  void* allocation = nullptr;
};

DeviceTables* upload_tables(const HostTables& ht, int device);
void destroy_device_tables(DeviceTables* t);

}  // namespace tchem_gb
