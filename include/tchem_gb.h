/*
 * C ABI of the GB300 engine for TChem-atm's batched box-model gas-chemistry time advance.
 *
 * Every entry point takes plain pointers and sizes. Device pointers are CUDA device
 * addresses; `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 * Calls that take device pointers are stream-ordered and asynchronous, like the Kokkos
 * launch they replace; the caller synchronises. Return value: TCHEM_GB_OK or an error code,
 * with a message available from tchem_gb_last_error() (thread-local).
 *
 * Reference interfaces replaced (paths inside the TChem-atm source tree):
 *   tchem_gb_mech_create_*      TChem::KineticModelData(yamlFile) + createNCAR_KineticModelConstData
 *                               src/core/TChem_KineticModelData.cpp:57-78,
 *                               src/core/TChem_KineticModelNCAR_ConstData.hpp:115-148
 *   tchem_gb_scenario_read      TChem::AtmChemistry::setScenarioConditions
 *                               src/core/TChem_AtmosphericChemistry.cpp:430-508
 *   tchem_gb_workspace_bytes    TChem::AtmosphericChemistry::getWorkSpaceSize
 *                               src/core/TChem_AtmosphericChemistry.hpp:47-81
 *   tchem_gb_time_advance       TChem::AtmosphericChemistry::runDeviceBatch (both overloads)
 *                               src/core/TChem_AtmosphericChemistry.hpp:83-155,
 *                               src/core/TChem_AtmosphericChemistry.cpp:211-271, 343-385
 *   tchem_gb_kforward           TChem::Impl::KForwardAerosol::team_invoke
 *                               src/core/impl/TChem_Impl_KForwardAerosol.hpp:44-145
 *   tchem_gb_reaction_rates     TChem::Impl::ReactionRatesAerosol::team_invoke (box-model RHS)
 *                               src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:57-143, 238-289
 *   tchem_gb_jacobian           AtmosphericChemistry_Problem::computeJacobian (analytic here)
 *                               src/core/problems/TChem_Impl_AtmosphericChemistry_Problem.hpp:202-213
 *   tchem_gb_scenario_photolysis_rates, tchem_gb_scenario_external_forcing
 *                               TChem::AtmChemistry::setScenarioConditionsPhotolysisReactions,
 *                               setScenarioConditionsExternalForcing
 *                               src/core/TChem_AtmosphericChemistry.cpp:512-631
 *   tchem_gb_e3sm_time_advance  TChem::AtmosphericChemistryE3SM::runDeviceBatch
 *                               src/core/TChem_AtmosphericChemistryE3SM.hpp:88-104
 *   tchem_gb_e3sm_reaction_rates, _rate_of_progress, _net_production_rates
 *                               TChem::ReactionRates / RateofProgress / NetProductionRates
 *                               ::runDeviceBatch, src/core/TChem_ReactionRates.hpp:59-72,
 *                               src/core/TChem_RateofProgress.hpp:60-75,
 *                               src/core/TChem_NetProductionRates.hpp:61-78
 *   tchem_gb_aero_create_*, tchem_gb_aero_scenario_particles
 *                               TChem::AerosolModelData (+ scenarioConditionParticles)
 *                               src/core/TChem_AerosolModelData.cpp:60-300
 *   tchem_gb_aero_time_advance  TChem::AerosolChemistry::runDeviceBatch
 *                               src/core/TChem_AerosolChemistry.hpp:87-103
 *   tchem_gb_aero_rhs           TChem::Impl::Aerosol_RHS::team_invoke
 *                               src/core/impl/TChem_Impl_Aerosol_RHS.hpp:57-100
 *   tchem_gb_numerics_read      TChem::Driver::createNumerics src/core/TChem_Driver.cpp:152-187
 * The host-model driver functions themselves (initialize, TChem_doTimestep, ...) are in
 * tchem_gb_driver.h (libtchem_gb_driver.so).
 */
#ifndef TCHEM_GB_H
#define TCHEM_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TCHEM_GB_ABI_VERSION 1

enum tchem_gb_error {
  TCHEM_GB_OK = 0,
  TCHEM_GB_ERR_ARG = 1,         /* invalid argument (TCHEM_CHECK_ERROR in the reference) */
  TCHEM_GB_ERR_PARSE = 2,       /* mechanism / scenario file could not be read */
  TCHEM_GB_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  TCHEM_GB_ERR_UNSUPPORTED = 4, /* feature outside the box-model path (e.g. JPL rate types) */
  TCHEM_GB_ERR_NOMEM = 5,       /* device allocation failed */
  TCHEM_GB_ERR_DEVICE = 6       /* a device-side bounded wait or check reported an error */
};

/* Per-sample status written by the time advance. The reference signals a failed sample with
 * dt_out < 0 (src/core/problems/TChem_Impl_AtmosphericChemistry.hpp:213-221); these codes
 * refine it. Failed samples also follow the reference convention state_out = 0 for the
 * active species, t_out = t_end, dt_out = -1. */
enum tchem_gb_sample_status {
  TCHEM_GB_SAMPLE_OK = 0,
  TCHEM_GB_SAMPLE_NEWTON_FAIL = 1, /* Newton failed on 4 successive step halvings */
  TCHEM_GB_SAMPLE_SKIPPED = 2,     /* t_out >= t_end on entry: nothing done */
  TCHEM_GB_SAMPLE_NEGATIVE_DT = 3, /* dt_in < 0: returned without touching the outputs */
  TCHEM_GB_SAMPLE_NONFINITE = 4,   /* non-finite value in the state or a step */
  TCHEM_GB_SAMPLE_DT_UNDERFLOW = 5, /* step size reached 0 before t_end */
  TCHEM_GB_SAMPLE_BAD_MECH = 6,     /* mech_of_sample names no mechanism of the call */
  TCHEM_GB_SAMPLE_TAPE_FULL = 7     /* more accepted steps than the trajectory record holds */
};

/* Mirrors TChem::TimeAdvance (src/core/TChem_Util.hpp:469-477), same field order and types. */
typedef struct tchem_gb_tadv {
  double tbeg, tend;
  double dt, dtmin, dtmax;
  int32_t max_num_newton_iterations;
  int32_t num_time_iterations_per_interval;
  int32_t num_outer_time_iterations_per_interval;
  int32_t jacobian_interval;
} tchem_gb_tadv;

/* Host view of a parsed mechanism in the reference's table layout
 * (TChem::KineticModelNCAR_ConstData, src/core/TChem_KineticModelNCAR_ConstData.hpp:30-113).
 * All pointers are owned by the mechanism and valid until tchem_gb_mech_destroy. */
typedef struct tchem_gb_kmcd_view {
  int32_t nSpec, nConstSpec, nReac, maxSpecInReac, M_index;
  double CONV_PPM;
  const int32_t* reacNreac;    /* [nReac] */
  const int32_t* reacNprod;    /* [nReac] */
  const int32_t* reacSidx;     /* [nReac][maxSpecInReac] */
  const double* reacNuki;      /* [nReac][maxSpecInReac] */
  const int32_t* convExponent; /* [nReac] */
  const int32_t* reacType;     /* [nReac]: 0 ARRHENIUS 1 TROE 2 CMAQ_H2O2 3 JPL 4 R_JPL_ARRHENIUS 5 PHOTO_RATE */
  int32_t nArrhenius;
  const int32_t* arrhenius_reaction; /* [nArrhenius] */
  const double* arrhenius_param;     /* [nArrhenius][5]: E, A, B, C, D */
  int32_t nTroe;
  const int32_t* reacPfal;           /* [nTroe] */
  const double* reacPpar;            /* [nTroe][8]: k0_A*1e6, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc, N */
  int32_t nCMAQ_H2O2;
  const int32_t* cmaq_reaction;      /* [nCMAQ_H2O2] */
  const double* cmaq_param;          /* [nCMAQ_H2O2][6]: A1, B1, C1, A2 (k2_A*1e6), B2, C2 */
  int32_t nEmission;
  const int32_t* emission_species;   /* [nEmission] */
  const double* emission_rate;       /* [nEmission] */
} tchem_gb_kmcd_view;

/* Host view of the E3SM rate tables of a parsed mechanism: the JPL_Coef, R_JPL_ArrheniusCoef,
 * adjust_reaction and prod_O1D members of TChem::KineticModelNCAR_ConstData
 * (src/core/TChem_KineticModelNCAR_ConstData.hpp:96-103, types src/core/TChem_Util.hpp:391-459).
 * Same ownership as tchem_gb_kmcd_view. */
typedef struct tchem_gb_e3sm_view {
  int32_t nJPL;
  const int32_t* jpl_reaction;  /* [nJPL] */
  const double* jpl_param;      /* [nJPL][7]: k0_A, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc */
  int32_t nRJPL;
  const int32_t* rjpl_reaction; /* [nRJPL] */
  const double* rjpl_param;     /* [nRJPL][10]: k0_A, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc, A, B, C */
  int32_t nAdjust;
  const int32_t* adjust_pair;   /* [nAdjust][2]: reaction, species; applied in this order */
  int32_t nProdO1D;
  const int32_t* o1d_index;     /* [nProdO1D][7]: reactions 1..3, photolysis reaction, species 1..3 */
  const double* o1d_param;      /* [nProdO1D][6]: A1, C1, A2, C2, A3, C3 */
} tchem_gb_e3sm_view;

/* Per-sample work counters of one time-advance call (the algorithmic-work inputs of the
 * roofline: flops = n_lu*(2/3)m^3 + n_solve*2m^2 + n_jac*F_jac + n_rhs*F_rhs). */
typedef struct tchem_gb_sample_stats {
  int32_t n_steps;       /* accepted steps */
  int32_t n_rejected;    /* step attempts rejected by the error test */
  int32_t n_newton_fail; /* step attempts abandoned because Newton did not converge */
  int32_t n_newton_iter; /* Newton iterations, both stages */
  int32_t n_lu;          /* LU factorizations */
  int32_t n_solve;       /* forward+backward solve pairs (Newton updates and error filter) */
  int32_t n_rhs;         /* right-hand-side evaluations */
  int32_t n_jac;         /* Jacobian evaluations */
} tchem_gb_sample_stats;

typedef struct tchem_gb_mech tchem_gb_mech; /* opaque */

const char* tchem_gb_last_error(void);
int tchem_gb_abi_version(void);

/* Parses an NCAR-format YAML file. When echo_path is non-NULL the mechanism echo
 * (the reference's kmod.echo format) is written there. */
int tchem_gb_mech_create_from_file(const char* yaml_path, const char* echo_path, tchem_gb_mech** out);
int tchem_gb_mech_create_from_string(const char* yaml_text, tchem_gb_mech** out);
void tchem_gb_mech_destroy(tchem_gb_mech* mech);
int tchem_gb_mech_host_view(const tchem_gb_mech* mech, tchem_gb_kmcd_view* view);
int tchem_gb_mech_e3sm_view(const tchem_gb_mech* mech, tchem_gb_e3sm_view* view);
/* Copies species name i (truncated as the reference stores it) into buf. */
int tchem_gb_mech_species_name(const tchem_gb_mech* mech, int i, char* buf, int buflen);
/* The static-order sparse LU of the mechanism's Newton matrix (no counterpart in the reference,
 * whose Tines solve factors the dense matrix with partial pivoting): the elimination program the
 * full-Newton FP32 form's one-warp shape runs for 33 to 128 active species. info[12] receives
 * m, nnz (entries of the filled pattern), n_ops (trailing updates), prog_len and the offsets
 * (int32 units into prog) of diag[m], pos[m], lc_ptr[m+1], lc[], uc_ptr[m+1], uc[], up_ptr[m+1]
 * and up[2 n_ops]: pos[s] is the elimination position of species s; diag[k] the entry of (k, k);
 * lc / uc list column k of L below / U above the diagonal as entry | row << 16; up holds step k's
 * updates as pairs (dst | l << 16, u): a[dst] -= a[l] * a[u]. Entries number the filled pattern
 * row-major in position order. prog (may be NULL) receives min(prog_cap, prog_len) values.
 * TCHEM_GB_ERR_UNSUPPORTED for mechanisms above 128 active species. */
int tchem_gb_mech_sparse_lu(const tchem_gb_mech* mech, int32_t* info, int32_t* prog, int prog_cap);

/* Scenario file -> state[nbatch][nSpec+3] on the host ([rho, p, T, x...]). */
int tchem_gb_scenario_batch_size(const char* yaml_path, int* nbatch);
int tchem_gb_scenario_read(const char* yaml_path, const tchem_gb_mech* mech, double* state_host, int nbatch);
/* Scenario file -> photolysis rates photo_host[nbatch][*n_photo] from photolysis_rates.r_0 ..
 * r_{n_photo-1} (host; *n_photo = 0 without that section; photo_host may be NULL to query
 * *n_photo). Every list must hold nbatch values. */
int tchem_gb_scenario_photolysis_rates(const char* yaml_path, int nbatch, double* photo_host, int* n_photo);
/* Scenario file -> external sources ext_host[nbatch][m] (host; zero where the file's
 * external_forcing section names no source); *count = the number of forcing entries. */
int tchem_gb_scenario_external_forcing(const char* yaml_path, const tchem_gb_mech* mech, int nbatch,
                                       double* ext_host, int* count);

/* ---- Aerosol model (SIMPOL.1 gas-particle phase transfer) -----------------------------------
 * TChem::AerosolModelData (src/core/TChem_AerosolModelData.hpp:30-80,
 * src/core/TChem_AerosolModelData.cpp:60-303) over a parsed gas mechanism. The aerosol problem's
 * ODE vector is [active gas species, particle 0's aerosol species, particle 1's, ...]
 * (src/core/TChem_AerosolChemistry.cpp:116-131); its state row is [rho, p, T, active gas,
 * constant gas, particles]. */
typedef struct tchem_gb_aero tchem_gb_aero; /* opaque */
typedef struct tchem_gb_aero_view {
  int32_t nSpec;          /* aerosol species per particle */
  int32_t nSpec_gas;      /* active gas species */
  int32_t nConstSpec_gas; /* constant gas species */
  int32_t nParticles;     /* computational particles */
  int32_t nSimpol;        /* SIMPOL_PHASE_TRANSFER entries */
  const double* molecular_weights; /* [nSpec] kg/mol */
  const double* aerosol_density;   /* [nSpec] kg/m3 */
  const double* aerosol_kappa;     /* [nSpec] */
  const int32_t* simpol_index;     /* [nSimpol][3]: aerosol index in the ODE vector (particle 0), gas
                                      index, compute_alpha (1: alpha from N star, 0: alpha = 0.1) */
  const double* simpol_param;      /* [nSimpol][7]: B1, B2, B3, B4, diffusion coeff [m2/s], N star,
                                      gas molecular weight [kg/mol] */
} tchem_gb_aero_view;
int tchem_gb_aero_create_from_file(const char* yaml_path, const tchem_gb_mech* gas, tchem_gb_aero** out);
int tchem_gb_aero_create_from_string(const char* yaml_text, const tchem_gb_mech* gas, tchem_gb_aero** out);
void tchem_gb_aero_destroy(tchem_gb_aero* aero);
int tchem_gb_aero_host_view(const tchem_gb_aero* aero, tchem_gb_aero_view* view);
/* AerosolModelData::setNumberofParticles (src/core/TChem_AerosolModelData.cpp:245-254). */
int tchem_gb_aero_set_number_of_particles(tchem_gb_aero* aero, int n_particles);
int tchem_gb_aero_species_name(const tchem_gb_aero* aero, int i, char* buf, int buflen);
/* AerosolModelData::scenarioConditionParticles (src/core/TChem_AerosolModelData.cpp:256-300):
 * num_conc[nbatch][nParticles] and the particle part of state rows of width dim (host arrays);
 * *found = 0 when the file has no particles section (nothing written). */
int tchem_gb_aero_scenario_particles(const char* yaml_path, const tchem_gb_aero* aero, int nbatch, double* num_conc,
                                     double* state, int dim, int* found);

/* Numerical form of the time advance. */
enum tchem_gb_form {
  TCHEM_GB_FORM_PLAIN_FP64 = 0, /* FP64 Newton LU: the parity form */
  /* The reference's full Newton with FP32 linear algebra -- an LU (one warp per sample,
     threads_per_sample = 32: dense with partial pivoting up to 32 species, the static-order sparse
     LU of tchem_gb_mech_sparse_lu from 33 to 128) or a Gauss-Jordan inverse (two or four warps per
     sample, threads_per_sample = 64 or 128) -- and one sweep of
     iterative refinement per Newton solve (FP64 residual of the linear system with the FP64
     Jacobian, FP32 correction); FP64 Newton residual, state and error control: follows the FP64
     form's Newton iterates. */
  TCHEM_GB_FORM_MIXED = 1,
  /* Simplified Newton with an FP32 Gauss-Jordan inverse of I - c J: the inverse is carried from
     the previous step's error filter while c changed by at most 30% (else formed at the first
     iterate) and reused by every Newton iteration of both stages; it is re-formed once per stage
     when the correction shrinks by less than half. Newton stops when every component of the FP64
     correction satisfies |dx_i| <= atol/sqrt(m) + rtol |y_i| (tol_newton), which implies the
     reference's 2-norm test. Stage guesses: the quadratic through the last step's y_n,
     y_{n+gamma}, y_{n+1} (stage 1) and the quadratic through y_n, f_n, y_{n+gamma} (stage 2). The
     local-error filter uses a fresh inverse of I - c J(y_{n+1}), the matrix of the reference's
     last Newton iteration, so the step-size sequence follows the FP64 form. jacobian_interval is
     not used. */
  TCHEM_GB_FORM_MIXED_SIMPLIFIED = 2
};

typedef struct tchem_gb_advance_opts {
  int32_t form;               /* tchem_gb_form */
  int32_t threads_per_sample; /* mixed forms: 32, 64 or 128 threads (1, 2 or 4 warps) per sample;
                                 0: the mechanism's tuned preference (tchem_gb_autotune), else the
                                 narrowest kernel shape for its size */
  int32_t reserved[6];        /* zero */
} tchem_gb_advance_opts;

/* Device workspace (bytes) a tchem_gb_time_advance call with these arguments needs. */
size_t tchem_gb_workspace_bytes(const tchem_gb_mech* const* mechs, int n_mechs, int nbatch,
                                const tchem_gb_advance_opts* opts);

/* Batched TR-BDF2 time advance of box-model samples on the current CUDA device.
 * All array arguments are device pointers:
 *   mechs[n_mechs]     host array of mechanism handles; mech_of_sample[nbatch] selects one per
 *                      sample (NULL: every sample uses mechs[0]) -- the kmcds overload of the
 *                      reference; samples of structurally identical mechanisms share a launch.
 *   tol_newton[2]      Newton {atol, rtol}; tol_time[m_max][2] per-species {atol, rtol}.
 *   fac                ignored (the Jacobian is analytic); may be NULL.
 *   tadv[nbatch]       per-sample time-advance controls.
 *   state[nbatch][nSpec+3] in; state_out may alias state. t_out is read (samples with
 *                      t_out >= tend are skipped, as the reference does) and written.
 *   status[nbatch]     tchem_gb_sample_status; stats[nbatch] optional work counters.
 *   workspace          device scratch of tchem_gb_workspace_bytes() bytes, or NULL to use a
 *                      library-owned cached allocation (not usable inside stream capture). A
 *                      caller-owned workspace must be zero-filled before its first use: its header
 *                      holds the device error word, which persists across calls until
 *                      tchem_gb_device_error reads and clears it.
 * Stream-ordered and asynchronous. */
int tchem_gb_time_advance(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                          const double* tol_newton, const double* tol_time, const double* fac,
                          const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                          double* state_out, int32_t* status, tchem_gb_sample_stats* stats, void* workspace,
                          size_t workspace_bytes, const tchem_gb_advance_opts* opts, void* stream);

/* Same computation on HOST arrays: copies in, advances, copies out and synchronizes the stream
 * (the runHostBatch-style entry point for callers without device memory of their own). */
int tchem_gb_time_advance_hostbuf(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample,
                                  int nbatch, const double* tol_newton, const double* tol_time,
                                  const tchem_gb_tadv* tadv, const double* state, double* t_out,
                                  double* dt_out, double* state_out, int32_t* status, tchem_gb_sample_stats* stats,
                                  const tchem_gb_advance_opts* opts, void* stream);

/* tchem_gb_time_advance for callers that may not allocate device memory (no counterpart in the
 * reference): a host model that owns every device allocation through its own pool, or a loop
 * where cudaMalloc/cudaFree would synchronise the device. Same arguments as
 * tchem_gb_time_advance without the workspace: the work-queue scratch is a fixed 1 MiB array
 * inside the library (held by every device context that loads it). The mechanisms' device tables
 * must already exist on the current device (call tchem_gb_workspace_bytes with them once at
 * set-up); calls needing more scratch than 1 MiB (batches mixing mechanism structures need 4 bytes
 * per sample and group) are rejected with TCHEM_GB_ERR_ARG; a mechanism outside the path gives
 * TCHEM_GB_ERR_UNSUPPORTED, as tchem_gb_time_advance does. That set-up call also looks up the
 * array's device address, which loads the module holding it (and so places its 1 MiB) on the
 * current device; without it, the first call of this entry point on a device does the lookup
 * itself and may allocate then. CUDA also places a kernel's code on the device at its first
 * launch (lazy module loading, the default): callers that must see no allocation at all include one
 * tchem_gb_time_advance call with the same mechanisms and form in their set-up (or run with
 * CUDA_MODULE_LOADING=EAGER). Make the set-up calls before any stream capture. All calls share
 * the array: calls that overlap on the GPU race and must be serialised. Device-side wait timeouts
 * are not reported through tchem_gb_device_error; samples no kernel reached keep the caller's
 * status value. */
int tchem_gb_time_advance_noalloc(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample,
                                  int nbatch, const double* tol_newton, const double* tol_time, const double* fac,
                                  const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                                  double* state_out, int32_t* status, tchem_gb_sample_stats* stats,
                                  const tchem_gb_advance_opts* opts, void* stream);

/* ---- Discrete adjoint (plain FP64 form, one mechanism) ------------------------------------
 * No counterpart in the reference (its TR-BDF2 has no adjoint); these extend runDeviceBatch
 * (src/core/TChem_AtmosphericChemistry.hpp:83-105) with the trajectory record and the
 * vector-Jacobian product of the end state.
 *
 * tchem_gb_time_advance_record: tchem_gb_time_advance in the plain FP64 form, one mechanism,
 * that also records per sample the accepted step sizes tape_dt[nbatch][tape_cap], the state of
 * the active species at the start of steps 0, 32, 64, ... in
 * tape_ckpt[nbatch][tape_cap/32 + 1][m], and the step count tape_nsteps[nbatch]. A sample that
 * needs more than tape_cap steps ends with status TCHEM_GB_SAMPLE_TAPE_FULL. k_scale[nReac]
 * (device, optional) multiplies each reaction's rate constant (exp(theta_r)). */
int tchem_gb_time_advance_record(const tchem_gb_mech* mech, int nbatch, const double* tol_newton,
                                 const double* tol_time, const double* k_scale, const tchem_gb_tadv* tadv,
                                 const double* state, double* t_out, double* dt_out, double* state_out,
                                 int32_t* status, tchem_gb_sample_stats* stats, double* tape_dt, double* tape_ckpt,
                                 int32_t* tape_nsteps, int tape_cap, void* stream);

/* Device workspace (bytes) of tchem_gb_adjoint for nbatch samples. */
size_t tchem_gb_adjoint_workspace_bytes(const tchem_gb_mech* mech, int nbatch);

/* Discrete adjoint of a recorded run: given lambda[nbatch][m] = dL/dy(t_end) for the active
 * species, writes grad_x0[nbatch][m] = dL/dy(t_0) and grad_k[nbatch][nReac] = dL/dtheta_r, where
 * exp(theta_r) multiplies reaction r's rate constant (so theta_r is the log of its
 * pre-exponential factors). The step sequence is the recorded one; state, tadv, tol_newton and
 * k_scale must be those of the recording call. status[nbatch] as for the time advance. */
int tchem_gb_adjoint(const tchem_gb_mech* mech, int nbatch, const double* tol_newton, const double* k_scale,
                     const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const double* tape_ckpt,
                     const int32_t* tape_nsteps, int tape_cap, const double* lambda, double* grad_x0, double* grad_k,
                     int32_t* status, void* workspace, size_t workspace_bytes, void* stream);

/* Autotuner (no counterpart in the reference, whose team sizes are fixed at launch): times the
 * form's kernel shapes (32, 64 and 128 threads per sample, where a shape exists for the
 * mechanism's size) on a probe batch of device arrays laid out as for tchem_gb_time_advance
 * (t_out is zeroed before every trial: the probe starts at t = 0; workspace may be NULL), keeps the
 * fastest as the mechanism's preference for calls with opts.threads_per_sample == 0, and returns
 * it in *chosen; ms_per_candidate[3] (optional) receives each trial's time (-1: not run).
 * Synchronizes the stream. tchem_gb_mech_set_threads_per_sample sets the preference directly
 * (0: the narrowest shape). */
int tchem_gb_autotune(tchem_gb_mech* mech, int form, int nbatch, const double* tol_newton, const double* tol_time,
                      const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                      double* state_out, int32_t* status, void* workspace, size_t workspace_bytes, void* stream,
                      int* chosen, float* ms_per_candidate);
int tchem_gb_mech_set_threads_per_sample(tchem_gb_mech* mech, int form, int threads_per_sample);

/* Synchronizes `stream`, then reads and clears the device error word of `workspace` (NULL: the
 * library-owned workspace). *device_error is 0 when no kernel reported a timed-out wait; bit 0
 * (1): a bounded wait expired; bit 1 (2): a tensor-core kernel's MMAs had not completed when it
 * released its tensor memory. */
int tchem_gb_device_error(void* workspace, void* stream, int32_t* device_error);

/* The carry-over step of the reference's host time loop between two tchem_gb_time_advance calls
 * (the parallel_reduce of src/examples/TChem_AtmosphericChemistry.cpp:340-350): for every sample
 * tadv[i].tbeg = t_out[i] and tadv[i].dt = dt_out[i]; when iters_per_interval > 0 it also sets
 * tadv[i].num_time_iterations_per_interval (the step budget of the next call); when t_sum is not
 * NULL, *t_sum = sum of t_out (the loop's stopping test is mean t >= 0.9999 tend). Device arrays,
 * stream-ordered, one kernel launch. */
int tchem_gb_time_advance_carry_over(tchem_gb_tadv* tadv, const double* t_out, const double* dt_out, int nbatch,
                                     int iters_per_interval, double* t_sum, void* stream);

/* Number of kernels the library has launched in this process (every entry point counts each
 * launch it made). No counterpart in the reference; for benchmarks and tests. */
long long tchem_gb_kernel_launches(void);

/* Unit entry points on device arrays (state[nbatch][nSpec+3]):
 *   kfor[nbatch][nReac] rate constants, omega[nbatch][m] net production rates (active species),
 *   jac[nbatch][m][m] d omega / d x (row-major). All mechanisms must share one structure. */
int tchem_gb_kforward(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                      const double* state, double* kfor, void* stream);
int tchem_gb_reaction_rates(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample,
                            int nbatch, const double* state, double* omega, void* stream);
int tchem_gb_jacobian(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                      const double* state, double* jac, void* stream);

/* ---- E3SM gas chemistry: photolysis rates and external sources as per-sample inputs ---------
 * TChem::AtmosphericChemistryE3SM::runDeviceBatch (src/core/TChem_AtmosphericChemistryE3SM.hpp:88-104,
 * src/core/TChem_AtmosphericChemistryE3SM.cpp:42-167) and the RHS-only batch APIs
 * ReactionRates, RateofProgress and NetProductionRates (src/core/TChem_ReactionRates.hpp:59-72,
 * src/core/TChem_RateofProgress.hpp:60-75, src/core/TChem_NetProductionRates.hpp:61-78), one
 * mechanism per call, device arrays, stream-ordered. The rate constants follow the E3SM forms:
 * ARRHENIUS and TROE without the ppm conversion factor, CMAQ_H2O2 with it
 * (src/core/impl/TChem_Impl_KForward.hpp:44-147), JPL and R_JPL_ARRHENIUS with [M] = x(M)
 * (src/core/impl/TChem_Impl_KForwardJPL.hpp:45-147), then the adjust_reaction factors in file
 * order and the prod_O1D modifier (src/core/impl/TChem_Impl_AdjustReactions.hpp:45-100).
 * Reactions 0 .. n_photo-1 without one of those rate types take photo_rates[s][r]
 * (src/core/impl/TChem_Impl_RateofProgress.hpp:70-80); reactions with neither are 0. The net
 * production rates of the active species start from external_sources[s][k]
 * (src/core/impl/TChem_Impl_NetProductionRates.hpp:52-112). photo_rates (with n_photo = 0) and
 * external_sources may be NULL (no photolysis input, zero sources).
 *   kfor[nbatch][nReac], rop[nbatch][nReac], omega[nbatch][m] (active species). */
int tchem_gb_e3sm_reaction_rates(const tchem_gb_mech* mech, int nbatch, const double* state,
                                 const double* photo_rates, int n_photo, double* kfor, void* stream);
int tchem_gb_e3sm_rate_of_progress(const tchem_gb_mech* mech, int nbatch, const double* state,
                                   const double* photo_rates, int n_photo, double* rop, void* stream);
int tchem_gb_e3sm_net_production_rates(const tchem_gb_mech* mech, int nbatch, const double* state,
                                       const double* photo_rates, int n_photo, const double* external_sources,
                                       double* omega, void* stream);
/* E3SM time advance: tchem_gb_time_advance for one mechanism with the per-sample inputs
 * photo_rates[nbatch][n_photo] and external_sources[nbatch][m], in any of the three forms. The
 * rate constants are evaluated once per sample, so the species that scale them ([M] of the JPL
 * forms, the adjust_reaction and prod_O1D species) must be constant species
 * (TCHEM_GB_ERR_UNSUPPORTED otherwise; the E3SM mechanisms keep M, N2, O2 and H2O constant).
 * The workspace also holds the per-sample rate constants: tchem_gb_e3sm_workspace_bytes. */
size_t tchem_gb_e3sm_workspace_bytes(const tchem_gb_mech* mech, int nbatch, const tchem_gb_advance_opts* opts);
int tchem_gb_e3sm_time_advance(const tchem_gb_mech* mech, int nbatch, const double* tol_newton,
                               const double* tol_time, const double* fac, const tchem_gb_tadv* tadv,
                               const double* state, const double* photo_rates, int n_photo,
                               const double* external_sources, double* t_out, double* dt_out, double* state_out,
                               int32_t* status, tchem_gb_sample_stats* stats, void* workspace,
                               size_t workspace_bytes, const tchem_gb_advance_opts* opts, void* stream);

/* ---- Gas-aerosol chemistry (SIMPOL.1 phase transfer): time advance and RHS --------------------
 * TChem::AerosolChemistry::runDeviceBatch (src/core/TChem_AerosolChemistry.hpp:87-103,
 * src/core/TChem_AerosolChemistry.cpp:30-172, 236-260): TR-BDF2 on the ODE vector [active gas,
 * particle 0's aerosol species, particle 1's, ...] of M = m + nParticles * nSpec entries, with one
 * gas mechanism (box-model rate forms) and one aerosol model per call; plain FP64 form, one warp
 * per sample, device arrays, stream-ordered.
 *   tol_time[M][2]; number_conc[nbatch][nParticles]; state and state_out rows [rho, p, T, active
 *   gas, constant gas, particles] of width 3 + nSpec + nParticles * nSpec_aerosol (may alias).
 * The Newton Jacobian is a forward difference of the RHS, column j with the step
 * 1e-8 max(|y_j|, 1e-20) (the reference's computeJacobian); fac, the reference's per-sample
 * difference factors, may be NULL and is not read. rho, p, T and the constant gas species are
 * copied through. Refused with TCHEM_GB_ERR_UNSUPPORTED: a SIMPOL entry whose gas species is a
 * constant species, M above 320, or rate forms outside the box model's. The workspace holds the
 * work queue, the device error word (tchem_gb_device_error) and, for large M, the Newton
 * matrices: tchem_gb_aero_workspace_bytes (NULL workspace: library-owned). */
size_t tchem_gb_aero_workspace_bytes(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch);
int tchem_gb_aero_time_advance(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch,
                               const double* tol_newton, const double* tol_time, const double* fac,
                               const tchem_gb_tadv* tadv, const double* state, const double* number_conc,
                               double* t_out, double* dt_out, double* state_out, int32_t* status,
                               tchem_gb_sample_stats* stats, void* workspace, size_t workspace_bytes, void* stream);
/* Aerosol RHS (src/core/impl/TChem_Impl_Aerosol_RHS.hpp:57-100) at each sample's state row:
 * omega[nbatch][M] in ODE-vector order. */
int tchem_gb_aero_rhs(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch, const double* state,
                      const double* number_conc, double* omega, void* stream);

/* Solver settings file of the host-model driver interface (TChem::Driver::createNumerics,
 * src/core/TChem_Driver.cpp:152-187): the solver_info mapping of a YAML file with the reference's
 * keys and defaults (a key that is absent or does not convert takes its default): atol_newton
 * 1e-10, rtol_newton 1e-6, dtmin 1e-8, atol_time 1e-12, rtol_time 1e-4, max_newton_iterations
 * 100, max_num_time_iterations 1000, team_size -1, vector_size -1, verbose false. */
typedef struct tchem_gb_numerics {
  double atol_newton, rtol_newton, dtmin, atol_time, rtol_time;
  int32_t max_newton_iterations, max_num_time_iterations, team_size, vector_size, verbose;
} tchem_gb_numerics;
int tchem_gb_numerics_read(const char* yaml_path, tchem_gb_numerics* out);

/* Tensor-core building block of the 300-species factorization (no counterpart in the reference):
 * for each of ntiles tiles, D[128][N] -= A[128][32] * B[32][N] with TF32 operands and FP32
 * accumulation on the 5th-generation tensor cores (tcgen05.mma kind::tf32, accumulator in TMEM),
 * the trailing update of a blocked LU with 32-column panels. Row-major FP32 device arrays, tile t
 * at A + t*128*32, B + t*32*N, D + t*128*N; N a multiple of 16 in [16, 256]. Bounded waits report
 * through tchem_gb_device_error. Validation on a GPU is pending. */
int tchem_gb_tc_tile_update_tf32(int ntiles, int N, const float* A, const float* B, float* D, void* stream);
/* Blocked FP32 LU with partial pivoting of nbatch matrices A[b][m][lda] (row-major, in place),
 * one CTA per matrix: 32-column panels on the CUDA cores (pivot: first largest magnitude in the
 * current row order, whole-row swaps; piv[b][k] = the row swapped with row k), U12 = L11^-1 A12 on
 * the CUDA cores, and the trailing update A22 -= L21 U12 on the tensor cores (TF32 operands, FP32
 * accumulation in TMEM, tiles of 128 rows x up to 256 columns). info[b] = 0, k + 1 when column k
 * has no usable pivot, -1 when a bounded wait expired. Device arrays; validation on a GPU is
 * pending. */
int tchem_gb_tc_lu_factor_tf32(int nbatch, int m, int lda, float* A, int32_t* piv, int32_t* info, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TCHEM_GB_H */
