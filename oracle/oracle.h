/*
 * CPU oracle for the batched box-model TR-BDF2 time advance.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the GPU engine's accuracy reference: it is loaded by
 * the tests, by the smoke check and by the CPU-baseline leg of bench.py, and by nothing on
 * the product path. It is a plain FP64 C++ restatement of the reference algorithm:
 *   rate constants   src/core/impl/TChem_Impl_KForwardAerosol.hpp:44-145
 *   RHS              src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:57-143, 238-289
 *   problem          src/core/problems/TChem_Impl_AtmosphericChemistry_Problem.hpp:64-81, 127-143
 *   batch driver     src/core/TChem_AtmosphericChemistry.cpp:42-167 (skip samples at t_end,
 *                    T, p, rho copied through)
 *   integrator       TR-BDF2 of Bank et al. (IEEE Trans. Electron Devices 32(10), 1985) with the
 *                    error estimate of Hosea & Shampine (Appl. Numer. Math. 20, 1996). The
 *                    reference's integrator (Tines TimeIntegratorTrBDF2) is an external
 *                    dependency absent from the source tree; the restatement keeps its call
 *                    interface (src/core/problems/TChem_Impl_AtmosphericChemistry.hpp:138-155)
 *                    and the behaviour the reference's own outputs pin: dt doubles per accepted
 *                    step while the error is negligible, is capped by dt_max, the last step lands
 *                    exactly on t_end and dt_out is 0 there
 *                    (src/unit-tests/CB05CL_AE5/references/full_gas.hdf5,
 *                    src/examples/runs/atmospheric_chemistry/Emission/Emissions.dat); Newton
 *                    failure halves dt up to 4 times, then the sample fails with state 0,
 *                    t_out = t_end, dt_out = -1 (src/core/impl/TChem_Impl_TimeIntegratorImplicitEuler.hpp:246-305).
 * The Jacobian is analytic (the reference uses forward differences or Sacado AD; both give
 * the same matrix to rounding, and the Newton fixed point does not depend on it). Newton stops when
 * ||dx|| <= atol + rtol ||y|| (2-norms); where a few huge entries dominate ||y|| (the aerosol number
 * concentrations of the E3SM uci_col scenario) that ends most stages after one iteration, so the
 * end state then depends on the stage guesses (oracle_set_newton_min_iterations makes it iterate).
 */
#ifndef TCHEM_GB_ORACLE_H
#define TCHEM_GB_ORACLE_H

#include "../include/tchem_gb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FP32 factorizations (lu_fp32 >= 1 below) as a tensor-core factorization computes them: 32-column
 * panels in FP32 and the trailing update with operands rounded to `bits` mantissa bits (10: TF32,
 * 7: BF16) and FP32 accumulation; 0 (default): the unblocked FP32 LU. A process-wide setting. */
int oracle_set_lu_tile_bits(int bits);
/* FP32 factorizations of n x n Newton matrices in a static symmetric order without pivoting, as a
 * sparse factorization computes them: row and column k are species order[k]; the substitutions are
 * column-oriented with the pivots' reciprocals. n = 0 restores partial pivoting. Process-wide. */
int oracle_set_lu_static_order(int n, const int32_t* order);
/* Full-Newton integrator test settings (process-wide): at least k Newton iterations per stage
 * before the convergence test may end it (1: the default), and an imposed sequence of accepted step
 * sizes dt[n] (step k takes dt[min(k, n - 1)], clipped to t_end as usual; the error estimate is not
 * used; n = 0 restores the error control). A Newton failure still halves the step. */
int oracle_set_newton_min_iterations(int k);
int oracle_set_step_sequence(int n, const double* dt);
/* One FP32 matrix a[n][n] factored as the tensor-core LU does: 32-column panels with partial
 * pivoting, trailing update on operands rounded to `keep` mantissa bits (10: TF32, 23: none);
 * lu[n][n] and piv[n] as LAPACK's sgetrf (0-based pivots). */
int oracle_lu_factor_blocked(int n, const float* a, int keep, float* lu, int32_t* piv);

/* kfor[nReac] for one (T, p). */
int oracle_kforward(const tchem_gb_kmcd_view* km, double T, double p, double* kfor);
/* omega[m] = d x_active / dt for x[nSpec] (constant species last). */
int oracle_reaction_rates(const tchem_gb_kmcd_view* km, double T, double p, const double* x, double* omega);
/* J[m][m] = d omega_i / d x_j (row-major), analytic. */
int oracle_jacobian(const tchem_gb_kmcd_view* km, double T, double p, const double* x, double* J);

/* Batched time advance with the reference's runDeviceBatch semantics on host arrays.
 * kms[n_mechs] with mech_of_sample[nbatch] (NULL: every sample uses kms[0]).
 * lu_fp32 = 0: FP64 Newton LU (the plain form); k >= 1: FP32 LU and solves with FP64 residuals
 * and k - 1 sweeps of iterative refinement of every Newton linear solve (FP64 residual with the
 * FP64 Jacobian, FP32 correction); k = 2 is the engine's mixed form.
 * simplified != 0: the simplified-Newton form of TCHEM_GB_FORM_MIXED_SIMPLIFIED (factors carried
 * across Newton iterations and steps, componentwise Newton test, error filter with I - c J(y_{n+1}));
 * the factors are LU here and a Gauss-Jordan inverse in the engine, which agree to the Newton
 * tolerance.
 * t_out is read (samples with t_out >= tend are skipped) and written.
 * nthreads <= 0 uses all OpenMP threads. stats may be NULL. */
int oracle_time_advance(const tchem_gb_kmcd_view* const* kms, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                        const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                        const double* state, double* t_out, double* dt_out, double* state_out, int32_t* status,
                        tchem_gb_sample_stats* stats, int lu_fp32, int simplified, int nthreads);

/* E3SM gas chemistry (the engine's tchem_gb_e3sm_* entry points), one sample per call for the
 * rates, x[nSpec] (constant species last), photo[n_photo] (NULL: none):
 *   oracle_e3sm_kforward          rate constants: photolysis rates into kfor[0, n_photo), then
 *                                 src/core/impl/TChem_Impl_KForward.hpp:44-147 (ARRHENIUS and TROE
 *                                 without the ppm conversion), TChem_Impl_KForwardJPL.hpp:45-147 and
 *                                 TChem_Impl_AdjustReactions.hpp:45-100, in the order of
 *                                 src/core/impl/TChem_Impl_RateofProgress.hpp:70-80 and
 *                                 TChem_Impl_ReactionRates.hpp:54-79
 *   oracle_e3sm_rate_of_progress  rop[nReac], src/core/impl/TChem_Impl_RateofProgress.hpp:84-98
 *   oracle_e3sm_net_production_rates
 *                                 omega[m] from ext[m] (NULL: zero) plus the stoichiometric sums,
 *                                 src/core/impl/TChem_Impl_NetProductionRates.hpp:52-112
 *   oracle_e3sm_time_advance      oracle_time_advance (one mechanism) with these rates, per-sample
 *                                 photo[nbatch][n_photo] and ext[nbatch][m]; rate constants once per
 *                                 sample (TCHEM_GB_ERR_UNSUPPORTED when an active species scales
 *                                 one, as the engine). */
int oracle_e3sm_kforward(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                         const double* x, const double* photo, int n_photo, double* kfor);
int oracle_e3sm_rate_of_progress(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                                 const double* x, const double* photo, int n_photo, double* rop);
int oracle_e3sm_net_production_rates(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                                     const double* x, const double* photo, int n_photo, const double* ext,
                                     double* omega);
int oracle_e3sm_time_advance(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, int nbatch,
                             const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                             const double* state, const double* photo, int n_photo, const double* ext, double* t_out,
                             double* dt_out, double* state_out, int32_t* status, tchem_gb_sample_stats* stats,
                             int lu_fp32, int simplified, int nthreads);

/* Aerosol chemistry with SIMPOL.1 gas-particle phase transfer (TChem::AerosolChemistry), ODE
 * vector x = [active gas species, particle 0's aerosol species, ...]:
 *   oracle_simpol_rhs     adds entry i_simpol's transfer for every particle to omega
 *                         (src/core/impl/TChem_Impl_SIMPOL_phase_transfer.hpp:60-150 with
 *                         TChem_Impl_SIMPOL_constant.hpp:50-130 and
 *                         TChem_Impl_SingleParticleUtils.hpp:50-170)
 *   oracle_aerosol_rhs    omega = gas RHS (box model, rate constants of KForwardAerosol) + every
 *                         particle's SIMPOL transfers (src/core/impl/TChem_Impl_Aerosol_RHS.hpp:60-105);
 *                         xconst = constant gas species
 *   oracle_aerosol_time_advance  the TR-BDF2 advance of the aerosol problem on state rows
 *                         [rho, p, T, active gas, constant gas, particles] with number_conc[nbatch][nParticles]
 *                         (src/core/TChem_AerosolChemistry.cpp:55-172), forward-difference Jacobian as
 *                         the reference's AerosolChemistry_Problem; tol_time[m_ode][2]. */
int oracle_simpol_rhs(const tchem_gb_aero_view* av, int i_simpol, double T, double p, const double* number_conc,
                      const double* x, double* omega);
int oracle_aerosol_rhs(const tchem_gb_kmcd_view* km, const tchem_gb_aero_view* av, double T, double p,
                       const double* number_conc, const double* x, const double* xconst, double* omega);
int oracle_aerosol_time_advance(const tchem_gb_kmcd_view* km, const tchem_gb_aero_view* av, int nbatch,
                                const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                                const double* state, const double* number_conc, double* t_out, double* dt_out,
                                double* state_out, int32_t* status, tchem_gb_sample_stats* stats, int nthreads);

/* Discrete adjoint of the plain form on a recorded step sequence (the engine's
 * tchem_gb_time_advance_record / tchem_gb_adjoint), restated densely on the CPU, one mechanism:
 *   oracle_time_advance_record: oracle_time_advance (FP64) recording the accepted step sizes
 *     tape_dt[nbatch][tape_cap] and counts tape_nsteps[nbatch]; k_scale[nReac] (optional)
 *     multiplies every rate constant.
 *   oracle_replay: the recorded steps re-run from state (no step-size control); y_end[nbatch][m].
 *   oracle_adjoint: lambda[nbatch][m] = dL/dy_end -> grad_x0 = dL/dy0, grad_k[nbatch][nReac] =
 *     dL/dtheta_r with k_r scaled by exp(theta_r).
 *   oracle_tangent: forward sensitivities dy_end along (dx0[nbatch][m], dtheta[nbatch][nReac]). */
int oracle_time_advance_record(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton,
                               const double* tol_time, const double* k_scale, const tchem_gb_tadv* tadv,
                               const double* state, double* t_out, double* dt_out, double* state_out,
                               int32_t* status, double* tape_dt, int32_t* tape_nsteps, int tape_cap, int nthreads);
int oracle_replay(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                  const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                  int tape_cap, double* y_end, int nthreads);
int oracle_adjoint(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                   const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                   int tape_cap, const double* lambda, double* grad_x0, double* grad_k, int nthreads);
int oracle_tangent(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                   const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                   int tape_cap, const double* dx0, const double* dtheta, double* dy_end, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
