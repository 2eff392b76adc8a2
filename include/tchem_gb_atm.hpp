// C++ face of the engine with the reference's names and argument order
// (TChem::AtmosphericChemistry, src/core/TChem_AtmosphericChemistry.hpp:47-157), over raw device
// pointers instead of Kokkos views. Header-only; link against libtchem_gb.so.
//
//   TChem::AtmosphericChemistry::runDeviceBatch(policy, tol_newton, tol_time, fac, tadv, state,
//                                               t_out, dt_out, state_out, kmcd)
// becomes
//   tchem_gb::AtmosphericChemistry::runDeviceBatch(stream, tol_newton, tol_time, fac, tadv, state,
//                                                  t_out, dt_out, state_out, kmcd, nbatch)
//
// Errors throw std::logic_error, as TCHEM_CHECK_ERROR does in the reference
// (src/core/TChem_Util.hpp:108-114); per-sample failures keep the reference convention
// (dt_out < 0, state_out = 0, t_out = t_end) and are detailed in the optional status array.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "tchem_gb.h"

namespace tchem_gb {

inline void check(int rc, const char* where) {
  if (rc != TCHEM_GB_OK) throw std::logic_error(std::string(where) + ": " + tchem_gb_last_error());
}

// Owning handle of a parsed mechanism (KineticModelData + KineticModelNCAR_ConstData).
class KineticModel {
 public:
  explicit KineticModel(const std::string& yaml_path, const char* echo_path = nullptr) {
    check(tchem_gb_mech_create_from_file(yaml_path.c_str(), echo_path, &m_), "tchem_gb_mech_create_from_file");
  }
  ~KineticModel() { tchem_gb_mech_destroy(m_); }
  KineticModel(const KineticModel&) = delete;
  KineticModel& operator=(const KineticModel&) = delete;
  const tchem_gb_mech* handle() const { return m_; }
  tchem_gb_kmcd_view view() const {
    tchem_gb_kmcd_view v{};
    check(tchem_gb_mech_host_view(m_, &v), "tchem_gb_mech_host_view");
    return v;
  }
  tchem_gb_e3sm_view e3sm_view() const {
    tchem_gb_e3sm_view v{};
    check(tchem_gb_mech_e3sm_view(m_, &v), "tchem_gb_mech_e3sm_view");
    return v;
  }

 private:
  tchem_gb_mech* m_ = nullptr;
};

// Owning handle of a parsed aerosol model (TChem::AerosolModelData over a gas KineticModel, which
// must outlive it).
class AerosolModel {
 public:
  AerosolModel(const std::string& yaml_path, const KineticModel& gas) {
    check(tchem_gb_aero_create_from_file(yaml_path.c_str(), gas.handle(), &a_), "tchem_gb_aero_create_from_file");
  }
  ~AerosolModel() { tchem_gb_aero_destroy(a_); }
  AerosolModel(const AerosolModel&) = delete;
  AerosolModel& operator=(const AerosolModel&) = delete;
  const tchem_gb_aero* handle() const { return a_; }
  tchem_gb_aero_view view() const {
    tchem_gb_aero_view v{};
    check(tchem_gb_aero_host_view(a_, &v), "tchem_gb_aero_host_view");
    return v;
  }
  void setNumberofParticles(int n) { check(tchem_gb_aero_set_number_of_particles(a_, n), "tchem_gb_aero_set_number_of_particles"); }
  // scenarioConditionParticles: num_conc[nbatch][nParticles] and the particle part of state rows
  // of width dim (host arrays); false when the file has no particles section.
  bool scenarioConditionParticles(const std::string& yaml_path, int nbatch, double* num_conc, double* state,
                                  int dim) const {
    int found = 0;
    check(tchem_gb_aero_scenario_particles(yaml_path.c_str(), a_, nbatch, num_conc, state, dim, &found),
          "tchem_gb_aero_scenario_particles");
    return found != 0;
  }

 private:
  tchem_gb_aero* a_ = nullptr;
};

struct AtmosphericChemistry {
  // getWorkSpaceSize(kmcd) for a batch of nbatch samples, in bytes of device memory.
  static size_t getWorkSpaceSize(const KineticModel& kmcd, int nbatch, int form = TCHEM_GB_FORM_PLAIN_FP64) {
    const tchem_gb_mech* h = kmcd.handle();
    tchem_gb_advance_opts o{};
    o.form = form;
    const size_t n = tchem_gb_workspace_bytes(&h, 1, nbatch, &o);
    if (n == 0) check(TCHEM_GB_ERR_ARG, "tchem_gb_workspace_bytes");
    return n;
  }

  // runDeviceBatch with one mechanism for every sample. All arrays are device pointers with the
  // reference's shapes: tol_newton[2], tol_time[m][2], tadv[nbatch], state[nbatch][nSpec+3],
  // t_out/dt_out[nbatch], state_out[nbatch][nSpec+3] (may equal state). fac is accepted and
  // ignored (the Jacobian is analytic).
  static void runDeviceBatch(void* stream, const double* tol_newton, const double* tol_time, const double* fac,
                             const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                             double* state_out, const KineticModel& kmcd, int nbatch, int32_t* status,
                             int form = TCHEM_GB_FORM_PLAIN_FP64, void* workspace = nullptr,
                             size_t workspace_bytes = 0) {
    const tchem_gb_mech* h = kmcd.handle();
    tchem_gb_advance_opts o{};
    o.form = form;
    check(tchem_gb_time_advance(&h, 1, nullptr, nbatch, tol_newton, tol_time, fac, tadv, state, t_out, dt_out,
                                state_out, status, nullptr, workspace, workspace_bytes, &o, stream),
          "tchem_gb_time_advance");
  }

  // The per-sample-mechanism overload (kmcds[B] in the reference): mech_of_sample[nbatch] is a
  // device array of indices into kmcds.
  static void runDeviceBatch(void* stream, const double* tol_newton, const double* tol_time, const double* fac,
                             const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                             double* state_out, const std::vector<const KineticModel*>& kmcds,
                             const int32_t* mech_of_sample, int nbatch, int32_t* status,
                             int form = TCHEM_GB_FORM_PLAIN_FP64) {
    std::vector<const tchem_gb_mech*> hs;
    for (const KineticModel* k : kmcds) hs.push_back(k->handle());
    tchem_gb_advance_opts o{};
    o.form = form;
    check(tchem_gb_time_advance(hs.data(), static_cast<int>(hs.size()), mech_of_sample, nbatch, tol_newton, tol_time,
                                fac, tadv, state, t_out, dt_out, state_out, status, nullptr, nullptr, 0, &o, stream),
          "tchem_gb_time_advance");
  }

  // Autotuner: times the form's kernel shapes on a probe batch (device arrays; t_out is zeroed
  // before every trial) and keeps the fastest as the mechanism's default; returns its threads
  // per sample.
  static int autotune(void* stream, KineticModel& kmcd, int form, int nbatch, const double* tol_newton,
                      const double* tol_time, const tchem_gb_tadv* tadv, const double* state, double* t_out,
                      double* dt_out, double* state_out, int32_t* status) {
    int chosen = 0;
    check(tchem_gb_autotune(const_cast<tchem_gb_mech*>(kmcd.handle()), form, nbatch, tol_newton, tol_time, tadv,
                            state, t_out, dt_out, state_out, status, nullptr, 0, stream, &chosen, nullptr),
          "tchem_gb_autotune");
    return chosen;
  }

  // Discrete adjoint (no counterpart in the reference): a plain FP64 run that records its steps,
  // then dL/dy0 and dL/dtheta (theta_r = log of reaction r's rate-constant scale) from
  // lambda = dL/dy(t_end). tape_dt [nbatch][tape_cap], tape_ckpt [nbatch][tape_cap/32 + 1][m],
  // tape_nsteps [nbatch] are caller-owned device arrays.
  static void recordDeviceBatch(void* stream, const double* tol_newton, const double* tol_time, const double* k_scale,
                                const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                                double* state_out, const KineticModel& kmcd, int nbatch, int32_t* status,
                                double* tape_dt, double* tape_ckpt, int32_t* tape_nsteps, int tape_cap) {
    check(tchem_gb_time_advance_record(kmcd.handle(), nbatch, tol_newton, tol_time, k_scale, tadv, state, t_out, dt_out,
                                       state_out, status, nullptr, tape_dt, tape_ckpt, tape_nsteps, tape_cap, stream),
          "tchem_gb_time_advance_record");
  }
  static void adjointDeviceBatch(void* stream, const double* tol_newton, const double* k_scale,
                                 const tchem_gb_tadv* tadv, const double* state, const KineticModel& kmcd, int nbatch,
                                 const double* tape_dt, const double* tape_ckpt, const int32_t* tape_nsteps,
                                 int tape_cap, const double* lambda, double* grad_x0, double* grad_k, int32_t* status) {
    check(tchem_gb_adjoint(kmcd.handle(), nbatch, tol_newton, k_scale, tadv, state, tape_dt, tape_ckpt, tape_nsteps,
                           tape_cap, lambda, grad_x0, grad_k, status, nullptr, 0, stream),
          "tchem_gb_adjoint");
  }

  // runHostBatch: host arrays, synchronous.
  static void runHostBatch(const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                           const double* state, double* t_out, double* dt_out, double* state_out,
                           const KineticModel& kmcd, int nbatch, int32_t* status,
                           int form = TCHEM_GB_FORM_PLAIN_FP64) {
    const tchem_gb_mech* h = kmcd.handle();
    tchem_gb_advance_opts o{};
    o.form = form;
    check(tchem_gb_time_advance_hostbuf(&h, 1, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out,
                                        state_out, status, nullptr, &o, nullptr),
          "tchem_gb_time_advance_hostbuf");
  }
};

// E3SM gas chemistry (TChem::AtmosphericChemistryE3SM, src/core/TChem_AtmosphericChemistryE3SM.hpp:47-104):
// runDeviceBatch with the per-sample photo_rates[nbatch][n_photo] and external_sources[nbatch][m]
// (either may be null). The rate constants are evaluated once per sample: [M], the adjust_reaction
// and prod_O1D species must be constant species.
struct AtmosphericChemistryE3SM {
  static size_t getWorkSpaceSize(const KineticModel& kmcd, int nbatch, int form = TCHEM_GB_FORM_PLAIN_FP64) {
    tchem_gb_advance_opts o{};
    o.form = form;
    const size_t n = tchem_gb_e3sm_workspace_bytes(kmcd.handle(), nbatch, &o);
    if (n == 0) check(TCHEM_GB_ERR_ARG, "tchem_gb_e3sm_workspace_bytes");
    return n;
  }
  static void runDeviceBatch(void* stream, const double* tol_newton, const double* tol_time, const double* fac,
                             const tchem_gb_tadv* tadv, const double* state, const double* photo_rates, int n_photo,
                             const double* external_sources, double* t_out, double* dt_out, double* state_out,
                             const KineticModel& kmcd, int nbatch, int32_t* status,
                             int form = TCHEM_GB_FORM_PLAIN_FP64, void* workspace = nullptr,
                             size_t workspace_bytes = 0) {
    tchem_gb_advance_opts o{};
    o.form = form;
    check(tchem_gb_e3sm_time_advance(kmcd.handle(), nbatch, tol_newton, tol_time, fac, tadv, state, photo_rates,
                                     n_photo, external_sources, t_out, dt_out, state_out, status, nullptr, workspace,
                                     workspace_bytes, &o, stream),
          "tchem_gb_e3sm_time_advance");
  }
};

// RHS-only batch APIs of the E3SM chemistry (src/core/TChem_ReactionRates.hpp:59-72,
// src/core/TChem_RateofProgress.hpp:60-75, src/core/TChem_NetProductionRates.hpp:61-78); device
// arrays: kfwd and rate_of_progress [nbatch][nReac], net_production_rates [nbatch][m].
struct ReactionRates {
  static void runDeviceBatch(void* stream, const double* state, double* kfwd, const KineticModel& kmcd, int nbatch,
                             const double* photo_rates = nullptr, int n_photo = 0) {
    check(tchem_gb_e3sm_reaction_rates(kmcd.handle(), nbatch, state, photo_rates, n_photo, kfwd, stream),
          "tchem_gb_e3sm_reaction_rates");
  }
};

struct RateofProgress {
  static void runDeviceBatch(void* stream, const double* state, const double* photo_rates, int n_photo,
                             double* rate_of_progress, const KineticModel& kmcd, int nbatch) {
    check(tchem_gb_e3sm_rate_of_progress(kmcd.handle(), nbatch, state, photo_rates, n_photo, rate_of_progress, stream),
          "tchem_gb_e3sm_rate_of_progress");
  }
};

struct NetProductionRates {
  static void runDeviceBatch(void* stream, const double* state, const double* photo_rates, int n_photo,
                             const double* external_sources, double* net_production_rates, const KineticModel& kmcd,
                             int nbatch) {
    check(tchem_gb_e3sm_net_production_rates(kmcd.handle(), nbatch, state, photo_rates, n_photo, external_sources,
                                             net_production_rates, stream),
          "tchem_gb_e3sm_net_production_rates");
  }
};

// Gas-aerosol (SIMPOL.1) time advance (TChem::AerosolChemistry, src/core/TChem_AerosolChemistry.hpp:51-103);
// device arrays: tol_time[M][2], number_conc[nbatch][nParticles], state rows [rho, p, T, gas,
// particles]; fac is not read.
struct AerosolChemistry {
  static size_t getWorkSpaceSize(const KineticModel& kmcd, const AerosolModel& amcd, int nbatch) {
    const size_t n = tchem_gb_aero_workspace_bytes(kmcd.handle(), amcd.handle(), nbatch);
    if (n == 0) check(TCHEM_GB_ERR_ARG, "tchem_gb_aero_workspace_bytes");
    return n;
  }
  static void runDeviceBatch(void* stream, const double* tol_newton, const double* tol_time, const double* fac,
                             const tchem_gb_tadv* tadv, const double* state, const double* number_conc,
                             double* t_out, double* dt_out, double* state_out, const KineticModel& kmcd,
                             const AerosolModel& amcd, int nbatch, int32_t* status, void* workspace = nullptr,
                             size_t workspace_bytes = 0) {
    check(tchem_gb_aero_time_advance(kmcd.handle(), amcd.handle(), nbatch, tol_newton, tol_time, fac, tadv, state,
                                     number_conc, t_out, dt_out, state_out, status, nullptr, workspace,
                                     workspace_bytes, stream),
          "tchem_gb_aero_time_advance");
  }
};

}  // namespace tchem_gb
