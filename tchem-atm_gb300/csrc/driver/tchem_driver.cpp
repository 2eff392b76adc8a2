// Host-model driver interface (libtchem_gb_driver.so): the reference's TChem::Driver and its
// extern "C" functions (src/core/TChem_Driver.hpp:28-132, src/core/TChem_Driver.cpp:88-640) over
// the engine's C ABI. The state and number-concentration rows live on the host, as the
// reference's do; TChem_doTimestep copies them to the device, runs the gas-aerosol TR-BDF2 kernel
// (tchem_gb_aero_time_advance) and copies them back. Device buffers are allocated on the first
// time step and kept until finalize().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/tchem_gb.h"
#include "../../../include/tchem_gb_driver.h"

namespace {

void check(int rc, const char* where) {
  if (rc != TCHEM_GB_OK) throw std::runtime_error(std::string(where) + ": " + tchem_gb_last_error());
}

void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

struct Driver {
  tchem_gb_mech* mech = nullptr;
  tchem_gb_aero* aero = nullptr;
  tchem_gb_kmcd_view gas{};
  tchem_gb_aero_view av{};
  tchem_gb_numerics num{};
  int nBatch = 0, len = 0, nP = 0, n_ode = 0;
  std::vector<double> state;         // [nBatch][len]: rho, p, T, gas species, particles
  std::vector<double> number_conc;   // [nBatch][nP]
  std::vector<std::string> gas_names, aero_names;
  // device copies (first time step on)
  double *d_state = nullptr, *d_nc = nullptr, *d_tol_newton = nullptr, *d_tol_time = nullptr;
  double *d_t = nullptr, *d_dt = nullptr;
  tchem_gb_tadv* d_tadv = nullptr;
  int32_t* d_status = nullptr;
  tchem_gb_sample_stats* d_stats = nullptr;
  void* d_ws = nullptr;
  size_t ws_bytes = 0;

  ~Driver() {
    for (void* p : {static_cast<void*>(d_state), static_cast<void*>(d_nc), static_cast<void*>(d_tol_newton),
                    static_cast<void*>(d_tol_time), static_cast<void*>(d_t), static_cast<void*>(d_dt),
                    static_cast<void*>(d_tadv), static_cast<void*>(d_status), static_cast<void*>(d_stats), d_ws})
      if (p) cudaFree(p);
    tchem_gb_aero_destroy(aero);
    tchem_gb_mech_destroy(mech);
  }

  void allocate_device() {
    if (d_state) return;
    check_cuda(cudaMalloc(&d_state, sizeof(double) * state.size()), "cudaMalloc(state)");
    check_cuda(cudaMalloc(&d_nc, sizeof(double) * std::max<size_t>(number_conc.size(), 1)), "cudaMalloc(num_conc)");
    check_cuda(cudaMalloc(&d_tol_newton, sizeof(double) * 2), "cudaMalloc(tol_newton)");
    check_cuda(cudaMalloc(&d_tol_time, sizeof(double) * 2 * n_ode), "cudaMalloc(tol_time)");
    check_cuda(cudaMalloc(&d_t, sizeof(double) * nBatch), "cudaMalloc(t)");
    check_cuda(cudaMalloc(&d_dt, sizeof(double) * nBatch), "cudaMalloc(dt)");
    check_cuda(cudaMalloc(&d_tadv, sizeof(tchem_gb_tadv) * nBatch), "cudaMalloc(tadv)");
    check_cuda(cudaMalloc(&d_status, sizeof(int32_t) * nBatch), "cudaMalloc(status)");
    check_cuda(cudaMalloc(&d_stats, sizeof(tchem_gb_sample_stats) * nBatch), "cudaMalloc(stats)");
    ws_bytes = tchem_gb_aero_workspace_bytes(mech, aero, nBatch);
    if (ws_bytes == 0) check(TCHEM_GB_ERR_ARG, "tchem_gb_aero_workspace_bytes");
    check_cuda(cudaMalloc(&d_ws, ws_bytes), "cudaMalloc(workspace)");
    // the workspace header (work queue, device error word) starts zeroed, as the C ABI requires
    check_cuda(cudaMemset(d_ws, 0, ws_bytes), "cudaMemset(workspace)");
    const double tol_newton[2] = {num.atol_newton, num.rtol_newton};
    std::vector<double> tol_time(2 * static_cast<size_t>(n_ode));
    for (int i = 0; i < n_ode; ++i) {
      tol_time[2 * i] = num.atol_time;
      tol_time[2 * i + 1] = num.rtol_time;
    }
    check_cuda(cudaMemcpy(d_tol_newton, tol_newton, sizeof(tol_newton), cudaMemcpyHostToDevice), "cudaMemcpy");
    check_cuda(cudaMemcpy(d_tol_time, tol_time.data(), sizeof(double) * tol_time.size(), cudaMemcpyHostToDevice),
               "cudaMemcpy");
  }

  void do_timestep(double del_t) {
    allocate_device();
    const size_t B = static_cast<size_t>(nBatch);
    std::vector<tchem_gb_tadv> tadv(B);
    for (auto& a : tadv) {
      a = tchem_gb_tadv{};
      a.tbeg = 0.0;
      a.tend = del_t;
      a.dt = num.dtmin;
      a.dtmin = num.dtmin;
      a.dtmax = del_t;
      a.max_num_newton_iterations = num.max_newton_iterations;
      a.num_time_iterations_per_interval = std::max(1, num.max_num_time_iterations);
      a.num_outer_time_iterations_per_interval = 1;
      a.jacobian_interval = 1;
    }
    std::vector<double> t(B, 0.0), dt(B, 0.0);
    std::vector<int32_t> status(B, TCHEM_GB_SAMPLE_OK);
    std::vector<tchem_gb_sample_stats> stats(B), total(B);
    check_cuda(cudaMemcpy(d_state, state.data(), sizeof(double) * state.size(), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!number_conc.empty())
      check_cuda(cudaMemcpy(d_nc, number_conc.data(), sizeof(double) * number_conc.size(), cudaMemcpyHostToDevice),
                 "cudaMemcpy");
    check_cuda(cudaMemcpy(d_t, t.data(), sizeof(double) * B, cudaMemcpyHostToDevice), "cudaMemcpy");
    std::vector<int> failed(B, 0);
    const int max_calls = std::max(1, num.max_num_time_iterations);
    for (int call = 0; call < max_calls; ++call) {
      check_cuda(cudaMemcpy(d_tadv, tadv.data(), sizeof(tchem_gb_tadv) * B, cudaMemcpyHostToDevice), "cudaMemcpy");
      check(tchem_gb_aero_time_advance(mech, aero, nBatch, d_tol_newton, d_tol_time, nullptr, d_tadv, d_state, d_nc,
                                       d_t, d_dt, d_state, d_status, d_stats, d_ws, ws_bytes, nullptr),
            "tchem_gb_aero_time_advance");
      check_cuda(cudaMemcpy(t.data(), d_t, sizeof(double) * B, cudaMemcpyDeviceToHost), "cudaMemcpy");
      check_cuda(cudaMemcpy(dt.data(), d_dt, sizeof(double) * B, cudaMemcpyDeviceToHost), "cudaMemcpy");
      check_cuda(cudaMemcpy(status.data(), d_status, sizeof(int32_t) * B, cudaMemcpyDeviceToHost), "cudaMemcpy");
      check_cuda(cudaMemcpy(stats.data(), d_stats, sizeof(tchem_gb_sample_stats) * B, cudaMemcpyDeviceToHost),
                 "cudaMemcpy");
      bool done = true, advanced = false;
      for (size_t b = 0; b < B; ++b) {
        // rows that failed in an earlier call are out of the step (their tend was set to their
        // tbeg, so the kernel skips them) and do not count as progress
        if (failed[b] || status[b] == TCHEM_GB_SAMPLE_SKIPPED) continue;
        if (status[b] == TCHEM_GB_SAMPLE_OK && t[b] > tadv[b].tbeg) advanced = true;
        total[b].n_steps += stats[b].n_steps;
        total[b].n_rejected += stats[b].n_rejected;
        total[b].n_newton_fail += stats[b].n_newton_fail;
        total[b].n_newton_iter += stats[b].n_newton_iter;
        total[b].n_lu += stats[b].n_lu;
        total[b].n_solve += stats[b].n_solve;
        total[b].n_rhs += stats[b].n_rhs;
        total[b].n_jac += stats[b].n_jac;
        if (status[b] != TCHEM_GB_SAMPLE_OK) {
          failed[b] = status[b];
          tadv[b].tend = tadv[b].tbeg;  // no further work on this row in later calls
          continue;
        }
        tadv[b].tbeg = t[b];
        if (dt[b] > 0.0) tadv[b].dt = dt[b];
        if (t[b] < del_t) done = false;
      }
      if (done || !advanced) break;  // every row at del_t, or a call that moved no row forward
    }
    int32_t derr = 0;
    check(tchem_gb_device_error(d_ws, nullptr, &derr), "tchem_gb_device_error");
    if (derr != 0) throw std::runtime_error("TChem_doTimestep: device error word " + std::to_string(derr));
    std::vector<double> out(state.size());
    check_cuda(cudaMemcpy(out.data(), d_state, sizeof(double) * out.size(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    for (size_t b = 0; b < B; ++b) {
      if (failed[b] || t[b] < del_t) {
        std::fprintf(stderr, "TChem_doTimestep: sample %zu did not reach t = %g (status %d, t = %g); its state is kept\n",
                     b, del_t, failed[b], t[b]);
        continue;
      }
      std::copy(out.begin() + b * len, out.begin() + (b + 1) * len, state.begin() + b * len);
    }
    if (num.verbose) {
      tchem_gb_sample_stats s{};
      for (size_t b = 0; b < B; ++b) {
        s.n_steps += total[b].n_steps;
        s.n_rhs += total[b].n_rhs;
        s.n_lu += total[b].n_lu;
        s.n_jac += total[b].n_jac;
        s.n_newton_iter += total[b].n_newton_iter;
        s.n_newton_fail += total[b].n_newton_fail;
        s.n_rejected += total[b].n_rejected;
      }
      std::printf("\nFinal Statistics (all samples):\n  Steps            = %d\n  RHS evals        = %d\n"
                  "  LU factorizations = %d\n  Jac evals        = %d\n  Newton iters     = %d\n"
                  "  Newton fails     = %d\n  Error test fails = %d\n",
                  s.n_steps, s.n_rhs, s.n_lu, s.n_jac, s.n_newton_iter, s.n_newton_fail, s.n_rejected);
    }
  }
};

Driver* g_driver = nullptr;

int copy_name(const std::string& name, char* result, size_t buffer_size) {
  if (result && buffer_size > 0) {
    const size_t k = std::min(name.size(), buffer_size - 1);
    std::memcpy(result, name.data(), k);
    result[k] = '\0';
  }
  return static_cast<int>(name.size());
}

bool valid_row(int iBatch) { return g_driver && iBatch >= 0 && iBatch < g_driver->nBatch; }

}  // namespace

extern "C" {

void initialize(const char* gasFile, const char* aeroFile, const char* numericsFile, const int nBatch) {
  finalize();
  auto* d = new Driver();
  try {
    if (!gasFile || !aeroFile || !numericsFile || nBatch < 1)
      throw std::invalid_argument("initialize: file names and a batch size of at least 1 are required");
    check(tchem_gb_mech_create_from_file(gasFile, nullptr, &d->mech), "gas mechanism");
    check(tchem_gb_mech_host_view(d->mech, &d->gas), "gas mechanism");
    check(tchem_gb_aero_create_from_file(aeroFile, d->mech, &d->aero), "aerosol model");
    check(tchem_gb_aero_host_view(d->aero, &d->av), "aerosol model");
    check(tchem_gb_numerics_read(numericsFile, &d->num), "solver settings");
    if (d->av.nParticles < 1) throw std::invalid_argument("initialize: the aerosol model gives no particles");
    d->nBatch = nBatch;
    d->nP = d->av.nParticles;
    d->len = 3 + d->gas.nSpec + d->av.nSpec * d->av.nParticles;
    d->n_ode = d->gas.nSpec - d->gas.nConstSpec + d->av.nSpec * d->av.nParticles;
    d->state.assign(static_cast<size_t>(nBatch) * d->len, 0.0);
    d->number_conc.assign(static_cast<size_t>(nBatch) * d->nP, 0.0);
    char buf[256];
    for (int i = 0; i < d->gas.nSpec; ++i) {
      check(tchem_gb_mech_species_name(d->mech, i, buf, sizeof(buf)), "species name");
      d->gas_names.emplace_back(buf);
    }
    for (int i = 0; i < d->av.nSpec; ++i) {
      check(tchem_gb_aero_species_name(d->aero, i, buf, sizeof(buf)), "aerosol species name");
      d->aero_names.emplace_back(buf);
    }
    std::printf("Number of Species %d \nNumber of Reactions %d \nNumber of aerosol species %d \n"
                "Maximum number of particles %d \n",
                d->gas.nSpec, d->gas.nReac, d->av.nSpec, d->av.nParticles);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "TChem initialize failed: %s\n", e.what());
    delete d;
    return;
  }
  g_driver = d;
}

void finalize(void) {
  delete g_driver;
  g_driver = nullptr;
}

int TChem_getNumberOfSpecies(void) { return g_driver ? g_driver->gas.nSpec : -1; }

int TChem_getLengthOfStateVector(void) { return g_driver ? g_driver->len : -1; }

int TChem_getStateVectorSize(void) { return g_driver ? g_driver->nBatch * g_driver->len : -1; }

void TChem_getStateVector(double* array, const int iBatch) {
  if (!array || !valid_row(iBatch)) return;
  std::memcpy(array, g_driver->state.data() + static_cast<size_t>(iBatch) * g_driver->len,
              sizeof(double) * g_driver->len);
}

void TChem_setStateVector(double* array, const int iBatch) {
  if (!array || !valid_row(iBatch)) return;
  std::memcpy(g_driver->state.data() + static_cast<size_t>(iBatch) * g_driver->len, array,
              sizeof(double) * g_driver->len);
}

void TChem_getAllStateVectorHost(double* view) {
  if (!view || !g_driver) return;
  std::memcpy(view, g_driver->state.data(), sizeof(double) * g_driver->state.size());
}

int TChem_getSpeciesName(int* index, char* result, const size_t buffer_size) {
  if (!g_driver || !index || *index < 0 || *index >= g_driver->gas.nSpec) return copy_name("", result, buffer_size);
  return copy_name(g_driver->gas_names[*index], result, buffer_size);
}

int TChem_getNumberConcentrationVectorSize(void) { return g_driver ? g_driver->nP : -1; }

void TChem_setNumberConcentrationVector(double* array, const int iBatch) {
  if (!array || !valid_row(iBatch)) return;
  std::memcpy(g_driver->number_conc.data() + static_cast<size_t>(iBatch) * g_driver->nP, array,
              sizeof(double) * g_driver->nP);
}

int TChem_getNumberOfAeroSpecies(void) { return g_driver ? g_driver->av.nSpec : -1; }

int TChem_getAerosolSpeciesName(int* index, char* result, const size_t buffer_size) {
  if (!g_driver || !index || *index < 0 || *index >= g_driver->av.nSpec) return copy_name("", result, buffer_size);
  return copy_name(g_driver->aero_names[*index], result, buffer_size);
}

static bool aero_index_ok(const int* index) { return g_driver && index && *index >= 0 && *index < g_driver->av.nSpec; }

double TChem_getAerosolSpeciesDensity(int* index) {
  return aero_index_ok(index) ? g_driver->av.aerosol_density[*index] : 0.0;
}

double TChem_getAerosolSpeciesMW(int* index) {
  return aero_index_ok(index) ? g_driver->av.molecular_weights[*index] : 0.0;
}

double TChem_getAerosolSpeciesKappa(int* index) {
  return aero_index_ok(index) ? g_driver->av.aerosol_kappa[*index] : 0.0;
}

void TChem_doTimestep(const double& del_t) {
  if (!g_driver) {
    std::fprintf(stderr, "TChem_doTimestep: the driver is not initialized\n");
    return;
  }
  try {
    g_driver->do_timestep(del_t);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "TChem_doTimestep failed: %s\n", e.what());
  }
}

}  // extern "C"
