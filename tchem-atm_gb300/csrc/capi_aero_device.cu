// C ABI: gas-aerosol (SIMPOL.1 phase transfer) time advance and right-hand side on the device
// (TChem::AerosolChemistry::runDeviceBatch, src/core/TChem_AerosolChemistry.cpp:236-260).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "aero_host.hpp"
#include "capi_internal.hpp"
#include "kernels.hpp"
#include "mech_host.hpp"

namespace tchem_gb {

void destroy_aero_device_tables(AeroDeviceTables* t) {
  if (!t) return;
  if (t->allocation) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(t->device);
    cudaFree(t->allocation);
    cudaSetDevice(prev);
  }
  delete t;
}

namespace {

constexpr int kAeroMaxWarpsPerBlock = 8;

size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

AeroDeviceTables* upload_aero_tables(const tchem_gb_aero& a, int device) {
  const size_t nS = a.am.simpol.size(), nA = static_cast<size_t>(a.am.nSpec);
  const size_t o_idx = 0, o_par = up256(sizeof(int32_t) * 3 * nS), o_den = o_par + up256(sizeof(double) * 7 * nS),
               o_mw = o_den + up256(sizeof(double) * nA), bytes = o_mw + up256(sizeof(double) * nA) + 256;
  std::vector<unsigned char> host(bytes, 0);
  if (nS) {
    std::memcpy(host.data() + o_idx, a.simpol_index.data(), sizeof(int32_t) * 3 * nS);
    std::memcpy(host.data() + o_par, a.simpol_param.data(), sizeof(double) * 7 * nS);
  }
  if (nA) {
    std::memcpy(host.data() + o_den, a.am.aerosol_density.data(), sizeof(double) * nA);
    std::memcpy(host.data() + o_mw, a.am.molecular_weights.data(), sizeof(double) * nA);
  }
  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) throw std::runtime_error("cudaSetDevice failed");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaSetDevice(prev);
    throw std::runtime_error(std::string("cudaMalloc for aerosol tables: ") + cudaGetErrorString(e));
  }
  e = cudaMemcpy(p, host.data(), bytes, cudaMemcpyHostToDevice);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaFree(p);
    throw std::runtime_error(std::string("cudaMemcpy for aerosol tables: ") + cudaGetErrorString(e));
  }
  auto* t = new AeroDeviceTables();
  t->device = device;
  t->allocation = p;
  unsigned char* b = static_cast<unsigned char*>(p);
  t->sim_idx = reinterpret_cast<const int32_t*>(b + o_idx);
  t->sim_par = reinterpret_cast<const double*>(b + o_par);
  t->density = reinterpret_cast<const double*>(b + o_den);
  t->mw = reinterpret_cast<const double*>(b + o_mw);
  return t;
}

AeroDeviceTables* aero_tables_for(const tchem_gb_aero* aero, int dev) {
  auto* a = const_cast<tchem_gb_aero*>(aero);
  std::lock_guard<std::mutex> lk(a->mu);
  if (static_cast<int>(a->device_tables.size()) <= dev) a->device_tables.resize(dev + 1, nullptr);
  if (!a->device_tables[dev]) a->device_tables[dev] = upload_aero_tables(*a, dev);
  return a->device_tables[dev];
}

const HostTables* host_tables_of(const tchem_gb_mech* mech) {
  auto* m = const_cast<tchem_gb_mech*>(mech);
  std::lock_guard<std::mutex> lk(m->mu);
  if (!m->host_tables) m->host_tables.reset(new HostTables(build_host_tables(m->km)));
  return m->host_tables.get();
}

// Checks that the gas mechanism and the aerosol model form a problem the kernel runs (host only,
// no device call) and fills the problem sizes of A (pointers are set at launch).
int aero_problem(const tchem_gb_mech* mech, const tchem_gb_aero* aero, const char* who, AeroDev& A) {
  const KineticModel& km = mech->km;
  const AerosolModel& am = aero->am;
  const int mg = km.nSpec - km.nConstSpec;
  if (am.nSpec_gas != mg || am.nConstSpec_gas != km.nConstSpec)
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": the aerosol model was built on another gas mechanism");
  if (am.nParticles < 1 || am.nSpec < 1)
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": the aerosol model needs particles and aerosol species");
  const HostTables* ht = nullptr;
  try {
    ht = host_tables_of(mech);
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": " + e.what());
  }
  if (!ht->supported) return fail(TCHEM_GB_ERR_UNSUPPORTED, std::string(who) + ": " + ht->unsupported_reason);
  for (const auto& s : am.simpol) {
    if (s.gas_sp_index < 0 || s.gas_sp_index >= mg)
      return fail(TCHEM_GB_ERR_UNSUPPORTED,
                  std::string(who) + ": a SIMPOL entry's gas species is not an active species");
    if (s.aerosol_sp_index < mg || s.aerosol_sp_index >= mg + am.nSpec)
      return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": a SIMPOL entry's aerosol index is out of range");
  }
  const long long M = static_cast<long long>(mg) + static_cast<long long>(am.nParticles) * am.nSpec;
  if (M > kAeroMaxOde)
    return fail(TCHEM_GB_ERR_UNSUPPORTED, std::string(who) + ": the aerosol ODE system has " + std::to_string(M) +
                                               " entries; the kernel takes at most " + std::to_string(kAeroMaxOde));
  A = AeroDev{};
  A.nA = am.nSpec;
  A.nP = am.nParticles;
  A.nS = static_cast<int32_t>(am.simpol.size());
  A.m_gas = mg;
  A.M = static_cast<int32_t>(M);
  // particle floors (src/core/impl/TChem_Impl_SingleParticleUtils.hpp: 1e-25 kg/m3 of mass,
  // 0.1 kg/mol, 1800 kg/m3), evaluated in long double as the reference's literals are
  const long double min_mass = 1.0e-25L, min_mw = 0.1L, min_density = 1800.0L;
  A.vol0 = static_cast<double>(min_mass / min_density);
  A.mass0 = static_cast<double>(min_mass);
  A.moles0 = static_cast<double>(min_mass / min_mw);
  return TCHEM_GB_OK;
}

struct AeroPlan {
  AeroWarpLayout wl{};
  const void* kernel = nullptr;
  int lda = 0, warps = 0, grid = 0;
  size_t smem = 0;
  bool matrix_in_smem = true;
  size_t gmat_offset = 0, gmat_elems = 0, bytes = 0;
};

AeroPlan make_aero_plan(const MechLayout& L, const AeroDev& A, int nbatch, int dev, bool rhs_only) {
  AeroPlan p;
  const DeviceInfo info = device_info(dev);
  p.lda = A.M | 1;
  const size_t avail = static_cast<size_t>(info.max_smem_optin) - 16 - static_cast<size_t>(L.blob_bytes);
  p.matrix_in_smem = !rhs_only;
  p.wl = aero_warp_layout(L, A, p.lda, p.matrix_in_smem);
  int W = static_cast<int>(std::min<size_t>(kAeroMaxWarpsPerBlock, avail / p.wl.bytes));
  if (W < 1 && p.matrix_in_smem) {
    p.matrix_in_smem = false;
    p.wl = aero_warp_layout(L, A, p.lda, false);
    W = static_cast<int>(std::min<size_t>(kAeroMaxWarpsPerBlock, avail / p.wl.bytes));
  }
  if (W < 1) throw std::invalid_argument("aerosol problem too large for the shared-memory working set");
  p.warps = W;
  p.smem = 16 + static_cast<size_t>(L.blob_bytes) + static_cast<size_t>(W) * p.wl.bytes;
  p.kernel = aero_kernel_ptr(A.M, rhs_only);
  if (!p.kernel) throw std::invalid_argument("aerosol ODE system too large");
  cudaFuncSetAttribute(p.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(p.smem));
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, p.kernel, W * 32, p.smem) != cudaSuccess || bps < 1) {
    cudaGetLastError();
    bps = 1;
  }
  const int need = (std::max(nbatch, 1) + W - 1) / W;
  p.grid = std::max(1, std::min(info.sm_count * bps, need));
  p.bytes = kHeaderBytes;
  if (!rhs_only && !p.matrix_in_smem) {
    p.gmat_elems = static_cast<size_t>(A.M) * p.lda;
    p.gmat_offset = p.bytes;
    p.bytes += up256(sizeof(double) * p.gmat_elems * static_cast<size_t>(p.grid) * W);
  }
  return p;
}

void fill_pointers(AeroDev& A, const AeroDeviceTables* t) {
  A.sim_idx = t->sim_idx;
  A.sim_par = t->sim_par;
  A.density = t->density;
  A.mw = t->mw;
}

}  // namespace
}  // namespace tchem_gb

using namespace tchem_gb;

extern "C" {

size_t tchem_gb_aero_workspace_bytes(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch) {
  if (!mech || !aero || nbatch < 0) {
    fail(TCHEM_GB_ERR_ARG, "tchem_gb_aero_workspace_bytes: bad argument");
    return 0;
  }
  AeroDev A;
  if (aero_problem(mech, aero, "tchem_gb_aero_workspace_bytes", A) != TCHEM_GB_OK) return 0;
  try {
    int dev = 0;
    cudaGetDevice(&dev);
    const DeviceTables* t = tables_for(mech, dev);
    return make_aero_plan(t->dev.L, A, nbatch, dev, false).bytes;
  } catch (const std::exception& e) {
    fail(TCHEM_GB_ERR_ARG, e.what());
    return 0;
  }
}

int tchem_gb_aero_time_advance(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch,
                               const double* tol_newton, const double* tol_time, const double* fac,
                               const tchem_gb_tadv* tadv, const double* state, const double* number_conc,
                               double* t_out, double* dt_out, double* state_out, int32_t* status,
                               tchem_gb_sample_stats* stats, void* workspace, size_t workspace_bytes, void* stream_v) {
  (void)fac;
  ProfileRegion region("TChem::AerosolChemistry::runDeviceBatch::kmcd array");
  const char* who = "tchem_gb_aero_time_advance";
  if (!mech || !aero || nbatch < 0) return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": bad model or batch size");
  AeroDev A;
  const int rc = aero_problem(mech, aero, who, A);
  if (rc != TCHEM_GB_OK) return rc;
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!tol_newton || !tol_time || !tadv || !state || !number_conc || !t_out || !dt_out || !state_out || !status)
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": null argument");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  int dev = 0;
  cudaGetDevice(&dev);
  AeroPlan plan;
  const DeviceTables* t = nullptr;
  try {
    t = tables_for(mech, dev);
    fill_pointers(A, aero_tables_for(aero, dev));
    plan = make_aero_plan(t->dev.L, A, nbatch, dev, false);
  } catch (const std::bad_alloc&) {
    return fail(TCHEM_GB_ERR_NOMEM, std::string(who) + ": allocation failed");
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": " + e.what());
  }
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (!ws) {
    try {
      ws = static_cast<unsigned char*>(owned_workspace(dev, plan.bytes));
    } catch (...) {
      return fail(TCHEM_GB_ERR_NOMEM, std::string(who) + ": workspace allocation failed");
    }
  } else if (workspace_bytes < plan.bytes) {
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": workspace smaller than tchem_gb_aero_workspace_bytes()");
  }
  cudaError_t e = cudaMemsetAsync(ws, 0, 64, stream);  // work queue (the error word persists until read)
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(workspace)");
  AeroParams P{};
  P.mech = t->dev;
  P.aero = A;
  P.wl = plan.wl;
  P.B = nbatch;
  P.n_gas = mech->km.nSpec;
  P.state_dim = 3 + mech->km.nSpec + A.nP * A.nA;
  P.number_conc = number_conc;
  P.tol_newton = tol_newton;
  P.tol_time = tol_time;
  P.tadv = tadv;
  P.state = state;
  P.state_out = state_out;
  P.t_out = t_out;
  P.dt_out = dt_out;
  P.status = status;
  P.stats = stats;
  P.omega = nullptr;
  P.gmat = plan.matrix_in_smem ? nullptr : reinterpret_cast<double*>(ws + plan.gmat_offset);
  P.gmat_stride = static_cast<int64_t>(plan.gmat_elems);
  P.lda = plan.lda;
  P.matrix_in_smem = plan.matrix_in_smem ? 1 : 0;
  P.queue = reinterpret_cast<int32_t*>(ws);
  P.error_word = reinterpret_cast<int32_t*>(ws + 64);
  e = launch_aero(P, false, plan.grid, plan.warps, plan.smem, stream);
  if (e != cudaSuccess) return cuda_fail(e, "aerosol time-advance kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}

int tchem_gb_aero_rhs(const tchem_gb_mech* mech, const tchem_gb_aero* aero, int nbatch, const double* state,
                      const double* number_conc, double* omega, void* stream_v) {
  const char* who = "tchem_gb_aero_rhs";
  if (!mech || !aero || nbatch < 0) return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": bad model or batch size");
  AeroDev A;
  const int rc = aero_problem(mech, aero, who, A);
  if (rc != TCHEM_GB_OK) return rc;
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!state || !number_conc || !omega) return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": null argument");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  int dev = 0;
  cudaGetDevice(&dev);
  AeroPlan plan;
  const DeviceTables* t = nullptr;
  unsigned char* ws = nullptr;
  try {
    t = tables_for(mech, dev);
    fill_pointers(A, aero_tables_for(aero, dev));
    plan = make_aero_plan(t->dev.L, A, nbatch, dev, true);
    ws = static_cast<unsigned char*>(owned_workspace(dev, plan.bytes));
  } catch (const std::bad_alloc&) {
    return fail(TCHEM_GB_ERR_NOMEM, std::string(who) + ": allocation failed");
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": " + e.what());
  }
  AeroParams P{};
  P.mech = t->dev;
  P.aero = A;
  P.wl = plan.wl;
  P.B = nbatch;
  P.n_gas = mech->km.nSpec;
  P.state_dim = 3 + mech->km.nSpec + A.nP * A.nA;
  P.number_conc = number_conc;
  P.state = state;
  P.omega = omega;
  P.lda = plan.lda;
  P.queue = nullptr;  // the RHS kernel strides over the samples
  P.error_word = reinterpret_cast<int32_t*>(ws + 64);
  cudaError_t e = launch_aero(P, true, plan.grid, plan.warps, plan.smem, stream);
  if (e != cudaSuccess) return cuda_fail(e, "aerosol RHS kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}

}  // extern "C"
