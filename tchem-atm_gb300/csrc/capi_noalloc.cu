// tchem_gb_time_advance_noalloc: the batched time advance for callers that may not allocate
// device memory. No counterpart in the reference.
//
// Who needs it: a host model that owns all device memory through its own pool and forbids any
// other allocation (a chemistry component inside a coupled climate model with a fixed device
// footprint), or a time-critical loop where cudaMalloc / cudaFree would synchronise the device and
// stall the caller's other streams. tchem_gb_time_advance either takes a workspace from the caller
// or allocates and caches one; this entry point does neither. Its work-queue scratch (queue heads,
// device error word, per-group sample counts and lists) lives in g_noalloc_scratch below, a fixed
// __device__ array that every context loading the library holds until the process exits.
//
// Limits and rules:
//  * kNoAllocScratchBytes (1 MiB) of scratch: enough for any single-structure batch; batches that
//    mix mechanism structures need 4 bytes per sample and structure group, and plain-form
//    mechanisms whose Newton matrix does not fit in shared memory need per-warp matrices, so such
//    calls may not fit and are rejected with TCHEM_GB_ERR_ARG.
//  * The mechanisms' device tables must already be on the current device: call
//    tchem_gb_workspace_bytes (or any other time-advance entry point) once at set-up, where
//    allocation is allowed. Otherwise the call is rejected with TCHEM_GB_ERR_ARG.
//  * The scratch array's device address is looked up once per device (cudaGetSymbolAddress),
//    which loads the module that holds the array and so allocates its 1 MiB then (CUDA loads
//    modules lazily by default). tchem_gb_workspace_bytes does this lookup at set-up for the
//    current device; a first call of this entry point on a device where nothing did it does
//    the lookup itself, and may therefore allocate once. Make the set-up call (or that first
//    call) before any stream capture.
//  * Every call on a device shares the one scratch array, which keeps the last call's contents.
//    Each call clears the parts that must start at zero (queue heads, error word, group counts)
//    on its stream before its kernels run. Calls that overlap on the GPU (other streams, other
//    threads) race on the scratch and give wrong results: serialise them.
//  * Device-side wait timeouts are not readable through tchem_gb_device_error for these calls; a
//    sample that no kernel reached keeps the status value the caller put there, so callers that
//    need to detect it pre-fill status with a value the engine never writes (e.g. -1).
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.hpp"
#include "mech_host.hpp"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;

// Host code must not use this name as an address (it is a host-side stand-in for the device
// array); it takes the device address from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
std::vector<void*> g_noalloc_ptr;  // device address of g_noalloc_scratch per device ordinal

// The device address of the scratch on device dev (looked up on first use); nullptr and *err set
// when the lookup fails.
void* scratch_address(int dev, cudaError_t* err) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (static_cast<int>(g_noalloc_ptr.size()) <= dev) g_noalloc_ptr.resize(dev + 1, nullptr);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (*err != cudaSuccess || !p) return nullptr;
    g_noalloc_ptr[dev] = p;
  }
  *err = cudaSuccess;
  return g_noalloc_ptr[dev];
}

}  // namespace

namespace tchem_gb {
bool noalloc_setup(int dev) {
  cudaError_t e = cudaSuccess;
  if (scratch_address(dev, &e)) return true;
  cudaGetLastError();  // a failed lookup here is reported by the entry point's own call
  return false;
}
}  // namespace tchem_gb

extern "C" int tchem_gb_time_advance_noalloc(const tchem_gb_mech* const* mechs, int n_mechs,
                                             const int32_t* mech_of_sample, int nbatch, const double* tol_newton,
                                             const double* tol_time, const double* fac, const tchem_gb_tadv* tadv,
                                             const double* state, double* t_out, double* dt_out, double* state_out,
                                             int32_t* status, tchem_gb_sample_stats* stats,
                                             const tchem_gb_advance_opts* opts, void* stream_v) {
  using tchem_gb::set_last_error;
  if (!mechs || n_mechs <= 0 || nbatch < 0) {
    set_last_error("tchem_gb_time_advance_noalloc: bad mechanisms or batch size");
    return TCHEM_GB_ERR_ARG;
  }
  if (nbatch == 0) return TCHEM_GB_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_error(std::string("tchem_gb_time_advance_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return TCHEM_GB_ERR_CUDA;
  }
  // The mechanism tables must be resident: uploading them would allocate.
  for (int i = 0; i < n_mechs; ++i) {
    if (!mechs[i]) {
      set_last_error("tchem_gb_time_advance_noalloc: null mechanism handle");
      return TCHEM_GB_ERR_ARG;
    }
    auto* m = const_cast<tchem_gb_mech*>(mechs[i]);
    std::lock_guard<std::mutex> lk(m->mu);
    if (!m->host_tables || static_cast<int>(m->device_tables.size()) <= dev || !m->device_tables[dev]) {
      set_last_error("tchem_gb_time_advance_noalloc: mechanism " + std::to_string(i) +
                     " has no tables on device " + std::to_string(dev) +
                     " yet; call tchem_gb_workspace_bytes with it once at set-up");
      return TCHEM_GB_ERR_ARG;
    }
  }
  // The scratch array's device address on this device (looked up once, with the device current).
  void* scratch = scratch_address(dev, &e);
  if (!scratch) {
    set_last_error(std::string("tchem_gb_time_advance_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return TCHEM_GB_ERR_CUDA;
  }
  size_t need = 0;
  const int rc = tchem_gb::workspace_bytes_checked(mechs, n_mechs, nbatch, opts, &need);
  if (rc != TCHEM_GB_OK) return rc;  // same code and message as tchem_gb_time_advance
  if (need > kNoAllocScratchBytes) {
    set_last_error("tchem_gb_time_advance_noalloc: this call needs " + std::to_string(need) +
                   " bytes of scratch but the fixed scratch holds " + std::to_string(kNoAllocScratchBytes) +
                   " bytes; split the batch or use tchem_gb_time_advance with a workspace");
    return TCHEM_GB_ERR_ARG;
  }
  // queue heads, device error word and group counts start at zero
  e = cudaMemsetAsync(scratch, 0, 256, static_cast<cudaStream_t>(stream_v));
  if (e != cudaSuccess) {
    set_last_error(std::string("tchem_gb_time_advance_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
    return TCHEM_GB_ERR_CUDA;
  }
  return tchem_gb_time_advance(mechs, n_mechs, mech_of_sample, nbatch, tol_newton, tol_time, fac, tadv, state, t_out,
                               dt_out, state_out, status, stats, scratch, kNoAllocScratchBytes, opts, stream_v);
}
