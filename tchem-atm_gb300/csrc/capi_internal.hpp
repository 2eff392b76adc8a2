// Host helpers shared by the C-ABI translation units that launch device work.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstddef>
#include <string>

#include "device_tables.hpp"
#include "mech_host.hpp"

namespace tchem_gb {

// Workspace header: work-queue heads at byte 0 (16 x int32), the device error word at 64
// (read and cleared by tchem_gb_device_error), group counts at 128.
constexpr size_t kHeaderBytes = 256;

struct DeviceInfo {
  int sm_count = 0;
  int max_smem_optin = 0;
};
DeviceInfo device_info(int dev);

// The mechanism's packed tables on device dev (built and uploaded on first use).
DeviceTables* tables_for(const tchem_gb_mech* mech, int dev);

// Library-owned workspace of at least `bytes` on device dev (grown on demand; throws
// std::bad_alloc when the allocation fails).
void* owned_workspace(int dev, size_t bytes);
void* owned_workspace_peek(int dev);

// Records msg as the last error and returns code.
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

// Adds n to the library's count of kernel launches (tchem_gb_kernel_launches); called by every
// entry point after each launch that was accepted.
void note_launch(int n = 1);

// tchem_gb_workspace_bytes with the error code kept (TCHEM_GB_ERR_UNSUPPORTED for a mechanism
// outside the path, TCHEM_GB_ERR_ARG for bad arguments); *bytes = 0 on error.
int workspace_bytes_checked(const tchem_gb_mech* const* mechs, int n_mechs, int nbatch,
                            const tchem_gb_advance_opts* opts, size_t* bytes);

// Resolves the device address of tchem_gb_time_advance_noalloc's fixed scratch on device dev
// (loading the module that holds it); returns false when the lookup failed.
bool noalloc_setup(int dev);

// A named profiling range around an entry point's host-side work (the launches it enqueues), under
// the region names of the reference's Kokkos::Profiling::pushRegion calls (e.g.
// src/core/TChem_AtmosphericChemistry.cpp:61,244), so NVTX-aware tools (nsys, ncu --nvtx) show the
// same regions a kokkos-tools user sees. Header-only NVTX: no cost when no tool is attached.
struct ProfileRegion {
  explicit ProfileRegion(const char* name) { nvtxRangePushA(name); }
  ~ProfileRegion() { nvtxRangePop(); }
  ProfileRegion(const ProfileRegion&) = delete;
  ProfileRegion& operator=(const ProfileRegion&) = delete;
};

}  // namespace tchem_gb
