// Host helpers shared by the C-ABI translation units that launch device work.
#pragma once

#include <cuda_runtime.h>

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

}  // namespace tchem_gb
