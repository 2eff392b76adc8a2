// Device-side building blocks shared by the time-advance kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/tchem_gb.h"
#include "device_tables.hpp"

namespace tchem_gb {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kMaxGroupMechs = 8;
// Iteration limit of every spin-wait on an mbarrier; on expiry the kernel records
// kErrBarrierTimeout in its error word and returns.
constexpr long long kSpinLimit = 1ll << 24;
constexpr int kErrBarrierTimeout = 1;
// A tensor-core kernel's second bounded wait for its MMAs also expired: it freed its TMEM while
// MMAs may still have been writing it (set together with kErrBarrierTimeout).
constexpr int kErrMmaInFlight = 2;

// Shared-memory views of the staged tables.
struct SmemTables {
  const double* emis;
  const int32_t* rf_ptr;
  const int16_t* rf_sp;
  const int32_t* pr_ptr;
  const int16_t* pr_r;
  const double* pr_nu;
  const int32_t* jz_rc;
  const int32_t* jz_ptr;
  const int16_t* jc_f;
  const double* jc_nu;
  const float* jc_nu32;
};

__device__ __forceinline__ SmemTables tables_at(const unsigned char* base, const MechLayout& L) {
  SmemTables t;
  t.emis = reinterpret_cast<const double*>(base + L.off_emis);
  t.rf_ptr = reinterpret_cast<const int32_t*>(base + L.off_rf_ptr);
  t.rf_sp = reinterpret_cast<const int16_t*>(base + L.off_rf_sp);
  t.pr_ptr = reinterpret_cast<const int32_t*>(base + L.off_pr_ptr);
  t.pr_r = reinterpret_cast<const int16_t*>(base + L.off_pr_r);
  t.pr_nu = reinterpret_cast<const double*>(base + L.off_pr_nu);
  t.jz_rc = reinterpret_cast<const int32_t*>(base + L.off_jz_rc);
  t.jz_ptr = reinterpret_cast<const int32_t*>(base + L.off_jz_ptr);
  t.jc_f = reinterpret_cast<const int16_t*>(base + L.off_jc_f);
  t.jc_nu = reinterpret_cast<const double*>(base + L.off_jc_nu);
  t.jc_nu32 = reinterpret_cast<const float*>(base + L.off_jc_nu32);
  return t;
}

// Stages `bytes` (a multiple of 16, both addresses 16-byte aligned) from global to shared
// memory with one TMA bulk copy completing on an mbarrier. Called by all threads of the CTA;
// every thread waits on the mbarrier for at most kSpinLimit polls. Returns false (uniformly
// across the CTA) when any thread gave up; the caller then exits without reading the tables.
__device__ __forceinline__ bool stage_to_smem(void* dst_smem, const void* src_gmem, uint32_t bytes,
                                              uint64_t* mbar) {
  const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(mbar));
  const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem));
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src_gmem), "r"(bytes), "r"(bar)
        : "memory");
  }
  uint32_t done = 0;
  long long it = 0;
  while (!done && it < kSpinLimit) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar)
        : "memory");
    ++it;
  }
  const bool failed = __syncthreads_or(done ? 0 : 1) != 0;
  if (failed && !done) {
    // Give the copy in flight a second bounded window before the CTA releases its shared memory.
    for (long long k = 0; k < kSpinLimit && !done; ++k) {
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(bar)
          : "memory");
    }
  }
  return !failed;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFullMask, v, o));
  return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  return v;
}

// Rate constant of reaction r at (T, p): src/core/impl/TChem_Impl_KForwardAerosol.hpp:62-134.
__device__ __forceinline__ double rate_constant(int type, const double* P, int conv_exp, double T, double t_1,
                                                double p, double conv) {
  const double one = 1.0;
  const double convp = pow(conv, static_cast<double>(conv_exp));
  if (type == RATE_ARRHENIUS) {
    const double A = P[0], B = P[1], C = P[2], D = P[3], E = P[4];
    return A * exp(C * t_1) * (B == 0.0 ? one : pow(T / D, B)) * (E == 0.0 ? one : (one + E * p)) * convp;
  }
  if (type == RATE_TROE) {
    const double k0_A = P[0], k0_B = P[1], k0_C = P[2], kinf_A = P[3], kinf_B = P[4], kinf_C = P[5], Fc = P[6],
                 N = P[7];
    const double k0 = k0_A * (k0_C == 0.0 ? one : exp(k0_C * t_1)) * (k0_B == 0.0 ? one : pow(T / 300.0, k0_B)) * conv;
    const double k0_kinf =
        k0 / (kinf_A * (kinf_C == 0.0 ? one : exp(kinf_C * t_1)) * (kinf_B == 0.0 ? one : pow(T / 300.0, kinf_B)));
    const double lg = log10(k0_kinf) / N;
    return k0 / (one + k0_kinf) * pow(Fc, one / (one + lg * lg)) * convp;
  }
  if (type == RATE_CMAQ_H2O2) {
    const double A1 = P[0], B1 = P[1], C1 = P[2], A2 = P[3], B2 = P[4], C2 = P[5];
    return (A1 * exp(C1 * t_1) * (B1 == 0.0 ? one : pow(T / 300.0, B1)) +
            A2 * exp(C2 * t_1) * (B2 == 0.0 ? one : pow(T / 300.0, B2)) * conv) *
           convp;
  }
  return 0.0;
}

// keff[r] = k_r(T, p) * prod of the constant-species factors of r, lanes over reactions.
__device__ __forceinline__ void compute_keff(const MechDev& M, const double* rate_param, double T, double p,
                                             const double* xconst, double* keff, int lane) {
  const double t_1 = 1.0 / T;
  const double conv = M.conv_ppm * p * t_1;
  for (int r = lane; r < M.L.R; r += 32) {
    double k = rate_constant(M.rate_type[r], rate_param + 8 * r, M.conv_exp[r], T, t_1, p, conv);
    for (int c = M.cf_ptr[r]; c < M.cf_ptr[r + 1]; ++c) k *= xconst[M.cf_idx[c]];
    keff[r] = k;
  }
}

}  // namespace tchem_gb
