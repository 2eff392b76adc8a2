// E3SM gas-chemistry rates: rate constants, rates of progress, net production rates and the
// per-sample effective rate constants of the E3SM time advance.
//
// The reference evaluates them per sample inside every RHS call: photolysis rates into
// kfor[0, n_photo) (src/core/impl/TChem_Impl_RateofProgress.hpp:70-80), then KForward
// (src/core/impl/TChem_Impl_KForward.hpp:44-147), KForwardJPL
// (src/core/impl/TChem_Impl_KForwardJPL.hpp:45-147) and AdjustReactions
// (src/core/impl/TChem_Impl_AdjustReactions.hpp:45-100), in the order of
// src/core/impl/TChem_Impl_ReactionRates.hpp:54-79; the net production rates start from the
// external sources and scatter nu * q with atomics
// (src/core/impl/TChem_Impl_NetProductionRates.hpp:52-112). Here one warp takes one sample: lanes
// over reactions for the rate forms and their adjust factors (the reference applies the adjust
// pairs serially in file order inside a Kokkos::single; grouped by reaction with that order kept,
// each reaction's product is the same, bit for bit), lane 0 for the prod_O1D modifier, and the net
// production rates gather per species over the CSR program of the device tables (no atomics; the
// reference's atomic order is unspecified). Per sample the work is about two FP64 transcendentals
// per reaction and a few hundred flops against about 1.7 KB in and out: on GB300 (FP64 about
// 1.3 TFLOP/s) these kernels are bound by the FP64 pipe and latency, not by HBM.
#include <cuda_runtime.h>

#include <algorithm>

#include "engine.cuh"
#include "kernels.hpp"

namespace tchem_gb {

namespace {

constexpr int kE3smWarps = 4;

// k0 or kinf of the JPL forms and the R_JPL denominator: A exp(C/T) (T/300)^B, exp and pow skipped
// where C or B is 0 (src/core/impl/TChem_Impl_KForwardJPL.hpp:71-80).
__device__ __forceinline__ double jpl_arr(double A, double B, double C, double T, double t_1) {
  return A * (C == 0.0 ? 1.0 : exp(C * t_1)) * (B == 0.0 ? 1.0 : pow(T / 300.0, B));
}

// Falloff of the JPL forms with [M] = mM: k0 / (1 + k0 [M] / kinf) * Fc^(1 / (1 + log10(xpo)^2)).
__device__ __forceinline__ double jpl_falloff(const double* P, double T, double t_1, double mM) {
  const double k0 = jpl_arr(P[0], P[1], P[2], T, t_1);
  const double kinf = jpl_arr(P[3], P[4], P[5], T, t_1);
  const double xpo = k0 * mM / kinf;
  const double lg = log10(xpo);
  const double factor = P[6] == 1.0 ? 1.0 : pow(P[6], 1.0 / (1.0 + lg * lg));
  return k0 / (1.0 + xpo) * factor;
}

// Rate constant of one reaction in its E3SM form (0 for E3_NONE).
__device__ __forceinline__ double e3sm_rate(int type, const double* P, int conv_exp, double T, double t_1, double p,
                                            double conv, double mM) {
  const double one = 1.0;
  switch (type) {
    case E3_ARRHENIUS:  // A, B, C, D, E; no ppm conversion (TChem_Impl_KForward.hpp:62-67)
      return P[0] * exp(P[2] * t_1) * (P[1] == 0.0 ? one : pow(T / P[3], P[1])) * (P[4] == 0.0 ? one : (one + P[4] * p));
    case E3_TROE: {  // the reacPpar values; no ppm conversion (TChem_Impl_KForward.hpp:88-122)
      const double k0 = P[0] * (P[2] == 0.0 ? one : exp(P[2] * t_1)) * (P[1] == 0.0 ? one : pow(T / 300.0, P[1]));
      const double k0_kinf =
          k0 / (P[3] * (P[5] == 0.0 ? one : exp(P[5] * t_1)) * (P[4] == 0.0 ? one : pow(T / 300.0, P[4])));
      const double lg = log10(k0_kinf) / P[7];
      return k0 / (one + k0_kinf) * pow(P[6], one / (one + lg * lg));
    }
    case E3_CMAQ_H2O2:  // with the ppm conversion (TChem_Impl_KForward.hpp:127-136)
      return (P[0] * exp(P[2] * t_1) * (P[1] == 0.0 ? one : pow(T / 300.0, P[1])) +
              P[3] * exp(P[5] * t_1) * (P[4] == 0.0 ? one : pow(T / 300.0, P[4])) * conv) *
             pow(conv, static_cast<double>(conv_exp));
    case E3_JPL:
      return jpl_falloff(P, T, t_1, mM);
    case E3_RJPL:
      return jpl_falloff(P, T, t_1, mM) / jpl_arr(P[7], P[8], P[9], T, t_1);
    default:
      return 0.0;
  }
}

template <int KIND>
__global__ void __launch_bounds__(kE3smWarps * 32) e3sm_kernel(const __grid_constant__ E3smParams P) {
  extern __shared__ __align__(16) double e3s[];
  const MechDev& M = P.mech;
  const MechLayout& L = M.L;
  const int R = L.R, m = L.m;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* kfor = e3s + static_cast<size_t>(warp) * R;
  for (int s = blockIdx.x * kE3smWarps + warp; s < P.B; s += gridDim.x * kE3smWarps) {
    const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
    const double p = row[1], T = row[2];
    const double* x = row + 3;  // [nSpec], constant species last
    const double t_1 = 1.0 / T;
    const double conv = M.conv_ppm * p * t_1;
    const double mM = x[M.M_index];
    const double* photo = P.photo ? P.photo + static_cast<size_t>(s) * P.n_photo : nullptr;
    for (int r = lane; r < R; r += 32) {
      const int type = M.e3_type[r];
      double k = type != E3_NONE ? e3sm_rate(type, M.e3_param + kE3smParams * r, M.conv_exp[r], T, t_1, p, conv, mM)
                                 : ((photo && r < P.n_photo) ? photo[r] : 0.0);
      for (int a = M.e3_adj_ptr[r]; a < M.e3_adj_ptr[r + 1]; ++a) k *= x[M.e3_adj_sp[a]];  // adjust factors
      kfor[r] = k;
    }
    __syncwarp();
    if (lane == 0) {  // the prod_O1D modifiers read one reaction's final rate and scale three others
      for (int i = 0; i < M.e3_no1d; ++i) {
        const int32_t* I = M.e3_o1d + 7 * i;
        const double* C = M.e3_o1d_par + 6 * i;
        const double fc = C[0] * exp(C[1] * t_1) * x[I[4]] + C[2] * exp(C[3] * t_1) * x[I[5]] +
                          C[4] * exp(C[5] * t_1) * x[I[6]];
        for (int j = 0; j < 3; ++j) kfor[I[j]] *= kfor[I[3]] / fc;
      }
    }
    __syncwarp();
    if constexpr (KIND == E3SM_KFOR) {
      for (int r = lane; r < R; r += 32) P.out[static_cast<size_t>(s) * R + r] = kfor[r];
    } else if constexpr (KIND == E3SM_KEFF) {
      // keff = k * the constant-species factors (one entry per unit of |nu|), as the time-advance
      // kernels fold them
      for (int r = lane; r < R; r += 32) {
        double k = kfor[r];
        for (int c = M.cf_ptr[r]; c < M.cf_ptr[r + 1]; ++c) k *= x[m + M.cf_idx[c]];
        P.out[static_cast<size_t>(s) * R + r] = k;
      }
    } else {
      // q_r = k_r prod_j x_j^|nu_j| over the reactant slots in the reference's order, the power
      // by repeated products (exact for |nu| = 1, correctly rounded for |nu| = 2)
      for (int r = lane; r < R; r += 32) {
        double q = kfor[r];
        const int nr = M.rx_n[2 * r];
        for (int j = 0; j < nr; ++j) {
          const double xs = x[M.rx_sidx[static_cast<size_t>(r) * M.rx_S + j]];
          const int niup = abs(static_cast<int>(M.rx_nu[static_cast<size_t>(r) * M.rx_S + j]));
          double pw = niup == 0 ? 1.0 : xs;
          for (int k = 1; k < niup; ++k) pw *= xs;
          q *= pw;
        }
        if constexpr (KIND == E3SM_ROP)
          P.out[static_cast<size_t>(s) * R + r] = q;
        else
          kfor[r] = q;
      }
      if constexpr (KIND == E3SM_OMEGA) {
        __syncwarp();
        const int32_t* pr_ptr = reinterpret_cast<const int32_t*>(M.blob + L.off_pr_ptr);
        const int16_t* pr_r = reinterpret_cast<const int16_t*>(M.blob + L.off_pr_r);
        const double* pr_nu = reinterpret_cast<const double*>(M.blob + L.off_pr_nu);
        const double* ext = P.ext ? P.ext + static_cast<size_t>(s) * m : nullptr;
        for (int k = lane; k < m; k += 32) {
          double acc = ext ? ext[k] : 0.0;
          for (int e = pr_ptr[k]; e < pr_ptr[k + 1]; ++e) acc += pr_nu[e] * kfor[pr_r[e]];
          P.out[static_cast<size_t>(s) * m + k] = acc;
        }
      }
    }
    __syncwarp();  // the next sample overwrites kfor
  }
}

}  // namespace

cudaError_t launch_e3sm(const E3smParams& P, E3smOut kind, int sm_count, cudaStream_t stream) {
  if (P.B <= 0) return cudaSuccess;
  const size_t smem = sizeof(double) * static_cast<size_t>(kE3smWarps) * std::max(P.mech.L.R, 1);
  const int need = (P.B + kE3smWarps - 1) / kE3smWarps;
  const int grid = std::max(1, std::min(need, std::max(sm_count, 1) * 16));
  const void* k = kind == E3SM_KFOR ? reinterpret_cast<const void*>(e3sm_kernel<E3SM_KFOR>)
                  : kind == E3SM_ROP ? reinterpret_cast<const void*>(e3sm_kernel<E3SM_ROP>)
                  : kind == E3SM_OMEGA ? reinterpret_cast<const void*>(e3sm_kernel<E3SM_OMEGA>)
                                       : reinterpret_cast<const void*>(e3sm_kernel<E3SM_KEFF>);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  switch (kind) {
    case E3SM_KFOR: e3sm_kernel<E3SM_KFOR><<<grid, kE3smWarps * 32, smem, stream>>>(P); break;
    case E3SM_ROP: e3sm_kernel<E3SM_ROP><<<grid, kE3smWarps * 32, smem, stream>>>(P); break;
    case E3SM_OMEGA: e3sm_kernel<E3SM_OMEGA><<<grid, kE3smWarps * 32, smem, stream>>>(P); break;
    default: e3sm_kernel<E3SM_KEFF><<<grid, kE3smWarps * 32, smem, stream>>>(P); break;
  }
  return cudaGetLastError();
}

}  // namespace tchem_gb
