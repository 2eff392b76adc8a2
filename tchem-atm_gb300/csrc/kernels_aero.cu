// Gas-aerosol TR-BDF2 time advance (SIMPOL.1 gas-particle phase transfer), plain FP64 form: one
// warp per sample, persistent work queue, on the step loop, Newton iteration and dense LU of the
// box-model plain form (fp64_core.cuh), which resolve the right-hand side and the Newton matrix
// on the aerosol context below.
//
// The ODE vector is [active gas species, particle 0's aerosol species, particle 1's, ...]
// (src/core/problems/TChem_Impl_AerosolChemistry_Problem.hpp:70-160, src/core/TChem_AerosolChemistry.cpp:126-135).
// Its right-hand side (src/core/impl/TChem_Impl_Aerosol_RHS.hpp:57-100) is the box-model gas RHS
// plus, per particle and SIMPOL entry, the transfer cond - evap
// (src/core/impl/TChem_Impl_SIMPOL_phase_transfer.hpp:60-150): the gas species loses
// number_conc * (cond - evap), the particle's aerosol species gains (cond - evap) / (kg m-3 -> ppm).
// The Jacobian is a forward difference of the RHS, column j with the step 1e-8 max(|y_j|, 1e-20),
// as the reference's computeJacobian (computeNumericalJacobian,
// TChem_Impl_AerosolChemistry_Problem.hpp:204-236).
// The right-hand side itself is in aero_rhs.cuh.
#include "advance.hpp"
#include "engine.cuh"
#include "fp64_core.cuh"
#include "kernels.hpp"
#include "aero_rhs.cuh"

namespace tchem_gb {

AeroWarpLayout aero_warp_layout(const MechLayout& L, const AeroDev& A, int lda, bool matrix_in_smem) {
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  AeroWarpLayout w{};
  size_t b = 0;
  auto take = [&](uint32_t& off, size_t bytes) {
    off = static_cast<uint32_t>(b);
    b += up16(bytes);
  };
  take(w.x, sizeof(double) * A.M);
  take(w.f, sizeof(double) * A.M);
  take(w.keff, sizeof(double) * L.R);
  take(w.q, sizeof(double) * L.R);
  take(w.w, sizeof(double) * A.M);
  take(w.piv, sizeof(int32_t) * A.M);
  take(w.simc, sizeof(double) * 4 * A.nS);
  take(w.part, sizeof(double) * 3 * A.nP);
  take(w.dsim, sizeof(double) * static_cast<size_t>(A.nP) * A.nS);
  take(w.nc, sizeof(double) * A.nP);
  take(w.A, matrix_in_smem ? sizeof(double) * static_cast<size_t>(A.M) * lda : 0);
  w.bytes = static_cast<uint32_t>(b);
  return w;
}

namespace fp64 {

// Per-sample context of the aerosol problem (the members fp64_core.cuh reads, plus the evaluation data).
template <int NPL>
struct AeroCtx {
  const WarpMem& W;
  int lane;
  int lda;
  tchem_gb_sample_stats st;
  const AeroEval& E;
};

template <int NPL>
__device__ __forceinline__ int sys_dim(const AeroCtx<NPL>& c) {
  return c.E.A.M;
}

template <int NPL>
__device__ __forceinline__ void publish(AeroCtx<NPL>& c, const double (&y)[NPL]) {
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = c.lane + 32 * k;
    if (i < c.E.A.M) c.W.x[i] = y[k];
  }
  __syncwarp();
}

template <int NPL>
__device__ __forceinline__ void fetch_f(const AeroCtx<NPL>& c, double (&f)[NPL]) {
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = c.lane + 32 * k;
    f[k] = i < c.E.A.M ? c.E.f[i] : 0.0;
  }
}

template <int NPL>
__device__ __forceinline__ void rhs(AeroCtx<NPL>& c, const double (&y)[NPL], double (&f)[NPL]) {
  publish(c, y);
  aero_eval<32>(c.E, c.lane);
  fetch_f(c, f);
  __syncwarp();
  ++c.st.n_rhs;
}

// A = I - coef * J(y), J by forward differences of the RHS, one column per evaluation.
template <int NPL>
__device__ __forceinline__ void newton_matrix(AeroCtx<NPL>& c, const double (&y)[NPL], double coef) {
  publish(c, y);
  double f0[NPL];
  aero_eval<32>(c.E, c.lane);
  fetch_f(c, f0);
  const int M = c.E.A.M, lda = c.lda;
  double* A = c.W.A;
  double* x = c.W.x;
  for (int j = 0; j < M; ++j) {
    const double yj = x[j];
    const double h = 1e-8 * fmax(fabs(yj), 1e-20);
    const double yh = yj + h;
    const double hh = yh - yj;
    __syncwarp();
    if (c.lane == 0) x[j] = yh;
    __syncwarp();
    aero_eval<32>(c.E, c.lane);
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      const int i = c.lane + 32 * k;
      if (i < M) A[i * lda + j] = (i == j ? 1.0 : 0.0) - coef * ((c.E.f[i] - f0[k]) / hh);
    }
    __syncwarp();
    if (c.lane == 0) x[j] = yj;
    __syncwarp();
  }
  ++c.st.n_jac;
}

}  // namespace fp64

namespace {

using namespace fp64;

template <int NPL, bool RHS_ONLY>
__global__ void __launch_bounds__(256, 1) aero_kernel(const __grid_constant__ AeroParams P) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  unsigned char* tables = smem + 16;
  const MechLayout& L = P.mech.L;
  if (!stage_to_smem(tables, P.mech.blob, static_cast<uint32_t>(L.blob_bytes), mbar)) {
    if (threadIdx.x == 0) atomicOr(P.error_word, kErrBarrierTimeout);
    return;
  }
  const SmemTables T = tables_at(tables, L);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* mine = tables + L.blob_bytes + static_cast<size_t>(warp) * P.wl.bytes;
  const AeroWarpLayout& wl = P.wl;
  WarpMem W;
  W.x = reinterpret_cast<double*>(mine + wl.x);
  W.keff = reinterpret_cast<double*>(mine + wl.keff);
  W.q = reinterpret_cast<double*>(mine + wl.q);
  W.d = nullptr;
  W.w = reinterpret_cast<double*>(mine + wl.w);
  W.piv = reinterpret_cast<int32_t*>(mine + wl.piv);
  if (RHS_ONLY) {
    W.A = nullptr;
  } else if (P.matrix_in_smem) {
    W.A = reinterpret_cast<double*>(mine + wl.A);
  } else {
    const long long gw = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp;
    W.A = P.gmat + gw * P.gmat_stride;
  }
  AeroEval E;
  E.x = W.x;
  E.keff = W.keff;
  E.q = W.q;
  E.f = reinterpret_cast<double*>(mine + wl.f);
  E.simc = reinterpret_cast<double*>(mine + wl.simc);
  E.part = reinterpret_cast<double*>(mine + wl.part);
  E.dsim = reinterpret_cast<double*>(mine + wl.dsim);
  E.nc = reinterpret_cast<double*>(mine + wl.nc);
  E.rf_ptr = T.rf_ptr;
  E.rf_sp = T.rf_sp;
  E.pr_ptr = T.pr_ptr;
  E.pr_r = T.pr_r;
  E.pr_nu = T.pr_nu;
  E.emis = T.emis;
  E.A = P.aero;
  E.R = L.R;

  const int mg = P.aero.m_gas, M = P.aero.M, n = P.n_gas;
  // the time advance pulls samples from the work queue; the RHS (uniform work) strides over them
  int next = blockIdx.x * (blockDim.x >> 5) + warp;
  while (true) {
    int s = 0;
    if constexpr (RHS_ONLY) {
      s = next;
      next += gridDim.x * (blockDim.x >> 5);
    } else {
      if (lane == 0) s = atomicAdd(P.queue, 1);
      s = __shfl_sync(kFullMask, s, 0);
    }
    if (s >= P.B) break;
    tchem_gb_tadv ta{};
    if constexpr (!RHS_ONLY) {
      ta = P.tadv[s];
      if (P.t_out[s] >= ta.tend) {
        if (lane == 0) {
          P.status[s] = TCHEM_GB_SAMPLE_SKIPPED;
          if (P.stats) P.stats[s] = tchem_gb_sample_stats{};
        }
        continue;
      }
    }
    const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
    const double p = row[1], Tk = row[2];
    compute_keff(P.mech, P.mech.rate_param, Tk, p, row + 3 + mg, W.keff, lane);
    for (int ip = lane; ip < P.aero.nP; ip += 32) E.nc[ip] = P.number_conc[static_cast<size_t>(s) * P.aero.nP + ip];
    aero_setup<32>(E, lane, Tk, p);
    __syncwarp();
    AeroCtx<NPL> c{W, lane, P.lda, tchem_gb_sample_stats{}, E};
    double y[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      const int i = lane + 32 * k;
      y[k] = i < mg ? row[3 + i] : (i < M ? row[3 + n + (i - mg)] : 0.0);
    }
    if constexpr (RHS_ONLY) {
      double f[NPL];
      rhs(c, y, f);
#pragma unroll
      for (int k = 0; k < NPL; ++k) {
        const int i = lane + 32 * k;
        if (i < M) P.omega[static_cast<size_t>(s) * M + i] = f[k];
      }
      continue;
    } else {
      double atol[NPL], rtol[NPL];
#pragma unroll
      for (int k = 0; k < NPL; ++k) {
        const int i = lane + 32 * k;
        atol[k] = (i < M) ? P.tol_time[2 * i] : 1.0;
        rtol[k] = (i < M) ? P.tol_time[2 * i + 1] : 0.0;
      }
      NewtonSettings nset{ta.max_num_newton_iterations, ta.jacobian_interval > 0 ? ta.jacobian_interval : 1,
                          P.tol_newton[0], P.tol_newton[1]};
      double t_o = 0.0, dt_o = 0.0;
      const int st = integrate(c, y, atol, rtol, ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax,
                               ta.num_time_iterations_per_interval, nset, t_o, dt_o);
      if (lane == 0) {
        P.status[s] = st;
        if (P.stats) P.stats[s] = c.st;
      }
      if (st == TCHEM_GB_SAMPLE_NEGATIVE_DT) continue;
      double* out = P.state_out + static_cast<size_t>(s) * P.state_dim;
      // rho, p, T and the constant gas species are copied through
      // (src/core/TChem_AerosolChemistry.cpp:160-172 writes back the active gas, the particles and T).
      for (int i = lane; i < n - mg; i += 32) out[3 + mg + i] = row[3 + mg + i];
      if (lane == 0) {
        const double rho = row[0];
        out[0] = rho;
        out[1] = p;
        out[2] = Tk;
        P.t_out[s] = t_o;
        P.dt_out[s] = dt_o;
      }
#pragma unroll
      for (int k = 0; k < NPL; ++k) {
        const int i = lane + 32 * k;
        if (i < mg) out[3 + i] = y[k];
        else if (i < M) out[3 + n + (i - mg)] = y[k];
      }
      __syncwarp();
    }
  }
}

template <int NPL>
const void* aero_ptr(bool rhs_only) {
  return rhs_only ? reinterpret_cast<const void*>(aero_kernel<NPL, true>)
                  : reinterpret_cast<const void*>(aero_kernel<NPL, false>);
}

template <int NPL>
cudaError_t launch_npl(const AeroParams& P, bool rhs_only, int grid, int warps, size_t smem, cudaStream_t stream) {
  const void* k = aero_ptr<NPL>(rhs_only);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  if (rhs_only)
    aero_kernel<NPL, true><<<grid, warps * 32, smem, stream>>>(P);
  else
    aero_kernel<NPL, false><<<grid, warps * 32, smem, stream>>>(P);
  return cudaGetLastError();
}

}  // namespace

const void* aero_kernel_ptr(int M, bool rhs_only) {
  if (M <= 32) return aero_ptr<1>(rhs_only);
  if (M <= 64) return aero_ptr<2>(rhs_only);
  if (M <= 128) return aero_ptr<4>(rhs_only);
  if (M <= 256) return aero_ptr<8>(rhs_only);
  if (M <= kAeroMaxOde) return aero_ptr<10>(rhs_only);
  return nullptr;
}

cudaError_t launch_aero(const AeroParams& P, bool rhs_only, int grid, int warps, size_t smem, cudaStream_t stream) {
  const int M = P.aero.M;
  if (M <= 32) return launch_npl<1>(P, rhs_only, grid, warps, smem, stream);
  if (M <= 64) return launch_npl<2>(P, rhs_only, grid, warps, smem, stream);
  if (M <= 128) return launch_npl<4>(P, rhs_only, grid, warps, smem, stream);
  if (M <= 256) return launch_npl<8>(P, rhs_only, grid, warps, smem, stream);
  if (M <= kAeroMaxOde) return launch_npl<10>(P, rhs_only, grid, warps, smem, stream);
  return cudaErrorInvalidValue;
}

}  // namespace tchem_gb
