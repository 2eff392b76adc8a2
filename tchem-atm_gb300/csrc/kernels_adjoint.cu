// Discrete adjoint of the plain FP64 TR-BDF2 form: one warp per sample, persistent work queue.
//
// Given the accepted step sizes and checkpoints recorded by the forward run (state at the start
// of every kTapeSegment-th step) and a cotangent lambda = dL/dy(t_end) of the active species,
// the kernel returns dL/dy(t_0) and dL/dtheta_r, where exp(theta_r) multiplies reaction r's rate
// constant (all of its pre-exponential factors at once), so dq_r/dtheta_r = q_r.
//
// The step sequence is the recorded one (step-size control is not differentiated). Per step
// with c = gamma/2 dt, the stages are
//   (1) y_g - c f(y_g) = y_n + c f(y_n)
//   (2) y_1 - c f(y_1) = cg y_g - cn y_n
// and, with exact stage solutions, their adjoint is
//   mu2 = (I - c J(y_1))^-T lambda_1,              dL/dtheta += c q(y_1) (nu^T mu2)
//   mu1 = (I - c J(y_g))^-T (cg mu2),              dL/dtheta += c (q(y_g) + q(y_n)) (nu^T mu1)
//   lambda_n = -cn mu2 + (I + c J(y_n))^T mu1.
// Within each segment the forward states y_n, y_g are recomputed from the checkpoint with the
// recorded step sizes (the same Newton code and inputs, so the same values) into a per-warp
// global buffer, then the segment is swept backward.
#include "advance.hpp"
#include "engine.cuh"
#include "fp64_core.cuh"
#include "kernels.hpp"

namespace tchem_gb {

using namespace fp64;

namespace {

// mu = A^-T b with the factors of lu_factor (P A = L U by row swaps):
// U^T z = b (forward over U's rows), L^T v = z (backward over L's rows), mu = P^T v.
template <int NPL>
__device__ __forceinline__ void lu_solve_t(Ctx<NPL>& c, const double (&b)[NPL], double (&x)[NPL]) {
  const double* A = c.W.A;
  double* w = c.W.w;
  const int m = c.L.m, lda = c.lda, lane = c.lane;
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = lane + 32 * k;
    if (i < m) w[i] = b[k];
  }
  __syncwarp();
  for (int j = 0; j < m; ++j) {
    const double zj = w[j] / A[j * lda + j];
    __syncwarp();
    if (lane == 0) w[j] = zj;
    for (int l = j + 1 + lane; l < m; l += 32) w[l] -= A[j * lda + l] * zj;
    __syncwarp();
  }
  for (int k = m - 1; k > 0; --k) {
    const double vk = w[k];
    for (int i = lane; i < k; i += 32) w[i] -= A[k * lda + i] * vk;
    __syncwarp();
  }
  if (lane == 0) {
    for (int k = m - 1; k >= 0; --k) {
      const int p = c.W.piv[k];
      if (p != k) { const double t = w[k]; w[k] = w[p]; w[p] = t; }
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = lane + 32 * k;
    x[k] = (i < m) ? w[i] : 0.0;
  }
  __syncwarp();
  ++c.st.n_solve;
}

// out = A^T mu for the dense matrix in W.A (mu in shared memory).
template <int NPL>
__device__ __forceinline__ void matvec_t(Ctx<NPL>& c, const double* mu, double (&out)[NPL]) {
  const double* A = c.W.A;
  const int m = c.L.m, lda = c.lda;
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int j = c.lane + 32 * k;
    double a0 = 0.0, a1 = 0.0;
    if (j < m) {
      int i = 0;
      for (; i + 1 < m; i += 2) {
        a0 += A[i * lda + j] * mu[i];
        a1 += A[(i + 1) * lda + j] * mu[i + 1];
      }
      if (i < m) a0 += A[i * lda + j] * mu[i];
    }
    out[k] = a0 + a1;
  }
}

template <int NPL>
__device__ __forceinline__ void publish_vec(Ctx<NPL>& c, double* dst, const double (&v)[NPL]) {
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = c.lane + 32 * k;
    if (i < c.L.m) dst[i] = v[k];
  }
  __syncwarp();
}

// gk[r] += coef * q[r] * (nu_r . mu) for the rates of progress left in W.q by the last rhs().
template <int NPL>
__device__ __forceinline__ void accumulate_gk(Ctx<NPL>& c, const MechDev& M, const double* mu, double coef,
                                              double* gk) {
  const int S = M.rx_S, half = S / 2, m = c.L.m;
  for (int r = c.lane; r < c.L.R; r += 32) {
    const int nr = M.rx_n[2 * r], np = M.rx_n[2 * r + 1];
    double dot = 0.0;
    for (int j = 0; j < nr; ++j) {
      const int sp = M.rx_sidx[r * S + j];
      if (sp < m) dot += M.rx_nu[r * S + j] * mu[sp];
    }
    for (int j = 0; j < np; ++j) {
      const int sp = M.rx_sidx[r * S + half + j];
      if (sp < m) dot += M.rx_nu[r * S + half + j] * mu[sp];
    }
    gk[r] += coef * c.W.q[r] * dot;
  }
  __syncwarp();
}

template <int NPL>
__global__ void __launch_bounds__(256, 1) adjoint_fp64_kernel(const __grid_constant__ AdjointParams P) {
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
  unsigned char* mine = tables + L.blob_bytes + static_cast<size_t>(warp) * P.warp_smem_bytes;
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  WarpMem W;
  W.x = reinterpret_cast<double*>(mine);
  mine += up16(sizeof(double) * L.m);
  W.keff = reinterpret_cast<double*>(mine);
  mine += up16(sizeof(double) * L.R);
  W.q = reinterpret_cast<double*>(mine);
  mine += up16(sizeof(double) * L.R);
  W.d = reinterpret_cast<double*>(mine);
  mine += up16(sizeof(double) * L.NF);
  W.w = reinterpret_cast<double*>(mine);
  mine += up16(sizeof(double) * L.m);
  W.piv = reinterpret_cast<int32_t*>(mine);
  mine += up16(sizeof(int32_t) * L.m);
  double* gk = reinterpret_cast<double*>(mine);  // [R] dL/dtheta of the current sample
  mine += up16(sizeof(double) * L.R);
  double* mu = reinterpret_cast<double*>(mine);  // [m] adjoint stage vector, for gathers
  mine += up16(sizeof(double) * L.m);
  const long long gw = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp;
  W.A = P.matrix_in_smem ? reinterpret_cast<double*>(mine) : P.gmat + gw * P.gmat_stride;
  double* seg = P.seg + gw * P.seg_stride;  // [kTapeSegment][2][m]: y_n, y_g of the segment's steps

  const int m = L.m;
  const double gamma = 2.0 - sqrt(2.0);
  const double d = 0.5 * gamma;
  const double cg = 1.0 / (gamma * (2.0 - gamma));
  const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
  const int ckpt_rows = P.tape_cap / kTapeSegment + 1;
  while (true) {
    int s = 0;
    if (lane == 0) s = atomicAdd(P.queue, 1);
    s = __shfl_sync(kFullMask, s, 0);
    if (s >= P.B) break;
    const tchem_gb_tadv ta = P.tadv[s];
    const int nsteps = P.tape_nsteps[s];
    if (nsteps < 0 || nsteps > P.tape_cap) {
      if (lane == 0) P.status[s] = TCHEM_GB_SAMPLE_TAPE_FULL;
      continue;
    }
    const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
    compute_keff(P.mech, P.rate_param, row[2], row[1], row + 3 + m, W.keff, lane);
    __syncwarp();
    if (P.k_scale) {
      for (int r = lane; r < L.R; r += 32) W.keff[r] *= P.k_scale[r];
    }
    for (int r = lane; r < L.R; r += 32) gk[r] = 0.0;
    __syncwarp();
    Ctx<NPL> c{L, T, W, lane, P.lda, tchem_gb_sample_stats{}};
    NewtonSettings ns{ta.max_num_newton_iterations, ta.jacobian_interval > 0 ? ta.jacobian_interval : 1,
                      P.tol_newton[0], P.tol_newton[1]};
    const double* tdt = P.tape_dt + static_cast<size_t>(s) * P.tape_cap;
    const double* ckpt = P.tape_ckpt + static_cast<size_t>(s) * ckpt_rows * m;
    double lam[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      const int i = lane + 32 * k;
      lam[k] = (i < m) ? P.lambda[static_cast<size_t>(s) * m + i] : 0.0;
    }
    int status = TCHEM_GB_SAMPLE_OK;
    for (int sg = (nsteps + kTapeSegment - 1) / kTapeSegment - 1; sg >= 0 && status == TCHEM_GB_SAMPLE_OK; --sg) {
      const int j0 = sg * kTapeSegment;
      const int len = min(kTapeSegment, nsteps - j0);
      // recompute the segment's forward states from its checkpoint
      double y[NPL], fn[NPL];
#pragma unroll
      for (int k = 0; k < NPL; ++k) {
        const int i = lane + 32 * k;
        y[k] = (i < m) ? ckpt[static_cast<size_t>(sg) * m + i] : 0.0;
      }
      rhs(c, y, fn);
      for (int j = 0; j < len; ++j) {
        const double coef = d * tdt[j0 + j];
        double yg[NPL], rv[NPL];
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const int i = lane + 32 * k;
          if (i < m) seg[(2 * j) * m + i] = y[k];
          rv[k] = y[k] + coef * fn[k];
          yg[k] = y[k];
        }
        if (!newton(c, yg, rv, coef, ns)) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const int i = lane + 32 * k;
          if (i < m) seg[(2 * j + 1) * m + i] = yg[k];
          rv[k] = cg * yg[k] - cn * y[k];
          y[k] = yg[k];
        }
        if (!newton(c, y, rv, coef, ns)) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
        rhs(c, y, fn);
      }
      if (status != TCHEM_GB_SAMPLE_OK) break;
      // backward sweep; y holds y_{n+1} of the step being reversed
      for (int j = len - 1; j >= 0; --j) {
        const double coef = d * tdt[j0 + j];
        double yg[NPL], yn[NPL], mu2[NPL], mu1[NPL], tmp[NPL];
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const int i = lane + 32 * k;
          yn[k] = (i < m) ? seg[(2 * j) * m + i] : 0.0;
          yg[k] = (i < m) ? seg[(2 * j + 1) * m + i] : 0.0;
        }
        // stage 2 at y_{n+1}
        newton_matrix(c, y, coef);
        if (!lu_factor(c)) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
        lu_solve_t(c, lam, mu2);
        rhs(c, y, tmp);
        publish_vec(c, mu, mu2);
        accumulate_gk(c, P.mech, mu, coef, gk);
        // stage 1 at y_gamma
#pragma unroll
        for (int k = 0; k < NPL; ++k) tmp[k] = cg * mu2[k];
        newton_matrix(c, yg, coef);
        if (!lu_factor(c)) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
        lu_solve_t(c, tmp, mu1);
        publish_vec(c, mu, mu1);
        rhs(c, yg, tmp);
        accumulate_gk(c, P.mech, mu, coef, gk);
        rhs(c, yn, tmp);
        accumulate_gk(c, P.mech, mu, coef, gk);
        // lambda_n = -cn mu2 + (I + c J(y_n))^T mu1
        newton_matrix(c, yn, -coef);
        matvec_t(c, mu, tmp);
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          lam[k] = -cn * mu2[k] + tmp[k];
          y[k] = yn[k];
        }
        __syncwarp();
      }
    }
    if (lane == 0) P.status[s] = status;
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      const int i = lane + 32 * k;
      if (i < m) P.grad_x0[static_cast<size_t>(s) * m + i] = status == TCHEM_GB_SAMPLE_OK ? lam[k] : 0.0;
    }
    for (int r = lane; r < L.R; r += 32)
      P.grad_k[static_cast<size_t>(s) * L.R + r] = status == TCHEM_GB_SAMPLE_OK ? gk[r] : 0.0;
    __syncwarp();
  }
}

template <int NPL>
cudaError_t launch_adjoint_npl(const AdjointParams& P, int grid, int warps, size_t smem, cudaStream_t stream) {
  auto k = adjoint_fp64_kernel<NPL>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, warps * 32, smem, stream>>>(P);
  return cudaGetLastError();
}

}  // namespace

size_t adjoint_warp_smem_bytes(const MechLayout& L, int lda, bool matrix_in_smem) {
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  return fp64_warp_smem_bytes(L, lda, matrix_in_smem) + up16(sizeof(double) * L.R) + up16(sizeof(double) * L.m);
}

const void* adjoint_kernel_ptr(int m) {
  if (m <= 32) return reinterpret_cast<const void*>(adjoint_fp64_kernel<1>);
  if (m <= 64) return reinterpret_cast<const void*>(adjoint_fp64_kernel<2>);
  if (m <= 128) return reinterpret_cast<const void*>(adjoint_fp64_kernel<4>);
  return reinterpret_cast<const void*>(adjoint_fp64_kernel<8>);
}

cudaError_t launch_adjoint(const AdjointParams& P, int grid, int warps, size_t smem, cudaStream_t stream) {
  const int m = P.mech.L.m;
  if (m <= 32) return launch_adjoint_npl<1>(P, grid, warps, smem, stream);
  if (m <= 64) return launch_adjoint_npl<2>(P, grid, warps, smem, stream);
  if (m <= 128) return launch_adjoint_npl<4>(P, grid, warps, smem, stream);
  if (m <= 256) return launch_adjoint_npl<8>(P, grid, warps, smem, stream);
  return cudaErrorInvalidValue;
}

}  // namespace tchem_gb
