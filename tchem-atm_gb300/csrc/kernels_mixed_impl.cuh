// Mixed-precision TR-BDF2 kernel template (instantiated per shape in kernels_mixed_v*.cu).
//
// One warp advances one sample. The Newton matrix A = I - c J is FP32 and register-resident
// with row ownership: lane l owns rows l + 32 s (s < RPT), MC registers per row. The LU uses
// partial pivoting without moving rows ("implicit" pivoting: every row records the step at which
// it became the pivot). The loop over elimination steps is not unrolled, so the code stays small
// enough for the instruction cache; instead every row's registers are shifted by one column per
// step (the update of column j writes register j - 1), so the current column is always register
// 0 and every register index is static. Per step:
//   * the pivot is the active row with the largest |A(:,k)|, found with redux.sync.max on the
//     magnitude bits and a ballot (ties -> lowest row index);
//   * the owner lane stores the pivot row's U part (shifted by one, 16-byte aligned) in shared
//     memory, where it stays for the back substitution, plus 1/pivot and the pivot's RHS value;
//   * every lane forms its multipliers, stores them (the L factor, by row) and applies the rank-1
//     update to its rows, skipping 4-column groups beyond the trailing width.
// The forward substitution of the Newton right-hand side is fused into the factorization; the
// back substitution walks the stored U rows. The right-hand side, the Newton residual, the state,
// the local-error estimate and the step-size control are FP64; the Jacobian, the LU and the
// triangular solves are FP32, and Newton iterates to the FP64 fixed point.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "advance.hpp"
#include "engine.cuh"

namespace tchem_gb {
namespace mixed {

// Row stride of the staging / U matrix for MC a multiple of 4: congruent to 4 mod 8, so the
// 16-byte row loads of 8 consecutive lanes hit distinct banks and the column walk of the back
// substitution (stride LDU - 1, odd) is conflict-free.
__host__ __device__ constexpr int ldu_for(int MC) { return (MC % 8 == 4) ? MC : MC + 4; }
// Row stride of the L factor: odd, so the per-lane column accesses are conflict-free.
__host__ __device__ inline int ldl_for(int m) { return m | 1; }

__host__ __device__ inline size_t up16(size_t b) { return (b + 15) & ~size_t(15); }

struct MixedSmem {
  double* x;      // [m] FP64 iterate for the RHS gathers
  double* keff;   // [R]
  double* q;      // [R]
  float* x32;     // [m]
  float* keff32;  // [R]
  float* d32;     // [NF]
  float* ustage;  // [m][LDU] Newton-matrix staging, then U rows in step order: U(k, k+1+j) at [k][j]
  float* lrow;    // [m][LDL] multiplier of row r at step k
  float* pinv;    // [m] 1 / pivot of step k
  int* piv;       // [m] pivot row of step k
  float* ybuf;    // [m] forward-substitution values in step order
  int* item;      // [4] work-queue item
};

__host__ __device__ inline size_t group_smem_bytes(const MechLayout& L, int MC) {
  const int LDU = ldu_for(MC), LDL = ldl_for(L.m);
  size_t b = 0;
  b += up16(sizeof(double) * L.m);
  b += up16(sizeof(double) * L.R) * 2;
  b += up16(sizeof(float) * L.m);
  b += up16(sizeof(float) * L.R);
  b += up16(sizeof(float) * L.NF);
  b += up16(sizeof(float) * static_cast<size_t>(L.m) * LDU);
  b += up16(sizeof(float) * static_cast<size_t>(L.m) * LDL);
  b += up16(sizeof(float) * L.m);
  b += up16(sizeof(int) * L.m);
  b += up16(sizeof(float) * L.m);
  b += up16(sizeof(int) * 4);
  return b;
}

__device__ inline MixedSmem carve(unsigned char* p, const MechLayout& L, int MC) {
  const int LDU = ldu_for(MC), LDL = ldl_for(L.m);
  MixedSmem s;
  auto take = [&](size_t bytes) { unsigned char* r = p; p += up16(bytes); return r; };
  s.x = reinterpret_cast<double*>(take(sizeof(double) * L.m));
  s.keff = reinterpret_cast<double*>(take(sizeof(double) * L.R));
  s.q = reinterpret_cast<double*>(take(sizeof(double) * L.R));
  s.x32 = reinterpret_cast<float*>(take(sizeof(float) * L.m));
  s.keff32 = reinterpret_cast<float*>(take(sizeof(float) * L.R));
  s.d32 = reinterpret_cast<float*>(take(sizeof(float) * L.NF));
  s.ustage = reinterpret_cast<float*>(take(sizeof(float) * static_cast<size_t>(L.m) * LDU));
  s.lrow = reinterpret_cast<float*>(take(sizeof(float) * static_cast<size_t>(L.m) * LDL));
  s.pinv = reinterpret_cast<float*>(take(sizeof(float) * L.m));
  s.piv = reinterpret_cast<int*>(take(sizeof(int) * L.m));
  s.ybuf = reinterpret_cast<float*>(take(sizeof(float) * L.m));
  s.item = reinterpret_cast<int*>(take(sizeof(int) * 4));
  return s;
}

template <int MC, int RPT>
struct Solver {
  static_assert(MC % 4 == 0, "MC must be a multiple of 4");
  static constexpr int LDU = ldu_for(MC);

  SmemTables T;
  MixedSmem M;
  int m, R, NZ, lane, LDL;
  tchem_gb_sample_stats st;

  float A[RPT][MC];  // active rows, shifted: register j holds column k + j at step k
  int step[RPT];     // step at which the row became the pivot (INT_MAX while active)

  __device__ __forceinline__ int row(int s) const { return lane + 32 * s; }

  // ---- FP64 right-hand side: src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:80-138 -----
  __device__ __forceinline__ void rhs(const double (&y)[RPT], double (&f)[RPT]) {
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < m) M.x[row(s)] = y[s];
    __syncwarp();
    for (int r = lane; r < R; r += 32) {
      double q = M.keff[r];
      for (int g = T.rf_ptr[r]; g < T.rf_ptr[r + 1]; ++g) q *= M.x[T.rf_sp[g]];
      M.q[r] = q;
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int i = row(s);
      double acc = 0.0;
      if (i < m) {
        acc = T.emis[i];
        for (int e = T.pr_ptr[i]; e < T.pr_ptr[i + 1]; ++e) acc += T.pr_nu[e] * M.q[T.pr_r[e]];
      }
      f[s] = acc;
    }
    __syncwarp();
    ++st.n_rhs;
  }

  // ---- FP32 Newton matrix A = I - coef J(y) into registers -----------------------------
  __device__ __forceinline__ void newton_matrix(const double (&y)[RPT], double coef) {
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < m) M.x32[row(s)] = static_cast<float>(y[s]);
    // identity rows into the staging matrix (columns >= m stay 0)
    for (int e = lane; e < m * (LDU / 4); e += 32) {
      const int i = e / (LDU / 4), j4 = (e - i * (LDU / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i == j4) v.x = 1.f;
      if (i == j4 + 1) v.y = 1.f;
      if (i == j4 + 2) v.z = 1.f;
      if (i == j4 + 3) v.w = 1.f;
      reinterpret_cast<float4*>(M.ustage + static_cast<size_t>(i) * LDU)[j4 / 4] = v;
    }
    __syncwarp();
    for (int r = lane; r < R; r += 32) {
      const int f0 = T.rf_ptr[r], f1 = T.rf_ptr[r + 1];
      for (int f = f0; f < f1; ++f) {
        float dv = M.keff32[r];
        for (int g = f0; g < f1; ++g)
          if (g != f) dv *= M.x32[T.rf_sp[g]];
        M.d32[f] = dv;
      }
    }
    __syncwarp();
    const float c = static_cast<float>(coef);
    for (int z = lane; z < NZ; z += 32) {
      const int rc = T.jz_rc[z];
      const int i = rc >> 16, j = rc & 0xffff;
      float J = 0.f;
      for (int e = T.jz_ptr[z]; e < T.jz_ptr[z + 1]; ++e) J += T.jc_nu32[e] * M.d32[T.jc_f[e]];
      M.ustage[static_cast<size_t>(i) * LDU + j] = (i == j ? 1.f : 0.f) - c * J;
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int i = row(s);
      if (i < m) {
        const float4* src = reinterpret_cast<const float4*>(M.ustage + static_cast<size_t>(i) * LDU);
#pragma unroll
        for (int j4 = 0; j4 < MC / 4; ++j4) {
          const float4 v = src[j4];
          A[s][4 * j4] = v.x;
          A[s][4 * j4 + 1] = v.y;
          A[s][4 * j4 + 2] = v.z;
          A[s][4 * j4 + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < MC; ++j) A[s][j] = 0.f;
      }
    }
    __syncwarp();  // the staging area is overwritten by the U rows from here on
    ++st.n_jac;
  }

  // ---- LU with the forward substitution of wf fused in --------------------------------------
  // wf: in, the FP32 right-hand side by row; out, the forward-eliminated values by row. On return
  // M.ybuf holds the same values in step order. Returns false on a zero or non-finite pivot.
  __device__ __forceinline__ bool factor_fwd(float (&wf)[RPT]) {
    bool act[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      act[s] = row(s) < m;
      step[s] = INT_MAX;
    }
#pragma unroll 1
    for (int k = 0; k < m; ++k) {
      uint32_t vb[RPT];
      uint32_t lm = 0u;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        vb[s] = act[s] ? (__float_as_uint(A[s][0]) & 0x7fffffffu) : 0u;
        lm = max(lm, vb[s]);
      }
      const uint32_t gm = __reduce_max_sync(kFullMask, lm);
      if (gm == 0u || gm >= 0x7f800000u) return false;  // zero column, inf or nan
      int p = -1;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const unsigned bal = __ballot_sync(kFullMask, vb[s] == gm);
        if (p < 0 && bal != 0u) p = (__ffs(bal) - 1) + 32 * s;
      }
      const int owner = p & 31, pslot = p >> 5;
      const int width = m - 1 - k;  // trailing columns after the pivot
      float* urow = M.ustage + static_cast<size_t>(k) * LDU;
      if (lane == owner) {
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          if (s == pslot) {
#pragma unroll
            for (int g = 0; g < MC / 4; ++g) {
              if (4 * g < width)
                reinterpret_cast<float4*>(urow)[g] =
                    make_float4(A[s][4 * g + 1], A[s][4 * g + 2], A[s][4 * g + 3], (4 * g + 4 < MC) ? A[s][4 * g + 4] : 0.f);
            }
            M.pinv[k] = __frcp_rn(A[s][0]);
            M.ybuf[k] = wf[s];
            M.piv[k] = p;
          }
        }
      }
      __syncwarp();
      const float pinv = M.pinv[k];
      const float yk = M.ybuf[k];
      float l[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) == p) {
          act[s] = false;
          step[s] = k;
        }
        l[s] = act[s] ? A[s][0] * pinv : 0.f;
        if (act[s]) {
          M.lrow[static_cast<size_t>(row(s)) * LDL + k] = l[s];
          wf[s] = fmaf(-l[s], yk, wf[s]);
        }
      }
      // rank-1 update with a one-column shift: new A[j] = A[j+1] - l * U(k, k+1+j)
#pragma unroll
      for (int g = 0; g < MC / 4; ++g) {
        if (4 * g < width) {
          const float4 u = reinterpret_cast<const float4*>(urow)[g];
#pragma unroll
          for (int s = 0; s < RPT; ++s) {
            A[s][4 * g] = fmaf(-l[s], u.x, A[s][4 * g + 1]);
            A[s][4 * g + 1] = fmaf(-l[s], u.y, A[s][4 * g + 2]);
            A[s][4 * g + 2] = fmaf(-l[s], u.z, A[s][4 * g + 3]);
            A[s][4 * g + 3] = fmaf(-l[s], u.w, (4 * g + 4 < MC) ? A[s][4 * g + 4] : 0.f);
          }
        }
      }
    }
    __syncwarp();
    ++st.n_lu;
    return true;
  }

  // Forward substitution with the stored multipliers (rows' values in wf, in place).
  __device__ __forceinline__ void forward(float (&wf)[RPT]) {
#pragma unroll 1
    for (int k = 0; k < m; ++k) {
      const int p = M.piv[k];
      float mine = 0.f;
#pragma unroll
      for (int s = 0; s < RPT; ++s)
        if ((p >> 5) == s) mine = wf[s];
      const float yk = __shfl_sync(kFullMask, mine, p & 31);
#pragma unroll
      for (int s = 0; s < RPT; ++s)
        if (step[s] > k && row(s) < m) wf[s] = fmaf(-M.lrow[static_cast<size_t>(row(s)) * LDL + k], yk, wf[s]);
    }
    // values by step for the back substitution
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < m) M.ybuf[step[s]] = wf[s];
    __syncwarp();
  }

  // Back substitution from M.ybuf (values in step order) to x in species order.
  __device__ __forceinline__ void backward(double (&x)[RPT]) {
    float ys[RPT], pv[RPT], xs[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      ys[s] = row(s) < m ? M.ybuf[row(s)] : 0.f;
      pv[s] = row(s) < m ? M.pinv[row(s)] : 0.f;
      xs[s] = 0.f;
    }
    __syncwarp();
#pragma unroll 1
    for (int k = m - 1; k >= 0; --k) {
      float mine = 0.f;
#pragma unroll
      for (int s = 0; s < RPT; ++s)
        if ((k >> 5) == s) mine = ys[s] * pv[s];
      const float xk = __shfl_sync(kFullMask, mine, k & 31);
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int i = row(s);
        if (i < k) ys[s] = fmaf(-M.ustage[static_cast<size_t>(i) * LDU + (k - i - 1)], xk, ys[s]);
        if (i == k) xs[s] = xk;
      }
    }
#pragma unroll
    for (int s = 0; s < RPT; ++s) x[s] = static_cast<double>(xs[s]);
    ++st.n_solve;
  }

  // x = A^{-1} b with the stored factors.
  __device__ __forceinline__ void solve(const double (&b)[RPT], double (&x)[RPT]) {
    float wf[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(b[s]);
    forward(wf);
    backward(x);
  }

  // ---- Newton on y - coef f(y) = rhs --------------------------------------------------------
  __device__ __forceinline__ bool newton(double (&y)[RPT], const double (&rv)[RPT], double coef, int max_newton,
                                         int jac_interval, double atol, double rtol) {
    for (int it = 0; it < max_newton; ++it) {
      double f[RPT], dx[RPT];
      float wf[RPT];
      rhs(y, f);
#pragma unroll
      for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(-((y[s] - coef * f[s]) - rv[s]));
      if (it % jac_interval == 0) {
        newton_matrix(y, coef);
        if (!factor_fwd(wf)) return false;
      } else {
        forward(wf);
      }
      backward(dx);
      ++st.n_newton_iter;
      double sdx = 0.0, sy = 0.0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m) {
          y[s] += dx[s];
          sdx += dx[s] * dx[s];
          sy += y[s] * y[s];
        }
      }
      const double ndx = sqrt(warp_sum(sdx)), ny = sqrt(warp_sum(sy));
      if (!isfinite(ndx) || !isfinite(ny)) return false;
      if (ndx <= atol + rtol * ny) return true;
    }
    return false;
  }

  // ---- TR-BDF2 (the algorithm of the plain kernel and of the oracle) ------------------------
  __device__ __forceinline__ int integrate(double (&y)[RPT], const double (&atol)[RPT], const double (&rtol)[RPT],
                                           double t_beg, double t_end, double dt_in, double dt_min, double dt_max,
                                           int max_iters, int max_newton, int jac_interval, double natol,
                                           double nrtol, double& t_out, double& dt_out) {
    if (dt_in < 0.0) return TCHEM_GB_SAMPLE_NEGATIVE_DT;
    const double gamma = 2.0 - sqrt(2.0);
    const double d = 0.5 * gamma;
    const double cg = 1.0 / (gamma * (2.0 - gamma));
    const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
    const double kappa = (-3.0 * gamma * gamma + 4.0 * gamma - 2.0) / (12.0 * (2.0 - gamma));
    const double e0 = 1.0 / gamma, e1 = -1.0 / (gamma * (1.0 - gamma)), e2 = 1.0 / (1.0 - gamma);
    double fn[RPT], fg[RPT], f1[RPT], yg[RPT], y1[RPT], rv[RPT];
    double t = t_beg, dt = dt_in;
    int status = TCHEM_GB_SAMPLE_OK;
    rhs(y, fn);
    for (int iter = 0; iter < max_iters && t < t_end; ++iter) {
      bool converged = false, last = false;
      for (int ntry = 0; ntry < 4; ++ntry) {
        dt = fmin(fmax(dt, dt_min), dt_max);
        last = dt >= t_end - t;
        if (last) dt = t_end - t;
        if (!(dt > 0.0)) { status = TCHEM_GB_SAMPLE_DT_UNDERFLOW; break; }
        const double coef = d * dt;
        // Both implicit stages run through one copy of the Newton code.
        bool ok = true;
#pragma unroll 1
        for (int stage = 0; stage < 2 && ok; ++stage) {
          double guess[RPT];
#pragma unroll
          for (int s = 0; s < RPT; ++s) {
            rv[s] = stage == 0 ? y[s] + coef * fn[s] : cg * yg[s] - cn * y[s];
            guess[s] = stage == 0 ? y[s] : yg[s];
          }
          ok = newton(guess, rv, coef, max_newton, jac_interval, natol, nrtol);
          if (ok) {
#pragma unroll
            for (int s = 0; s < RPT; ++s) {
              if (stage == 0) yg[s] = guess[s];
              else y1[s] = guess[s];
            }
            if (stage == 0) rhs(yg, fg);
          }
        }
        if (ok) { converged = true; break; }
        ++st.n_newton_fail;
        dt *= 0.5;
      }
      if (status != TCHEM_GB_SAMPLE_OK) break;
      if (!converged) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
      rhs(y1, f1);
      double est[RPT], estf[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) est[s] = 2.0 * kappa * dt * (e0 * fn[s] + e1 * fg[s] + e2 * f1[s]);
      solve(est, estf);
      double err = 0.0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m) {
          const double wgt = atol[s] + rtol[s] * fmax(fabs(y[s]), fabs(y1[s]));
          err = fmax(err, fabs(estf[s]) / wgt);
        }
      }
      err = warp_max(err);
      if (!isfinite(err)) { status = TCHEM_GB_SAMPLE_NONFINITE; break; }
      if (err <= 1.0 || dt <= dt_min) {
        t = last ? t_end : t + dt;
#pragma unroll
        for (int s = 0; s < RPT; ++s) { y[s] = y1[s]; fn[s] = f1[s]; }
        ++st.n_steps;
        double fac = err > 0.0 ? 0.9 * cbrt(1.0 / err) : 2.0;
        fac = fmax(0.2, fmin(2.0, fac));
        dt = fmin(dt * fac, dt_max);
        if (t + dt > t_end) dt = t_end - t;
      } else {
        ++st.n_rejected;
        dt *= fmax(0.2, 0.9 * cbrt(1.0 / err));
      }
    }
    t_out = t;
    dt_out = dt;
    if (status != TCHEM_GB_SAMPLE_OK) {
#pragma unroll
      for (int s = 0; s < RPT; ++s) y[s] = 0.0;
      t_out = t_end;
      dt_out = -1.0;
    }
    return status;
  }
};

// One warp per sample, persistent work queue (same outer protocol as the plain kernel).
template <int MC, int RPT>
__global__ void __launch_bounds__(256, 1) trbdf2_mixed_kernel(const __grid_constant__ AdvanceParams P) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  unsigned char* tables = smem + 16;
  const MechLayout& L = P.mech.L;
  if (!stage_to_smem(tables, P.mech.blob, static_cast<uint32_t>(L.blob_bytes), mbar)) {
    if (threadIdx.x == 0) atomicOr(P.error_word, kErrBarrierTimeout);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t gbytes = group_smem_bytes(L, MC);
  Solver<MC, RPT> S;
  S.T = tables_at(tables, L);
  S.M = carve(tables + L.blob_bytes + warp * gbytes, L, MC);
  S.m = L.m;
  S.R = L.R;
  S.NZ = L.NZ;
  S.lane = lane;
  S.LDL = ldl_for(L.m);
  const int m = L.m;
  const int n_items = P.n_items_dev ? *P.n_items_dev : P.n_items;

  while (true) {
    int item = 0;
    if (lane == 0) item = atomicAdd(P.queue, 1);
    item = __shfl_sync(kFullMask, item, 0);
    if (item >= n_items) break;
    const int smp = P.items ? P.items[item] : item;
    const tchem_gb_tadv ta = P.tadv[smp];
    if (P.t_out[smp] >= ta.tend) {
      if (lane == 0) {
        P.status[smp] = TCHEM_GB_SAMPLE_SKIPPED;
        if (P.stats) P.stats[smp] = tchem_gb_sample_stats{};
      }
      continue;
    }
    const int gm = P.mech_of_sample ? P.mech_of_sample[smp] : 0;
    const int slot = (gm >= 0 && gm < kMaxMechs) ? P.slot_of_mech[gm] : -1;
    if (slot < 0) {
      if (lane == 0) P.status[smp] = TCHEM_GB_SAMPLE_BAD_MECH;
      continue;
    }
    const double* row = P.state + static_cast<size_t>(smp) * P.state_dim;
    const double p = row[1], Tk = row[2];
    {
      const double t_1 = 1.0 / Tk;
      const double conv = P.mech.conv_ppm * p * t_1;
      const double* rp = P.rate_param[slot];
      for (int r = lane; r < L.R; r += 32) {
        double k = rate_constant(P.mech.rate_type[r], rp + 8 * r, P.mech.conv_exp[r], Tk, t_1, p, conv);
        for (int c = P.mech.cf_ptr[r]; c < P.mech.cf_ptr[r + 1]; ++c) k *= row[3 + m + P.mech.cf_idx[c]];
        S.M.keff[r] = k;
        S.M.keff32[r] = static_cast<float>(k);
      }
    }
    __syncwarp();
    S.st = tchem_gb_sample_stats{};
    double y[RPT], atol[RPT], rtol[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int i = S.row(s);
      y[s] = (i < m) ? row[3 + i] : 0.0;
      atol[s] = (i < m) ? P.tol_time[2 * i] : 1.0;
      rtol[s] = (i < m) ? P.tol_time[2 * i + 1] : 0.0;
    }
    double t_o = 0.0, dt_o = 0.0;
    const int jac_int = ta.jacobian_interval > 0 ? ta.jacobian_interval : 1;
    const int stt = S.integrate(y, atol, rtol, ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax,
                                ta.num_time_iterations_per_interval, ta.max_num_newton_iterations, jac_int,
                                P.tol_newton[0], P.tol_newton[1], t_o, dt_o);
    if (lane == 0) {
      P.status[smp] = stt;
      if (P.stats) P.stats[smp] = S.st;
    }
    if (stt != TCHEM_GB_SAMPLE_NEGATIVE_DT) {
      double* out = P.state_out + static_cast<size_t>(smp) * P.state_dim;
      for (int i = lane; i < P.state_dim - 3 - m; i += 32) out[3 + m + i] = row[3 + m + i];
      if (lane == 0) {
        const double rho = row[0];
        out[0] = rho;
        out[1] = p;
        out[2] = Tk;
        P.t_out[smp] = t_o;
        P.dt_out[smp] = dt_o;
      }
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int i = S.row(s);
        if (i < m) out[3 + i] = y[s];
      }
    }
    __syncwarp();
  }
}

}  // namespace mixed
}  // namespace tchem_gb
