// Building blocks of the plain FP64 TR-BDF2 form, shared by the time-advance kernel
// (kernels_fp64.cu) and the discrete-adjoint kernel (kernels_adjoint.cu): the per-warp shared
// memory view, FP64 right-hand side, Newton matrix, dense LU with partial pivoting and its
// solves, Newton iteration and the TR-BDF2 step loop.
#pragma once

#include "advance.hpp"
#include "engine.cuh"

namespace tchem_gb {
namespace fp64 {


struct WarpMem {
  double* x;     // [m] current iterate, for gathers
  double* keff;  // [R]
  double* q;     // [R] rates of progress
  double* d;     // [NF] Jacobian factor-slot derivatives
  double* w;     // [m] triangular-solve vector
  int32_t* piv;  // [m]
  double* A;     // [m][lda] Newton matrix / LU factors
};

template <int NPL>
struct Ctx {
  const MechLayout& L;
  const SmemTables& T;
  const WarpMem& W;
  int lane;
  int lda;
  tchem_gb_sample_stats st;
};

// Size of the Newton system of a context (the aerosol context of kernels_aero.cu has its own).
template <int NPL>
__device__ __forceinline__ int sys_dim(const Ctx<NPL>& c) {
  return c.L.m;
}

template <int NPL>
__device__ __forceinline__ void publish(Ctx<NPL>& c, const double (&y)[NPL]) {
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = c.lane + 32 * k;
    if (i < c.L.m) c.W.x[i] = y[k];
  }
  __syncwarp();
}

// f = omega(y): src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:80-138.
template <int NPL>
__device__ __forceinline__ void rhs(Ctx<NPL>& c, const double (&y)[NPL], double (&f)[NPL]) {
  publish(c, y);
  const SmemTables& T = c.T;
  for (int r = c.lane; r < c.L.R; r += 32) {
    double q = c.W.keff[r];
    for (int g = T.rf_ptr[r]; g < T.rf_ptr[r + 1]; ++g) q *= c.W.x[T.rf_sp[g]];
    c.W.q[r] = q;
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = c.lane + 32 * k;
    double acc = 0.0;
    if (i < c.L.m) {
      acc = T.emis[i];
      for (int e = T.pr_ptr[i]; e < T.pr_ptr[i + 1]; ++e) acc += T.pr_nu[e] * c.W.q[T.pr_r[e]];
    }
    f[k] = acc;
  }
  __syncwarp();
  ++c.st.n_rhs;
}

// A = I - coef * J(y), analytic Jacobian.
template <int NPL>
__device__ __forceinline__ void newton_matrix(Ctx<NPL>& c, const double (&y)[NPL], double coef) {
  publish(c, y);
  const SmemTables& T = c.T;
  const int m = c.L.m, lda = c.lda;
  for (int r = c.lane; r < c.L.R; r += 32) {
    const int f0 = T.rf_ptr[r], f1 = T.rf_ptr[r + 1];
    for (int f = f0; f < f1; ++f) {
      double dv = c.W.keff[r];
      for (int g = f0; g < f1; ++g)
        if (g != f) dv *= c.W.x[T.rf_sp[g]];
      c.W.d[f] = dv;
    }
  }
  double* A = c.W.A;
  for (int i = 0; i < m; ++i)
    for (int j = c.lane; j < m; j += 32) A[i * lda + j] = (i == j) ? 1.0 : 0.0;
  __syncwarp();
  for (int z = c.lane; z < c.L.NZ; z += 32) {
    const int rc = T.jz_rc[z];
    const int i = rc >> 16, j = rc & 0xffff;
    double J = 0.0;
    for (int e = T.jz_ptr[z]; e < T.jz_ptr[z + 1]; ++e) J += T.jc_nu[e] * c.W.d[T.jc_f[e]];
    A[i * lda + j] = (i == j ? 1.0 : 0.0) - coef * J;
  }
  __syncwarp();
  ++c.st.n_jac;
}

// In-place LU with partial pivoting (first maximum in current row order), row swaps.
// C: a per-sample context (Ctx, or the aerosol context) with W.A, W.piv, lda, lane and st.
template <class C>
__device__ __forceinline__ bool lu_factor(C& c) {
  double* A = c.W.A;
  const int m = sys_dim(c), lda = c.lda, lane = c.lane;
  for (int k = 0; k < m; ++k) {
    double best = -1.0;
    int bi = m;
    for (int i = k + lane; i < m; i += 32) {
      const double v = fabs(A[i * lda + k]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(kFullMask, best, o);
      const int oi = __shfl_xor_sync(kFullMask, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (!(best > 0.0) || !isfinite(best)) return false;
    if (lane == 0) c.W.piv[k] = bi;
    if (bi != k) {
      for (int j = lane; j < m; j += 32) {
        const double a = A[k * lda + j];
        A[k * lda + j] = A[bi * lda + j];
        A[bi * lda + j] = a;
      }
    }
    __syncwarp();
    const double inv = 1.0 / A[k * lda + k];
    for (int i = k + 1 + lane; i < m; i += 32) A[i * lda + k] *= inv;
    __syncwarp();
    const int w = m - k - 1;
    if (w > 0) {
      const int total = w * w;
      int i = lane / w, j = lane - (lane / w) * w;
      for (int e = lane; e < total; e += 32) {
        const int ii = k + 1 + i, jj = k + 1 + j;
        A[ii * lda + jj] -= A[ii * lda + k] * A[k * lda + jj];
        j += 32;
        while (j >= w) { j -= w; ++i; }
      }
    }
    __syncwarp();
  }
  ++c.st.n_lu;
  return true;
}

// x = A^{-1} b with the factors of lu_factor.
template <int NPL, class C>
__device__ __forceinline__ void lu_solve(C& c, const double (&b)[NPL], double (&x)[NPL]) {
  const double* A = c.W.A;
  double* w = c.W.w;
  const int m = sys_dim(c), lda = c.lda, lane = c.lane;
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = lane + 32 * k;
    if (i < m) w[i] = b[k];
  }
  __syncwarp();
  if (lane == 0) {
    for (int k = 0; k < m; ++k) {
      const int p = c.W.piv[k];
      if (p != k) { const double t = w[k]; w[k] = w[p]; w[p] = t; }
    }
  }
  __syncwarp();
  for (int k = 0; k < m; ++k) {
    const double wk = w[k];
    for (int i = k + 1 + lane; i < m; i += 32) w[i] -= A[i * lda + k] * wk;
    __syncwarp();
  }
  for (int k = m - 1; k >= 0; --k) {
    const double wk = w[k] / A[k * lda + k];
    __syncwarp();
    if (lane == 0) w[k] = wk;
    for (int i = lane; i < k; i += 32) w[i] -= A[i * lda + k] * wk;
    __syncwarp();
  }
#pragma unroll
  for (int k = 0; k < NPL; ++k) {
    const int i = lane + 32 * k;
    x[k] = (i < m) ? w[i] : 0.0;
  }
  __syncwarp();
  ++c.st.n_solve;
}

struct NewtonSettings {
  int max_newton, jac_interval;
  double atol, rtol;
};

// Solves y - coef f(y) = rhs from the guess in y. rhs and newton_matrix resolve on the context type.
template <int NPL, class C>
__device__ __forceinline__ bool newton(C& c, double (&y)[NPL], const double (&rhs_v)[NPL], double coef, const NewtonSettings& s) {
  for (int it = 0; it < s.max_newton; ++it) {
    double f[NPL], g[NPL], dx[NPL];
    rhs(c, y, f);
#pragma unroll
    for (int k = 0; k < NPL; ++k) g[k] = -((y[k] - coef * f[k]) - rhs_v[k]);
    if (it % s.jac_interval == 0) {
      newton_matrix(c, y, coef);
      if (!lu_factor(c)) return false;
    }
    lu_solve(c, g, dx);
    ++c.st.n_newton_iter;
    double sdx = 0.0, sy = 0.0;
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      if (c.lane + 32 * k < sys_dim(c)) {
        y[k] += dx[k];
        sdx += dx[k] * dx[k];
        sy += y[k] * y[k];
      }
    }
    const double ndx = sqrt(warp_sum(sdx)), ny = sqrt(warp_sum(sy));
    if (!isfinite(ndx) || !isfinite(ny)) return false;
    if (ndx <= s.atol + s.rtol * ny) return true;
  }
  return false;
}

// One sample's trajectory record (dt == nullptr: not recorded): accepted step sizes and the
// state at the start of steps 0, kTapeSegment, 2 kTapeSegment, ...
struct Tape {
  double* dt;    // [cap]
  double* ckpt;  // [cap / kTapeSegment + 1][m]
  int cap;
};

// TR-BDF2 integration of one sample (same algorithm as the oracle's Sample::integrate).
template <int NPL, class C>
__device__ int integrate(C& c, double (&y)[NPL], const double (&atol)[NPL], const double (&rtol)[NPL],
                         double t_beg, double t_end, double dt_in, double dt_min, double dt_max, int max_iters,
                         const NewtonSettings& s, double& t_out, double& dt_out, const Tape& tape = Tape{}) {
  if (dt_in < 0.0) return TCHEM_GB_SAMPLE_NEGATIVE_DT;
  const double gamma = 2.0 - sqrt(2.0);
  const double d = 0.5 * gamma;
  const double cg = 1.0 / (gamma * (2.0 - gamma));
  const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
  const double kappa = (-3.0 * gamma * gamma + 4.0 * gamma - 2.0) / (12.0 * (2.0 - gamma));
  const double e0 = 1.0 / gamma, e1 = -1.0 / (gamma * (1.0 - gamma)), e2 = 1.0 / (1.0 - gamma);
  const int m = sys_dim(c);

  double fn[NPL], fg[NPL], f1[NPL], yg[NPL], y1[NPL], rv[NPL];
  double t = t_beg, dt = dt_in;
  int status = TCHEM_GB_SAMPLE_OK;
  rhs(c, y, fn);
  for (int iter = 0; iter < max_iters && t < t_end; ++iter) {
    bool converged = false, last = false;
    for (int ntry = 0; ntry < 4; ++ntry) {
      dt = fmin(fmax(dt, dt_min), dt_max);
      last = dt >= t_end - t;
      if (last) dt = t_end - t;
      if (!(dt > 0.0)) { status = TCHEM_GB_SAMPLE_DT_UNDERFLOW; break; }
      const double coef = d * dt;
#pragma unroll
      for (int k = 0; k < NPL; ++k) { rv[k] = y[k] + coef * fn[k]; yg[k] = y[k]; }
      bool ok = newton(c, yg, rv, coef, s);
      if (ok) {
        rhs(c, yg, fg);
#pragma unroll
        for (int k = 0; k < NPL; ++k) { rv[k] = cg * yg[k] - cn * y[k]; y1[k] = yg[k]; }
        ok = newton(c, y1, rv, coef, s);
      }
      if (ok) { converged = true; break; }
      ++c.st.n_newton_fail;
      dt *= 0.5;
    }
    if (status != TCHEM_GB_SAMPLE_OK) break;
    if (!converged) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
    rhs(c, y1, f1);
    double est[NPL], estf[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) est[k] = 2.0 * kappa * dt * (e0 * fn[k] + e1 * fg[k] + e2 * f1[k]);
    lu_solve(c, est, estf);
    double err = 0.0;
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      if (c.lane + 32 * k < m) {
        const double wgt = atol[k] + rtol[k] * fmax(fabs(y[k]), fabs(y1[k]));
        err = fmax(err, fabs(estf[k]) / wgt);
      }
    }
    err = warp_max(err);
    if (!isfinite(err)) { status = TCHEM_GB_SAMPLE_NONFINITE; break; }
    if (err <= 1.0 || dt <= dt_min) {
      if (tape.dt) {
        const int n = c.st.n_steps;
        if (n >= tape.cap) { status = TCHEM_GB_SAMPLE_TAPE_FULL; break; }
        if (c.lane == 0) tape.dt[n] = dt;
        if (n % kTapeSegment == 0) {
#pragma unroll
          for (int k = 0; k < NPL; ++k) {
            const int i = c.lane + 32 * k;
            if (i < m) tape.ckpt[static_cast<size_t>(n / kTapeSegment) * m + i] = y[k];
          }
        }
      }
      t = last ? t_end : t + dt;
#pragma unroll
      for (int k = 0; k < NPL; ++k) { y[k] = y1[k]; fn[k] = f1[k]; }
      ++c.st.n_steps;
      double fac = err > 0.0 ? 0.9 * cbrt(1.0 / err) : 2.0;
      fac = fmax(0.2, fmin(2.0, fac));
      dt = fmin(dt * fac, dt_max);
      if (t + dt > t_end) dt = t_end - t;
    } else {
      ++c.st.n_rejected;
      dt *= fmax(0.2, 0.9 * cbrt(1.0 / err));
    }
  }
  t_out = t;
  dt_out = dt;
  if (status != TCHEM_GB_SAMPLE_OK) {
#pragma unroll
    for (int k = 0; k < NPL; ++k) y[k] = 0.0;
    t_out = t_end;
    dt_out = -1.0;
  }
  return status;
}


}  // namespace fp64
}  // namespace tchem_gb
