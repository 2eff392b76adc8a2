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
//
// Registers hold the matrix rows and the Newton iterate; everything touched once per step (the
// FP64 stage vectors, tolerances, counters) lives in shared memory at offsets taken from the kernel
// parameters, so no register is spent on addresses.
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

// Stage vectors kept in shared memory (FP64, [kVec][m]).
// V_YP / V_YGP: simplified form: y_n and y_gamma of the last accepted step (stage-1 predictor);
// FP32-LU form: the refinement's vector and the point of the factored Jacobian.
enum Vec { V_FN = 0, V_FG = 1, V_YP = 2, V_ATOL = 3, V_RTOL = 4, V_YGP = 5, kVec = 6 };
// Work counters kept in shared memory, in tchem_gb_sample_stats order.
enum Stat { S_STEPS = 0, S_REJ = 1, S_NFAIL = 2, S_NEWTON = 3, S_LU = 4, S_SOLVE = 5, S_RHS = 6, S_JAC = 7 };

// src_section: a per-group source-term section (the E3SM kernels' per-sample external sources).
// lu_nnz > 0: the sparse-LU shape (the factors' entries replace the dense staging matrix).
inline MixedLayout make_layout(const MechLayout& L, int MC, bool simplified, bool src_section = false,
                               int lu_nnz = 0) {
  auto up16 = [](size_t b) { return static_cast<uint32_t>((b + 15) & ~size_t(15)); };
  MixedLayout ml{};
  ml.LDU = ldu_for(MC);
  ml.LDL = L.m | 1;
  ml.simplified = simplified ? 1 : 0;
  uint32_t o = 0;
  ml.x = o; o += up16(sizeof(double) * L.m);
  ml.keff = o; o += up16(sizeof(double) * L.R);
  ml.q = o; o += up16(sizeof(double) * (L.R + 1));  // q[R] = 0 is the padding target
  ml.vec = o; o += up16(sizeof(double) * kVec * L.m);
  ml.x32 = o; o += up16(sizeof(float) * L.m);
  ml.keff32 = o; o += up16(sizeof(float) * L.R);
  ml.d32 = o; o += up16(sizeof(float) * (L.NF + 1));  // d32[NF] = 0 is the padding target
  ml.ustage = o;
  if (lu_nnz == 0) o += up16(sizeof(float) * static_cast<size_t>(L.m) * ml.LDU);
  ml.lu = o; o += up16(sizeof(float) * static_cast<size_t>(lu_nnz));
  ml.lrow = o;  // L factor by row (LU forms only)
  if (!simplified) o += up16(sizeof(float) * static_cast<size_t>(L.m) * ml.LDL);
  ml.pinv = o; o += up16(sizeof(float) * L.m);
  ml.piv = o; o += up16(sizeof(int) * L.m);
  ml.ybuf = o; o += up16(sizeof(float) * MC);  // MC >= m
  ml.stats = o; o += up16(sizeof(int) * 8);
  ml.red = o; o += 256;  // cross-warp reductions of multi-warp samples (2 x 8 u32, 2 x 8 f64, 2 f32)
  ml.item = o; o += up16(sizeof(int) * 4);
  ml.src = 0;
  if (src_section) { ml.src = o; o += up16(sizeof(double) * L.m); }
  ml.warp_bytes = o;
  return ml;
}

// SIMP selects the simplified-Newton form (Gauss-Jordan inverse); each form is its own kernel so
// that neither carries the other's code through the instruction cache.
//
// G > 1 (simplified form only) spreads one sample over G warps of one CTA, one row per thread:
// loops stride over the group's 32 G threads, the sliced-ELL programs go slice by slice to the
// group's warps, and reductions and the pivot broadcast go through shared memory with a named
// barrier per group.
//
// E3 selects the E3SM inputs: per-sample rate constants (P.keff_in) and source terms (P.src_in,
// staged into the group's shared memory) instead of the mechanism's rate parameters and emissions.
// A separate instantiation, so the other kernels compile exactly as without it.
//
// FULLGJ (with SIMP) keeps the Gauss-Jordan linear algebra but runs the reference's full Newton
// (a new matrix every jacobian_interval iterations, the reference's stage guesses and 2-norm
// test) with one FP64-residual refinement sweep per solve, like the FP32-LU form: it follows the
// FP64 Newton iterates with matrix-vector solves instead of triangular ones.
//
// SP (with FULLGJ, one warp) replaces the dense linear algebra by the static-order sparse LU
// (sparse_lu.hpp): the Newton matrix is assembled into the filled pattern's entries in shared
// memory, factored without pivot search by the mechanism's update program (one __syncwarp per
// elimination step) and applied by column-oriented substitutions; full Newton and the refinement
// sweep are unchanged. MC is then only the width of the solve vector (>= m).
template <int MC, int RPT, bool SIMP, int G = 1, bool FULLGJ = false, bool E3 = false, bool SP = false>
struct Solver {
  static_assert(!FULLGJ || SIMP, "the full-Newton Gauss-Jordan variant uses the inverse");
  static_assert(!SP || (FULLGJ && G == 1 && !E3), "the sparse-LU shape is a one-warp full-Newton shape");
  static constexpr bool kSimplifiedNewton = SIMP && !FULLGJ;
  static_assert(MC % 4 == 0, "MC must be a multiple of 4");
  static_assert(G == 1 || RPT == 1, "multi-warp samples: one row per thread");
  static constexpr int LDU = ldu_for(MC);
  static constexpr int NT = 32 * G;                       // threads per sample
  static constexpr int NROWS = NT * RPT;                  // rows held in registers
  static_assert(NROWS <= 128, "row index must fit the pivot key");
  static constexpr uint32_t KMASK = NROWS <= 64 ? 63u : 127u;  // low key bits holding the row

  const AdvanceParams& P;
  const unsigned char* tb;  // staged tables
  unsigned char* wb;        // this sample's region
  int lane;                 // lane in the warp
  int tid;                  // thread in the sample's group (== lane for G == 1)
  int wid;                  // warp in the group
  int bar;                  // named barrier of the group (G > 1)
  int rp = 0;               // rotating slot of the cross-warp reductions

  float A[RPT][MC];  // active rows, shifted: register j holds column k + j at step k
  int step[RPT];     // step at which the row became the pivot (INT_MAX while active)
  // simplified-Newton form: the stored inverse is valid / was formed in the current stage, and
  // the coefficient c it was formed with
  bool have_inv = false, fresh = false;
  double c_inv = 0.0;

  __device__ __forceinline__ int m() const { return P.mech.L.m; }
  // thread index in the sample's group (the lane itself for one warp per sample)
  __device__ __forceinline__ int gt() const {
    if constexpr (G == 1) {
      return lane;
    } else {
      return tid;
    }
  }
  // first sliced-ELL slice of this warp (slices go round-robin to the group's warps)
  __device__ __forceinline__ int wslice() const {
    if constexpr (G == 1) {
      return 0;
    } else {
      return wid;
    }
  }
  __device__ __forceinline__ int row(int s) const {
    if constexpr (G == 1) {
      return lane + 32 * s;
    } else {
      return tid + NT * s;
    }
  }
  template <typename Tp>
  __device__ __forceinline__ Tp* w(uint32_t off) const { return reinterpret_cast<Tp*>(wb + off); }
  template <typename Tp>
  __device__ __forceinline__ const Tp* t(int32_t off) const { return reinterpret_cast<const Tp*>(tb + off); }
  __device__ __forceinline__ double& vec(int v, int i) const { return w<double>(P.ml.vec)[v * m() + i]; }
  __device__ __forceinline__ void count(int which) const {
    if (gt() == 0) ++w<int>(P.ml.stats)[which];
  }

  // ---- group synchronisation and reductions (G == 1: warp primitives) -----------------------
  __device__ __forceinline__ void gsync() const {
    if constexpr (G == 1) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(NT) : "memory");
    }
  }
  // Every cross-warp reduction passes one barrier; two rotating slots keep a warp that runs
  // ahead from overwriting values a slower warp has not read yet.
  __device__ __forceinline__ uint32_t gmax_u32(uint32_t v) {
    v = __reduce_max_sync(kFullMask, v);
    if constexpr (G == 1) {
      return v;
    } else {
      uint32_t* r = w<uint32_t>(P.ml.red) + 8 * rp;
      rp ^= 1;
      if (lane == 0) r[wid] = v;
      gsync();
      uint32_t mx = r[0];
#pragma unroll
      for (int i = 1; i < G; ++i) mx = max(mx, r[i]);
      return mx;
    }
  }
  __device__ __forceinline__ uint32_t gor_u32(uint32_t v) {
    v = __reduce_or_sync(kFullMask, v);
    if constexpr (G == 1) {
      return v;
    } else {
      uint32_t* r = w<uint32_t>(P.ml.red) + 8 * rp;
      rp ^= 1;
      if (lane == 0) r[wid] = v;
      gsync();
      uint32_t o = r[0];
#pragma unroll
      for (int i = 1; i < G; ++i) o |= r[i];
      return o;
    }
  }
  __device__ __forceinline__ double gsum_f64(double v) {
    v = warp_sum(v);
    if constexpr (G == 1) {
      return v;
    } else {
      double* r = reinterpret_cast<double*>(w<unsigned char>(P.ml.red) + 64) + 8 * rp;
      rp ^= 1;
      if (lane == 0) r[wid] = v;
      gsync();
      double t = r[0];
#pragma unroll
      for (int i = 1; i < G; ++i) t += r[i];
      return t;
    }
  }
  __device__ __forceinline__ double gmax_f64(double v) {
    v = warp_max(v);
    if constexpr (G == 1) {
      return v;
    } else {
      double* r = reinterpret_cast<double*>(w<unsigned char>(P.ml.red) + 64) + 8 * rp;
      rp ^= 1;
      if (lane == 0) r[wid] = v;
      gsync();
      double mx = r[0];
#pragma unroll
      for (int i = 1; i < G; ++i) mx = fmax(mx, r[i]);
      return mx;
    }
  }

  // ---- FP64 right-hand side: src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:80-138 -----
  // f = omega(y), y in registers (by row); f returned by row.
  __device__ __forceinline__ void rhs(const double (&y)[RPT], double (&f)[RPT]) {
    const MechLayout& L = P.mech.L;
    double* x = w<double>(P.ml.x);
    double* q = w<double>(P.ml.q);
    const double* keff = w<double>(P.ml.keff);
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < L.m) x[row(s)] = y[s];
    gsync();
    const int32_t* rf_ptr = t<int32_t>(L.off_rf_ptr);
    const int16_t* rf_sp = t<int16_t>(L.off_rf_sp);
#pragma unroll 2
    for (int r = gt(); r < L.R; r += NT) {
      const int g0 = rf_ptr[r], g1 = rf_ptr[r + 1];
      double qq = keff[r];
      if (g1 > g0) qq *= x[rf_sp[g0]];
      if (g1 > g0 + 1) qq *= x[rf_sp[g0 + 1]];
      for (int g = g0 + 2; g < g1; ++g) qq *= x[rf_sp[g]];
      q[r] = qq;
    }
    gsync();
    // net production over species slices (sliced ELL); results staged in x by species
    const int32_t* ws_sp = t<int32_t>(L.off_ws_sp);
    const int32_t* ws_cnt = t<int32_t>(L.off_ws_cnt);
    const int32_t* ws_off = t<int32_t>(L.off_ws_off);
    const int16_t* wse_r = t<int16_t>(L.off_wse_r);
    const double* wse_nu = t<double>(L.off_wse_nu);
    const double* emis;
    if constexpr (E3)
      emis = w<double>(P.ml.src);  // the sample's E3SM source term
    else
      emis = t<double>(L.off_emis);
#pragma unroll 2
    for (int sl = wslice(); sl < L.NWS; sl += G) {
      const int sp = ws_sp[sl * 32 + lane];
      const int cnt = ws_cnt[sl];
      const int base = ws_off[sl] + lane;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int c = 0;
      for (; c + 4 <= cnt; c += 4) {
        const int e = base + 32 * c;
        const int r0 = wse_r[e], r1 = wse_r[e + 32], r2 = wse_r[e + 64], r3 = wse_r[e + 96];
        a0 += wse_nu[e] * q[r0];
        a1 += wse_nu[e + 32] * q[r1];
        a2 += wse_nu[e + 64] * q[r2];
        a3 += wse_nu[e + 96] * q[r3];
      }
      for (; c < cnt; ++c) a0 += wse_nu[base + 32 * c] * q[wse_r[base + 32 * c]];
      if (sp >= 0) x[sp] = emis[sp] + ((a0 + a1) + (a2 + a3));
    }
    gsync();
#pragma unroll
    for (int s = 0; s < RPT; ++s) f[s] = row(s) < L.m ? x[row(s)] : 0.0;
    gsync();
    count(S_RHS);
  }

  // ---- FP64 Jacobian-vector product J(x_J) v (mixed form's refinement residual) ----------
  // x_J: the point the factored matrix was built at (stage-vector slot V_YGP); v by row.
  // dq_r/dx . v = keff_r sum_f v[sp_f] prod_{g != f} x[sp_g], then the net-production program
  // without emissions.
  __device__ __forceinline__ void jvec(const double (&v)[RPT], double (&out)[RPT]) {
    const MechLayout& L = P.mech.L;
    double* x = w<double>(P.ml.x);
    double* vv = &vec(V_YP, 0);
    double* q = w<double>(P.ml.q);
    const double* keff = w<double>(P.ml.keff);
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < L.m) {
        x[row(s)] = vec(V_YGP, row(s));
        vv[row(s)] = v[s];
      }
    gsync();
    const int32_t* rf_ptr = t<int32_t>(L.off_rf_ptr);
    const int16_t* rf_sp = t<int16_t>(L.off_rf_sp);
    for (int r = gt(); r < L.R; r += NT) {
      const int g0 = rf_ptr[r], g1 = rf_ptr[r + 1];
      double dq = 0.0;
      if (g1 - g0 == 1) {
        dq = vv[rf_sp[g0]];
      } else if (g1 - g0 == 2) {
        const int a = rf_sp[g0], b = rf_sp[g0 + 1];
        dq = vv[a] * x[b] + x[a] * vv[b];
      } else {
        for (int f = g0; f < g1; ++f) {
          double p = vv[rf_sp[f]];
          for (int g = g0; g < g1; ++g)
            if (g != f) p *= x[rf_sp[g]];
          dq += p;
        }
      }
      q[r] = keff[r] * dq;
    }
    gsync();
    const int32_t* ws_sp = t<int32_t>(L.off_ws_sp);
    const int32_t* ws_cnt = t<int32_t>(L.off_ws_cnt);
    const int32_t* ws_off = t<int32_t>(L.off_ws_off);
    const int16_t* wse_r = t<int16_t>(L.off_wse_r);
    const double* wse_nu = t<double>(L.off_wse_nu);
    for (int sl = wslice(); sl < L.NWS; sl += G) {
      const int sp = ws_sp[sl * 32 + lane];
      const int cnt = ws_cnt[sl];
      const int base = ws_off[sl] + lane;
      double a0 = 0.0, a1 = 0.0;
      int c = 0;
      for (; c + 2 <= cnt; c += 2) {
        const int e = base + 32 * c;
        a0 += wse_nu[e] * q[wse_r[e]];
        a1 += wse_nu[e + 32] * q[wse_r[e + 32]];
      }
      if (c < cnt) a0 += wse_nu[base + 32 * c] * q[wse_r[base + 32 * c]];
      if (sp >= 0) x[sp] = a0 + a1;
    }
    gsync();
#pragma unroll
    for (int s = 0; s < RPT; ++s) out[s] = row(s) < L.m ? x[row(s)] : 0.0;
    gsync();
    count(S_RHS);
  }

  // ---- FP32 Newton matrix A = I - coef J(y) into registers -----------------------------
  __device__ __forceinline__ void newton_matrix(const double (&y)[RPT], double coef) {
    const MechLayout& L = P.mech.L;
    const int mm = L.m;
    float* x32 = w<float>(P.ml.x32);
    float* d32 = w<float>(P.ml.d32);
    float* stage = w<float>(P.ml.ustage);
    const float* keff32 = w<float>(P.ml.keff32);
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < mm) x32[row(s)] = static_cast<float>(y[s]);
    // identity rows into the staging matrix (columns >= m stay 0)
    for (int e = gt(); e < mm * (LDU / 4); e += NT) {
      const int i = e / (LDU / 4), j4 = (e - i * (LDU / 4)) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i == j4) v.x = 1.f;
      if (i == j4 + 1) v.y = 1.f;
      if (i == j4 + 2) v.z = 1.f;
      if (i == j4 + 3) v.w = 1.f;
      reinterpret_cast<float4*>(stage + i * LDU)[j4 / 4] = v;
    }
    gsync();
    const int32_t* rf_ptr = t<int32_t>(L.off_rf_ptr);
    const int16_t* rf_sp = t<int16_t>(L.off_rf_sp);
#pragma unroll 2
    for (int r = gt(); r < L.R; r += NT) {
      const int f0 = rf_ptr[r], f1 = rf_ptr[r + 1];
      const float kr = keff32[r];
      if (f1 - f0 == 1) {
        d32[f0] = kr;
      } else if (f1 - f0 == 2) {
        const float xa = x32[rf_sp[f0]], xb = x32[rf_sp[f0 + 1]];
        d32[f0] = kr * xb;
        d32[f0 + 1] = kr * xa;
      } else {
        for (int f = f0; f < f1; ++f) {
          float dv = kr;
          for (int g = f0; g < f1; ++g)
            if (g != f) dv *= x32[rf_sp[g]];
          d32[f] = dv;
        }
      }
    }
    gsync();
    const float c = static_cast<float>(coef);
    const int32_t* js_rc = t<int32_t>(L.off_js_rc);
    const int32_t* js_cnt = t<int32_t>(L.off_js_cnt);
    const int32_t* js_off = t<int32_t>(L.off_js_off);
    const int16_t* jse_f = t<int16_t>(L.off_jse_f);
    const float* jse_nu = t<float>(L.off_jse_nu32);
    // Jacobian nonzeros over slices (sliced ELL): uniform trip counts, independent loads
#pragma unroll 2
    for (int sl = wslice(); sl < L.NJS; sl += G) {
      const int rc = js_rc[sl * 32 + lane];
      const int cnt = js_cnt[sl];
      const int base = js_off[sl] + lane;
      float J0 = 0.f, J1 = 0.f;
      int cc = 0;
      for (; cc + 2 <= cnt; cc += 2) {
        const int e = base + 32 * cc;
        const int f0 = jse_f[e], f1 = jse_f[e + 32];
        J0 += jse_nu[e] * d32[f0];
        J1 += jse_nu[e + 32] * d32[f1];
      }
      if (cc < cnt) J0 += jse_nu[base + 32 * cc] * d32[jse_f[base + 32 * cc]];
      if (rc >= 0) {
        const int i = rc >> 16, j = rc & 0xffff;
        stage[i * LDU + j] = (i == j ? 1.f : 0.f) - c * (J0 + J1);
      }
    }
    gsync();
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int i = row(s);
      if (i < mm) {
        const float4* src = reinterpret_cast<const float4*>(stage + i * LDU);
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
    gsync();  // the staging area is overwritten by the U rows from here on
    count(S_JAC);
  }

  // Rank-1 update with a one-column shift on groups [G0, G1): new A[j] = A[j+1] - l * U(k, k+1+j).
  // All of the chunk's U loads are issued before its FMAs.
  // ext: the value shifted into the last register (0 for the LU; the new inverse column for
  // Gauss-Jordan).
  template <int G0, int G1>
  __device__ __forceinline__ void update_chunk(const float (&l)[RPT], const float* urow, const float (&ext)[RPT]) {
    float4 u[G1 - G0];
#pragma unroll
    for (int g = G0; g < G1; ++g) u[g - G0] = reinterpret_cast<const float4*>(urow)[g];
#pragma unroll
    for (int g = G0; g < G1; ++g) {
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        A[s][4 * g] = fmaf(-l[s], u[g - G0].x, A[s][4 * g + 1]);
        A[s][4 * g + 1] = fmaf(-l[s], u[g - G0].y, A[s][4 * g + 2]);
        A[s][4 * g + 2] = fmaf(-l[s], u[g - G0].z, A[s][4 * g + 3]);
        A[s][4 * g + 3] = fmaf(-l[s], u[g - G0].w, (4 * g + 4 < MC) ? A[s][4 * g + 4] : ext[s]);
      }
    }
  }

  // Pivot key of this lane's active rows: |a| bits with the low 6 mantissa bits replaced by
  // 63 - row, so one redux.sync.max picks the row of largest magnitude (up to a relative 2^-17),
  // ties to the lowest row.
  __device__ __forceinline__ uint32_t pivot_key(const bool (&act)[RPT]) const {
    uint32_t key = 0u;
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const uint32_t kb = ((__float_as_uint(A[s][0]) & 0x7fffffffu) & ~KMASK) | (KMASK - static_cast<uint32_t>(row(s)));
      key = max(key, act[s] ? kb : 0u);
    }
    return key;
  }

  // The owner lane stores registers 1..MC-1 of its row in slot pslot, then a 0, at urow (MC
  // floats, 16-byte aligned) with predicated vector stores; no branch on the owner.
  __device__ __forceinline__ void publish_row(float* urow, int pslot, bool is_owner) const {
    constexpr int NG = MC / 4;
    const uint32_t ua = static_cast<uint32_t>(__cvta_generic_to_shared(urow));
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 4 * g + q + 1;
        v[q] = j < MC ? A[0][j] : 0.f;
#pragma unroll
        for (int s = 1; s < RPT; ++s)
          if (pslot == s) v[q] = j < MC ? A[s][j] : 0.f;
      }
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %0, 0;\n @p st.shared.v4.f32 [%1], {%2, %3, %4, %5};\n}\n" ::"r"(
              static_cast<int>(is_owner)),
          "r"(ua + 16u * g), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3])
          : "memory");
    }
  }

  // ---- LU with the forward substitution of wf fused in --------------------------------------
  // wf: in, the FP32 right-hand side by row; out, the forward-eliminated values by row. On return
  // ybuf holds the same values in step order. Returns false on a zero or non-finite pivot.
  //
  // The pivot row's U part is published with predicated (branch-free) stores by its owner lane;
  // the next step's pivot reduction is issued as soon as the first column group is updated, so
  // its latency overlaps the rest of the update.
  __device__ __forceinline__ bool factor_fwd(float (&wf)[RPT]) {
    constexpr int NG = MC / 4;
    constexpr int C1 = (NG + 2) / 3, C2 = (2 * NG + 2) / 3;
    const int mm = m();
    float* ustage = w<float>(P.ml.ustage);
    float* lrow = w<float>(P.ml.lrow);
    float* pinv_s = w<float>(P.ml.pinv);
    float* ybuf = w<float>(P.ml.ybuf);
    int* piv = w<int>(P.ml.piv);
    const int LDL = P.ml.LDL;
    bool act[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      act[s] = row(s) < mm;
      step[s] = INT_MAX;
    }
    uint32_t gk = gmax_u32(pivot_key(act));
#pragma unroll 1
    for (int k = 0; k < mm; ++k) {
      if ((gk & ~KMASK) == 0u || (gk & ~KMASK) >= 0x7f800000u) return false;  // zero column, inf or nan
      const int p = static_cast<int>(KMASK - (gk & KMASK));
      const int owner = static_cast<int>(static_cast<unsigned>(p) % NT), pslot = static_cast<int>(static_cast<unsigned>(p) / NT);
      const bool is_owner = gt() == owner;
      float pv_mine = A[0][0], w_mine = wf[0];
#pragma unroll
      for (int s = 1; s < RPT; ++s)
        if (pslot == s) { pv_mine = A[s][0]; w_mine = wf[s]; }
      // publish the pivot row's U part (registers 1..MC-1) with predicated stores
      float* urow = ustage + k * LDU;
      publish_row(urow, pslot, is_owner);
      float pval, yk;
      if constexpr (G == 1) {
        pval = __shfl_sync(kFullMask, pv_mine, owner);
        yk = __shfl_sync(kFullMask, w_mine, owner);
      } else {
        float* pvb = reinterpret_cast<float*>(w<unsigned char>(P.ml.red) + 192) + 2 * (k & 1);
        if (is_owner) {
          pvb[0] = pv_mine;
          pvb[1] = w_mine;
        }
        gsync();  // the pivot, its right-hand side and the published row are visible to the group
        pval = pvb[0];
        yk = pvb[1];
      }
      const float pinv = __fdividef(1.f, pval);
      if (is_owner) {
        pinv_s[k] = pinv;
        ybuf[k] = yk;
        piv[k] = p;
      }
      float l[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) == p) {
          act[s] = false;
          step[s] = k;
        }
        l[s] = act[s] ? A[s][0] * pinv : 0.f;
        if (act[s]) {
          lrow[row(s) * LDL + k] = l[s];
          wf[s] = fmaf(-l[s], yk, wf[s]);
        }
      }
      if constexpr (G == 1) __syncwarp();
      // first group (holds the next pivot column), then the next step's pivot reduction, then
      // the rest of the update
      const float zero[RPT] = {};
      update_chunk<0, 1>(l, urow, zero);
      gk = gmax_u32(pivot_key(act));
      const int width = mm - 1 - k;
      update_chunk<1, C1>(l, urow, zero);
      if (4 * C1 < width) {
        update_chunk<C1, C2>(l, urow, zero);
        if (4 * C2 < width) update_chunk<C2, NG>(l, urow, zero);
      }
      if constexpr (G == 1) __syncwarp();
    }
    gsync();  // factors, step-ordered values and pivots visible to the group
    count(S_LU);
    return true;
  }


  // ---- Gauss-Jordan inverse (simplified-Newton form) ---------------------------------------
  // In-place Gauss-Jordan with implicit partial pivoting on the register rows (Gauss-Jordan
  // elimination with partial pivoting; e.g. Golub & Van Loan, Matrix Computations, 3.1 and
  // 3.4). Column k is eliminated at step k from the not-yet-used row of largest |A(:,k)|; every
  // other row is updated with l = A(r,k) / pivot, and the eliminated column is replaced by the
  // inverse's column k (-l, and 1 in the pivot row), shifted in at the end of the rotating
  // register window. Pivot rows keep their unscaled values; every later update preserves that
  // row's scale, so each row is multiplied by its pivot's reciprocal once at the end. After m
  // steps, register j of the row pivoted at step i holds inverse(i, p_(j - (MC - m))) where
  // p_k is the row pivoted at step k (registers below MC - m hold zeros). The rows are stored
  // to ustage (row-major by physical row) for apply_inverse. Returns false on a zero or
  // non-finite pivot.
  __device__ __forceinline__ bool invert() {
    constexpr int NG = MC / 4;
    const int mm = m();
    float* ustage = w<float>(P.ml.ustage);
    bool act[RPT];
    float pr[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      act[s] = row(s) < mm;
      step[s] = INT_MAX;
      pr[s] = 0.f;
    }
    uint32_t gk = gmax_u32(pivot_key(act));
#pragma unroll 1
    for (int k = 0; k < mm; ++k) {
      if ((gk & ~KMASK) == 0u || (gk & ~KMASK) >= 0x7f800000u) return false;  // zero column, inf or nan
      const int p = static_cast<int>(KMASK - (gk & KMASK));
      const int owner = static_cast<int>(static_cast<unsigned>(p) % NT), pslot = static_cast<int>(static_cast<unsigned>(p) / NT);
      const bool is_owner = gt() == owner;
      float pv_mine = A[0][0];
#pragma unroll
      for (int s = 1; s < RPT; ++s)
        if (pslot == s) pv_mine = A[s][0];
      float* urow = ustage + k * LDU;
      publish_row(urow, pslot, is_owner);
      float pval;
      if constexpr (G == 1) {
        pval = __shfl_sync(kFullMask, pv_mine, owner);
      } else {
        float* pvb = reinterpret_cast<float*>(w<unsigned char>(P.ml.red) + 192);
        if (is_owner) pvb[k & 1] = pv_mine;
        gsync();  // the pivot value and the published row are visible to the group
        pval = pvb[k & 1];
      }
      const float pinv = __fdividef(1.f, pval);
      float l[RPT], ext[RPT];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const bool piv_row = row(s) == p;
        if (piv_row) {
          act[s] = false;
          step[s] = k;
          pr[s] = pinv;
        }
        l[s] = piv_row ? 0.f : A[s][0] * pinv;
        ext[s] = piv_row ? 1.f : -l[s];
      }
      if constexpr (G == 1) __syncwarp();
      update_chunk<0, 1>(l, urow, ext);
      gk = gmax_u32(pivot_key(act));
      constexpr int C1 = (NG + 2) / 3, C2 = (2 * NG + 2) / 3;
      update_chunk<1, C1>(l, urow, ext);
      update_chunk<C1, C2>(l, urow, ext);
      update_chunk<C2, NG>(l, urow, ext);
      if constexpr (G == 1) __syncwarp();
    }
    if constexpr (G > 1) gsync();  // every warp is done reading the pivot rows
    // scaled rows to ustage (the pivot-row copies above are no longer needed)
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      if (row(s) < mm) {
        float4* dst = reinterpret_cast<float4*>(ustage + row(s) * LDU);
#pragma unroll
        for (int g = 0; g < NG; ++g)
          dst[g] = make_float4(A[s][4 * g] * pr[s], A[s][4 * g + 1] * pr[s], A[s][4 * g + 2] * pr[s],
                               A[s][4 * g + 3] * pr[s]);
      }
    }
    gsync();
    count(S_LU);
    return true;
  }

  // x = A^{-1} g with the stored Gauss-Jordan inverse (g, x by row). ybuf holds g in step order
  // after MC - m leading zeros; pinv is reused as the step-ordered result buffer.
  __device__ __forceinline__ void apply_inverse(const float (&gf)[RPT], double (&x)[RPT]) {
    constexpr int NG = MC / 4;
    const int mm = m();
    const int off = MC - mm;
    float* gs = w<float>(P.ml.ybuf);
    float* xs = w<float>(P.ml.pinv);
    const float* inv = w<float>(P.ml.ustage);
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < mm) gs[off + step[s]] = gf[s];
    gsync();
    float a0[RPT], a1[RPT], a2[RPT], a3[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) a0[s] = a1[s] = a2[s] = a3[s] = 0.f;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const float4 gv = reinterpret_cast<const float4*>(gs)[g];
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < mm) {
          const float4 av = reinterpret_cast<const float4*>(inv + row(s) * LDU)[g];
          a0[s] = fmaf(av.x, gv.x, a0[s]);
          a1[s] = fmaf(av.y, gv.y, a1[s]);
          a2[s] = fmaf(av.z, gv.z, a2[s]);
          a3[s] = fmaf(av.w, gv.w, a3[s]);
        }
      }
    }
    gsync();
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < mm) xs[step[s]] = (a0[s] + a1[s]) + (a2[s] + a3[s]);
    gsync();
#pragma unroll
    for (int s = 0; s < RPT; ++s) x[s] = row(s) < mm ? static_cast<double>(xs[row(s)]) : 0.0;
    gsync();
    count(S_SOLVE);
  }

  // ---- static-order sparse LU (SP) --------------------------------------------------------
  __device__ __forceinline__ const int32_t* lp(int32_t off) const { return P.mech.lu_prog + off; }

  // A = I - coef J(y) (FP32) into the filled pattern's entries: zero, unit diagonal, then the
  // Jacobian nonzeros through the sliced-ELL program (each slot's entry from the js_e table).
  __device__ __forceinline__ void newton_matrix_sp(const double (&y)[RPT], double coef) {
    const MechLayout& L = P.mech.L;
    const int mm = L.m;
    float* x32 = w<float>(P.ml.x32);
    float* d32 = w<float>(P.ml.d32);
    float* lu = w<float>(P.ml.lu);
    const float* keff32 = w<float>(P.ml.keff32);
    const int nz4 = (P.mech.lu.nnz + 3) >> 2;
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < mm) x32[row(s)] = static_cast<float>(y[s]);
    for (int e = lane; e < nz4; e += 32) reinterpret_cast<float4*>(lu)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    const int32_t* diag = lp(P.mech.lu.off_diag);
    for (int k = lane; k < mm; k += 32) lu[__ldg(diag + k)] = 1.f;
    const int32_t* rf_ptr = t<int32_t>(L.off_rf_ptr);
    const int16_t* rf_sp = t<int16_t>(L.off_rf_sp);
#pragma unroll 2
    for (int r = lane; r < L.R; r += 32) {
      const int f0 = rf_ptr[r], f1 = rf_ptr[r + 1];
      const float kr = keff32[r];
      if (f1 - f0 == 1) {
        d32[f0] = kr;
      } else if (f1 - f0 == 2) {
        const float xa = x32[rf_sp[f0]], xb = x32[rf_sp[f0 + 1]];
        d32[f0] = kr * xb;
        d32[f0 + 1] = kr * xa;
      } else {
        for (int f = f0; f < f1; ++f) {
          float dv = kr;
          for (int g = f0; g < f1; ++g)
            if (g != f) dv *= x32[rf_sp[g]];
          d32[f] = dv;
        }
      }
    }
    __syncwarp();
    const float c = static_cast<float>(coef);
    const int32_t* js_rc = t<int32_t>(L.off_js_rc);
    const int16_t* js_e = t<int16_t>(L.off_js_e);
    const int32_t* js_cnt = t<int32_t>(L.off_js_cnt);
    const int32_t* js_off = t<int32_t>(L.off_js_off);
    const int16_t* jse_f = t<int16_t>(L.off_jse_f);
    const float* jse_nu = t<float>(L.off_jse_nu32);
#pragma unroll 2
    for (int sl = 0; sl < L.NJS; ++sl) {
      const int rc = js_rc[sl * 32 + lane];
      const int cnt = js_cnt[sl];
      const int base = js_off[sl] + lane;
      float J0 = 0.f, J1 = 0.f;
      int cc = 0;
      for (; cc + 2 <= cnt; cc += 2) {
        const int e = base + 32 * cc;
        const int f0 = jse_f[e], f1 = jse_f[e + 32];
        J0 += jse_nu[e] * d32[f0];
        J1 += jse_nu[e + 32] * d32[f1];
      }
      if (cc < cnt) J0 += jse_nu[base + 32 * cc] * d32[jse_f[base + 32 * cc]];
      if (rc >= 0) {
        const int i = rc >> 16, j = rc & 0xffff;
        lu[js_e[sl * 32 + lane]] = (i == j ? 1.f : 0.f) - c * (J0 + J1);
      }
    }
    __syncwarp();
    count(S_JAC);
  }

  // In-place factorization P A P^T = L U in the static order: per step k the pivot's reciprocal
  // (kept in pinv for the back substitution), the column of L scaled by it, then the step's
  // trailing updates, lane-strided over the program's lists. Returns false on a zero or
  // non-finite pivot (the same for every lane: the pivot is one shared-memory word).
  __device__ __forceinline__ bool factor_sp() {
    const int mm = m();
    float* lu = w<float>(P.ml.lu);
    float* dinv = w<float>(P.ml.pinv);
    const SparseLuLayout& S = P.mech.lu;
    const int32_t* diag = lp(S.off_diag);
    const int32_t* lcp = lp(S.off_lc_ptr);
    const int32_t* lc = lp(S.off_lc);
    const int32_t* upp = lp(S.off_up_ptr);
    const int2* up = reinterpret_cast<const int2*>(lp(S.off_up));
#pragma unroll 1
    for (int k = 0; k < mm; ++k) {
      const float piv = lu[__ldg(diag + k)];
      if (!(fabsf(piv) > 0.f) || !(fabsf(piv) < INFINITY)) return false;
      const float rinv = __frcp_rn(piv);
      if (lane == 0) dinv[k] = rinv;
      const int a1 = __ldg(lcp + k + 1);
      for (int q = __ldg(lcp + k) + lane; q < a1; q += 32) {
        const int e = __ldg(lc + q) & 0xffff;
        lu[e] *= rinv;
      }
      __syncwarp();
      const int b1 = __ldg(upp + k + 1);
      for (int q = __ldg(upp + k) + lane; q < b1; q += 32) {
        const int2 op = __ldg(up + q);
        const int dst = op.x & 0xffff, l = static_cast<int>(static_cast<uint32_t>(op.x) >> 16);
        lu[dst] = fmaf(-lu[l], lu[op.y], lu[dst]);
      }
      __syncwarp();
    }
    count(S_LU);
    return true;
  }

  // x = A^{-1} g with the sparse factors (g, x by row): g scattered to position order in ybuf,
  // forward substitution by columns of L, back substitution by columns of U (x_k = z_k / u_kk).
  __device__ __forceinline__ void solve_sp(const float (&gf)[RPT], double (&x)[RPT]) {
    const int mm = m();
    const float* lu = w<float>(P.ml.lu);
    const float* dinv = w<float>(P.ml.pinv);
    float* wv = w<float>(P.ml.ybuf);
    const SparseLuLayout& S = P.mech.lu;
    const int32_t* pos = lp(S.off_pos);
    const int32_t* lcp = lp(S.off_lc_ptr);
    const int32_t* lc = lp(S.off_lc);
    const int32_t* ucp = lp(S.off_uc_ptr);
    const int32_t* uc = lp(S.off_uc);
    int ps[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      ps[s] = row(s) < mm ? __ldg(pos + row(s)) : 0;
      if (row(s) < mm) wv[ps[s]] = gf[s];
    }
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < mm; ++k) {
      const float zk = wv[k];
      const int a1 = __ldg(lcp + k + 1);
      for (int q = __ldg(lcp + k) + lane; q < a1; q += 32) {
        const int v = __ldg(lc + q);
        const int i = static_cast<int>(static_cast<uint32_t>(v) >> 16);
        wv[i] = fmaf(-lu[v & 0xffff], zk, wv[i]);
      }
      __syncwarp();
    }
#pragma unroll 1
    for (int k = mm - 1; k >= 0; --k) {
      const float xk = wv[k] * dinv[k];
      const int a1 = __ldg(ucp + k + 1);
      for (int q = __ldg(ucp + k) + lane; q < a1; q += 32) {
        const int v = __ldg(uc + q);
        const int i = static_cast<int>(static_cast<uint32_t>(v) >> 16);
        wv[i] = fmaf(-lu[v & 0xffff], xk, wv[i]);
      }
      __syncwarp();
      if (lane == 0) wv[k] = xk;  // after every lane has read z_k
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < RPT; ++s) x[s] = row(s) < mm ? static_cast<double>(wv[ps[s]]) : 0.0;
    __syncwarp();
    count(S_SOLVE);
  }

  // Forward substitution with the stored multipliers (rows' values in wf, in place); leaves the
  // values in step order in ybuf.
  __device__ __forceinline__ void forward(float (&wf)[RPT]) {
    const int mm = m();
    const float* lrow = w<float>(P.ml.lrow);
    const int* piv = w<int>(P.ml.piv);
    float* ybuf = w<float>(P.ml.ybuf);
    const int LDL = P.ml.LDL;
#pragma unroll 1
    for (int k = 0; k < mm; ++k) {
      const int p = piv[k];
      float yk;
      if constexpr (G == 1) {
        float mine = 0.f;
#pragma unroll
        for (int s = 0; s < RPT; ++s)
          if ((p >> 5) == s) mine = wf[s];
        yk = __shfl_sync(kFullMask, mine, p & 31);
      } else {
        // the pivot row's value is final at its step: its owner writes it where the others read it
        if (gt() == p % NT) ybuf[k] = wf[0];
        gsync();
        yk = ybuf[k];
      }
#pragma unroll
      for (int s = 0; s < RPT; ++s)
        if (step[s] > k && row(s) < mm) wf[s] = fmaf(-lrow[row(s) * LDL + k], yk, wf[s]);
    }
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < mm) ybuf[step[s]] = wf[s];
    gsync();
  }

  // Back substitution from ybuf (values in step order) to x in species order.
  __device__ __forceinline__ void backward(double (&x)[RPT]) {
    const int mm = m();
    const float* ustage = w<float>(P.ml.ustage);
    const float* ybuf = w<float>(P.ml.ybuf);
    const float* pinv_s = w<float>(P.ml.pinv);
    float ys[RPT], pv[RPT], xs[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      ys[s] = row(s) < mm ? ybuf[row(s)] : 0.f;
      pv[s] = row(s) < mm ? pinv_s[row(s)] : 0.f;
      xs[s] = 0.f;
    }
    gsync();
    float* xb = w<float>(P.ml.ybuf);  // G > 1: x_k by step, for the group (ybuf is read above)
#pragma unroll 1
    for (int k = mm - 1; k >= 0; --k) {
      float xk;
      if constexpr (G == 1) {
        float mine = 0.f;
#pragma unroll
        for (int s = 0; s < RPT; ++s)
          if ((k >> 5) == s) mine = ys[s] * pv[s];
        xk = __shfl_sync(kFullMask, mine, k & 31);
      } else {
        if (gt() == k % NT) xb[k] = ys[0] * pv[0];
        gsync();
        xk = xb[k];
      }
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        const int i = row(s);
        if (i < k) ys[s] = fmaf(-ustage[i * (LDU - 1) + k - 1], xk, ys[s]);
        if (i == k) xs[s] = xk;
      }
    }
#pragma unroll
    for (int s = 0; s < RPT; ++s) x[s] = static_cast<double>(xs[s]);
    gsync();  // ybuf is reused by the next solve
    count(S_SOLVE);
  }

  // ---- Newton on y - coef f(y) = rhs --------------------------------------------------------
  __device__ __forceinline__ bool newton(double (&y)[RPT], const double (&rv)[RPT], double coef, int max_newton,
                                         int jac_interval, double atol, double rtol) {
    for (int it = 0; it < max_newton; ++it) {
      double f[RPT], dx[RPT], g[RPT];
      float wf[RPT];
      rhs(y, f);
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        g[s] = -((y[s] - coef * f[s]) - rv[s]);
        wf[s] = static_cast<float>(g[s]);
      }
      if (it % jac_interval == 0) {
        newton_matrix(y, coef);
        put(V_YGP, y);  // the point of the factored Jacobian, for the refinement residual
        if (!factor_fwd(wf)) return false;
      } else {
        forward(wf);
      }
      backward(dx);
      {
        // one sweep of iterative refinement: FP64 residual of (I - c J) dx = g, FP32 correction
        double jd[RPT], corr[RPT];
        jvec(dx, jd);
#pragma unroll
        for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(g[s] - (dx[s] - coef * jd[s]));
        forward(wf);
        backward(corr);
#pragma unroll
        for (int s = 0; s < RPT; ++s) dx[s] += corr[s];
      }
      count(S_NEWTON);
      double sdx = 0.0, sy = 0.0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m()) {
          y[s] += dx[s];
          sdx += dx[s] * dx[s];
          sy += y[s] * y[s];
        }
      }
      const double ndx = sqrt(gsum_f64(sdx)), ny = sqrt(gsum_f64(sy));
      if (!isfinite(ndx) || !isfinite(ny)) return false;
      if (ndx <= atol + rtol * ny) return true;
    }
    return false;
  }

  // ---- simplified Newton on y - coef f(y) = rhs with the stored inverse --------------------
  // The inverse of I - c_inv J (carried, or formed here at the first iterate) serves every
  // iteration; it is re-formed once per stage at the current iterate when the max-norm of the
  // correction (rounded to FP32) shrinks by less than half. Converged when every
  // |dx_i| <= atol / sqrt(m) + rtol |y_i|, which implies the reference's 2-norm test
  // (||dx|| <= atol + rtol ||y||, Minkowski's inequality); no FP64 reduction, division or square
  // root per iteration.
  __device__ __forceinline__ bool newton_simplified(double (&y)[RPT], const double (&rv)[RPT], double coef,
                                                    int max_newton, double atol_c, double rtol) {
    float prev = 0.f;
    bool refresh = !have_inv;
    for (int it = 0; it < max_newton; ++it) {
      double f[RPT], dx[RPT];
      float wf[RPT];
      rhs(y, f);
#pragma unroll
      for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(-((y[s] - coef * f[s]) - rv[s]));
      if (refresh) {
        newton_matrix(y, coef);
        if (!invert()) return false;
        have_inv = true;
        fresh = true;
        refresh = false;
        c_inv = coef;
      }
      apply_inverse(wf, dx);
      count(S_NEWTON);
      bool finite = true, conv = true;
      uint32_t dbits = 0u;  // |dx| rounded to FP32: non-negative floats order like their bits
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m()) {
          y[s] += dx[s];
          finite = finite && isfinite(dx[s]) && isfinite(y[s]);
          conv = conv && fabs(dx[s]) <= atol_c + rtol * fabs(y[s]);
          dbits = max(dbits, __float_as_uint(static_cast<float>(fabs(dx[s]))));
        }
      }
      bool all_finite, all_conv;
      float dmax;
      if constexpr (G == 1) {
        all_finite = __all_sync(kFullMask, finite);
        dmax = __uint_as_float(__reduce_max_sync(kFullMask, dbits));
        all_conv = __all_sync(kFullMask, conv);
      } else {
        const uint32_t flags = gor_u32((finite ? 0u : 1u) | (conv ? 0u : 2u));
        all_finite = !(flags & 1u);
        all_conv = !(flags & 2u);
        dmax = __uint_as_float(gmax_u32(dbits));
      }
      if (!all_finite) return false;
      if (it > 0 && !fresh && dmax > 0.5f * prev) refresh = true;
      prev = dmax;
      if (all_conv) return true;
    }
    return false;
  }

  // x = A^{-1} g with the current FP32 factors: the Gauss-Jordan inverse or the sparse LU.
  __device__ __forceinline__ void lin_solve(const float (&gf)[RPT], double (&x)[RPT]) {
    if constexpr (SP) {
      solve_sp(gf, x);
    } else {
      apply_inverse(gf, x);
    }
  }

  // ---- full Newton with the Gauss-Jordan inverse and one refinement sweep per solve --------
  __device__ __forceinline__ bool newton_full_gj(double (&y)[RPT], const double (&rv)[RPT], double coef,
                                                 int max_newton, int jac_interval, double atol, double rtol) {
    for (int it = 0; it < max_newton; ++it) {
      double f[RPT], dx[RPT], g[RPT], jd[RPT], corr[RPT];
      float wf[RPT];
      rhs(y, f);
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        g[s] = -((y[s] - coef * f[s]) - rv[s]);
        wf[s] = static_cast<float>(g[s]);
      }
      if (it % jac_interval == 0) {
        put(V_YGP, y);  // the point of the factored Jacobian, for the refinement residual
        if constexpr (SP) {
          newton_matrix_sp(y, coef);
          if (!factor_sp()) return false;
        } else {
          newton_matrix(y, coef);
          if (!invert()) return false;
        }
      }
      lin_solve(wf, dx);
      // refinement: FP64 residual of (I - c J) dx = g, correction through the FP32 factors
      jvec(dx, jd);
#pragma unroll
      for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(g[s] - (dx[s] - coef * jd[s]));
      lin_solve(wf, corr);
      count(S_NEWTON);
      double sdx = 0.0, sy = 0.0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m()) {
          dx[s] += corr[s];
          y[s] += dx[s];
          sdx += dx[s] * dx[s];
          sy += y[s] * y[s];
        }
      }
      const double ndx = sqrt(gsum_f64(sdx)), ny = sqrt(gsum_f64(sy));
      if (!isfinite(ndx) || !isfinite(ny)) return false;
      if (ndx <= atol + rtol * ny) return true;
    }
    return false;
  }

  // Stores a row-distributed vector into the shared stage-vector slot v.
  __device__ __forceinline__ void put(int v, const double (&a)[RPT]) const {
#pragma unroll
    for (int s = 0; s < RPT; ++s)
      if (row(s) < m()) vec(v, row(s)) = a[s];
  }

  // ---- TR-BDF2 (the algorithm of the plain kernel and of the oracle) ------------------------
  __device__ __forceinline__ int integrate(double (&y)[RPT], double t_beg, double t_end, double dt_in, double dt_min,
                                           double dt_max, int max_iters, int max_newton, int jac_interval,
                                           double natol, double nrtol, double& t_out, double& dt_out) {
    if (dt_in < 0.0) return TCHEM_GB_SAMPLE_NEGATIVE_DT;
    const double gamma = 2.0 - sqrt(2.0);
    const double d = 0.5 * gamma;
    const double cg = 1.0 / (gamma * (2.0 - gamma));
    const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
    const double kappa = (-3.0 * gamma * gamma + 4.0 * gamma - 2.0) / (12.0 * (2.0 - gamma));
    const double e0 = 1.0 / gamma, e1 = -1.0 / (gamma * (1.0 - gamma)), e2 = 1.0 / (1.0 - gamma);
    double yg[RPT], y1[RPT];
    double t = t_beg, dt = dt_in;
    double dtp = 0.0;  // simplified form: last accepted step size (V_YP / V_YGP valid when have_prev)
    bool have_prev = false;
    const double natol_c = natol / sqrt(static_cast<double>(m()));
    int status = TCHEM_GB_SAMPLE_OK;
    {
      double fn[RPT];
      rhs(y, fn);
      put(V_FN, fn);
    }
    for (int iter = 0; iter < max_iters && t < t_end; ++iter) {
      bool converged = false, last = false;
      for (int ntry = 0; ntry < 4; ++ntry) {
        dt = fmin(fmax(dt, dt_min), dt_max);
        last = dt >= t_end - t;
        if (last) dt = t_end - t;
        if (!(dt > 0.0)) { status = TCHEM_GB_SAMPLE_DT_UNDERFLOW; break; }
        const double coef = d * dt;
        if constexpr (kSimplifiedNewton) {
          // keep the carried inverse while c moved by at most 30%
          if (!(have_inv && fabs(coef / c_inv - 1.0) <= 0.3)) have_inv = false;
        }
        // Both implicit stages run through one copy of the Newton code.
        bool ok = true;
#pragma unroll 1
        for (int stage = 0; stage < 2 && ok; ++stage) {
          double guess[RPT], rv[RPT];
#pragma unroll
          for (int s = 0; s < RPT; ++s) {
            const int i = row(s) < m() ? row(s) : 0;
            rv[s] = stage == 0 ? y[s] + coef * vec(V_FN, i) : cg * yg[s] - cn * y[s];
            guess[s] = stage == 0 ? y[s] : yg[s];
          }
          if constexpr (kSimplifiedNewton) {
            if (stage == 0 && have_prev) {
              // stage-1 guess: the quadratic through the last step's y_{n-1}, y_{n-1+gamma}, y_n
              const double t0 = -dtp, t1 = -(1.0 - gamma) * dtp, tt = gamma * dt;
              const double l0 = (tt - t1) * tt / ((t0 - t1) * t0);
              const double l1 = (tt - t0) * tt / ((t1 - t0) * t1);
              const double l2 = (tt - t0) * (tt - t1) / (t0 * t1);
#pragma unroll
              for (int s = 0; s < RPT; ++s) {
                const int i = row(s) < m() ? row(s) : 0;
                guess[s] = l0 * vec(V_YP, i) + l1 * vec(V_YGP, i) + l2 * y[s];
              }
            } else if (stage == 1) {
              // stage-2 guess: the quadratic with p(t) = y_n, p'(t) = f_n, p(t + gamma dt) = y_gamma
              const double a = 1.0 / (gamma * gamma), b = dt * (1.0 - 1.0 / gamma);
#pragma unroll
              for (int s = 0; s < RPT; ++s) {
                const int i = row(s) < m() ? row(s) : 0;
                guess[s] = (1.0 - a) * y[s] + a * yg[s] + b * vec(V_FN, i);
              }
            }
            fresh = false;
            ok = newton_simplified(guess, rv, coef, max_newton, natol_c, nrtol);
          } else if constexpr (SIMP) {
            ok = newton_full_gj(guess, rv, coef, max_newton, jac_interval, natol, nrtol);
          } else {
            ok = newton(guess, rv, coef, max_newton, jac_interval, natol, nrtol);
          }
          if (ok) {
#pragma unroll
            for (int s = 0; s < RPT; ++s) {
              if (stage == 0) yg[s] = guess[s];
              else y1[s] = guess[s];
            }
            if (stage == 0) {
              double fg[RPT];
              rhs(yg, fg);
              put(V_FG, fg);
            }
          }
        }
        if (ok) { converged = true; break; }
        count(S_NFAIL);
        dt *= 0.5;
      }
      if (status != TCHEM_GB_SAMPLE_OK) break;
      if (!converged) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
      double f1[RPT], estf[RPT];
      rhs(y1, f1);
      {
        double est[RPT];
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          const int i = row(s) < m() ? row(s) : 0;
          est[s] = 2.0 * kappa * dt * (e0 * vec(V_FN, i) + e1 * vec(V_FG, i) + e2 * f1[s]);
        }
        float wf[RPT];
#pragma unroll
        for (int s = 0; s < RPT; ++s) wf[s] = static_cast<float>(est[s]);
        if constexpr (FULLGJ) {
          // filter with the last Newton iteration's factors (the reference's matrix)
          lin_solve(wf, estf);
        } else if constexpr (SIMP) {
          // filter with I - c J(y_{n+1}); the inverse is carried into the next step
          newton_matrix(y1, d * dt);
          if (invert()) {
            have_inv = true;
            c_inv = d * dt;
            apply_inverse(wf, estf);
          } else {
            have_inv = false;
#pragma unroll
            for (int s = 0; s < RPT; ++s) estf[s] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: status 4
          }
        } else {
          forward(wf);
          backward(estf);
        }
      }
      double err = 0.0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        if (row(s) < m()) {
          const double wgt = vec(V_ATOL, row(s)) + vec(V_RTOL, row(s)) * fmax(fabs(y[s]), fabs(y1[s]));
          err = fmax(err, fabs(estf[s]) / wgt);
        }
      }
      err = gmax_f64(err);
      if (!isfinite(err)) { status = TCHEM_GB_SAMPLE_NONFINITE; break; }
      if (err <= 1.0 || dt <= dt_min) {
        t = last ? t_end : t + dt;
        if constexpr (kSimplifiedNewton) {
          put(V_YP, y);
          put(V_YGP, yg);
          dtp = dt;
          have_prev = true;
        }
#pragma unroll
        for (int s = 0; s < RPT; ++s) y[s] = y1[s];
        put(V_FN, f1);
        count(S_STEPS);
        double fac = err > 0.0 ? 0.9 * cbrt(1.0 / err) : 2.0;
        fac = fmax(0.2, fmin(2.0, fac));
        dt = fmin(dt * fac, dt_max);
        if (t + dt > t_end) dt = t_end - t;
      } else {
        count(S_REJ);
        dt *= fmax(0.2, 0.9 * cbrt(1.0 / err));
      }
      gsync();
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

// One sample per group of G warps (G = 1: one warp), persistent work queue (same outer protocol as
// the plain kernel).
// Shapes with one row per thread hold half the matrix registers of the two-rows-per-lane shapes,
// so they fit 168 registers and run 12 warps per SM (the 52-column two-warp shape 128 registers
// and 16 warps); the others run 8. The sparse-LU shapes hold no matrix registers: 16 warps for up
// to 64 species (shared memory then limits the samples per CTA), 8 for up to 128.
template <int MC, int RPT, bool SIMP, int G, bool FULLGJ = false, bool E3 = false, bool SP = false>
constexpr int max_threads() {
  if (SP) return RPT <= 2 ? 512 : 256;
  return (RPT == 1 && MC <= 52 && G == 2) ? 512 : ((RPT == 1 && MC <= 64) ? 384 : 256);
}

template <int MC, int RPT, bool SIMP, int G, bool FULLGJ = false, bool E3 = false, bool SP = false>
__global__ void __launch_bounds__(max_threads<MC, RPT, SIMP, G, FULLGJ, E3, SP>(), 1)
    trbdf2_mixed_kernel(const __grid_constant__ AdvanceParams P) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  unsigned char* tables = smem + 16;
  const MechLayout& L = P.mech.L;
  if (!stage_to_smem(tables, P.mech.blob, static_cast<uint32_t>(L.blob_bytes), mbar)) {
    if (threadIdx.x == 0) atomicOr(P.error_word, kErrBarrierTimeout);
    return;
  }
  constexpr int NT = 32 * G;
  const int group = threadIdx.x / NT, tid = threadIdx.x % NT, lane = threadIdx.x & 31;
  Solver<MC, RPT, SIMP, G, FULLGJ, E3, SP> S{P, tables, tables + L.blob_bytes + group * P.ml.warp_bytes, lane, tid, tid >> 5,
                             1 + group};
  const int m = L.m;
  const int n_items = P.n_items_dev ? *P.n_items_dev : P.n_items;
  int* stats = S.template w<int>(P.ml.stats);
  double* keff = S.template w<double>(P.ml.keff);
  float* keff32 = S.template w<float>(P.ml.keff32);
  int* item_s = S.template w<int>(P.ml.item);

  while (true) {
    if (tid == 0) item_s[0] = atomicAdd(P.queue, 1);
    S.gsync();
    const int item = item_s[0];
    S.gsync();
    if (item >= n_items) break;
    const int smp = P.items ? P.items[item] : item;
    const tchem_gb_tadv ta = P.tadv[smp];
    if (P.t_out[smp] >= ta.tend) {
      if (tid == 0) {
        P.status[smp] = TCHEM_GB_SAMPLE_SKIPPED;
        if (P.stats) P.stats[smp] = tchem_gb_sample_stats{};
      }
      continue;
    }
    const int gm = P.mech_of_sample ? P.mech_of_sample[smp] : 0;
    const int slot = (gm >= 0 && gm < kMaxMechs) ? P.slot_of_mech[gm] : -1;
    if (slot < 0) {
      if (tid == 0) P.status[smp] = TCHEM_GB_SAMPLE_BAD_MECH;
      continue;
    }
    const double* row = P.state + static_cast<size_t>(smp) * P.state_dim;
    const double p = row[1], Tk = row[2];
    if constexpr (E3) {
      for (int r = tid; r < L.R; r += NT) {
        const double k = P.keff_in[static_cast<size_t>(smp) * L.R + r];
        keff[r] = k;
        keff32[r] = static_cast<float>(k);
      }
      double* src = S.template w<double>(P.ml.src);
      for (int i = tid; i < m; i += NT) src[i] = P.src_in[smp * P.src_stride + i];
    } else {
      const double t_1 = 1.0 / Tk;
      const double conv = P.mech.conv_ppm * p * t_1;
      const double* rp = P.rate_param[slot];
      for (int r = tid; r < L.R; r += NT) {
        double k = rate_constant(P.mech.rate_type[r], rp + 8 * r, P.mech.conv_exp[r], Tk, t_1, p, conv);
        for (int c = P.mech.cf_ptr[r]; c < P.mech.cf_ptr[r + 1]; ++c) k *= row[3 + m + P.mech.cf_idx[c]];
        keff[r] = k;
        keff32[r] = static_cast<float>(k);
      }
    }
    for (int i = tid; i < m; i += NT) {
      S.vec(V_ATOL, i) = P.tol_time[2 * i];
      S.vec(V_RTOL, i) = P.tol_time[2 * i + 1];
    }
    if (tid < 8) stats[tid] = 0;
    if (tid == 0) {
      S.template w<double>(P.ml.q)[L.R] = 0.0;
      S.template w<float>(P.ml.d32)[L.NF] = 0.f;
    }
    if constexpr (SIMP)
      for (int j = tid; j < MC; j += NT) S.template w<float>(P.ml.ybuf)[j] = 0.f;  // leading zeros of apply_inverse
    S.have_inv = false;
    S.gsync();
    double y[RPT];
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
      const int i = S.row(s);
      y[s] = (i < m) ? row[3 + i] : 0.0;
    }
    double t_o = 0.0, dt_o = 0.0;
    const int jac_int = ta.jacobian_interval > 0 ? ta.jacobian_interval : 1;
    const int stt = S.integrate(y, ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax, ta.num_time_iterations_per_interval,
                                ta.max_num_newton_iterations, jac_int, P.tol_newton[0], P.tol_newton[1], t_o, dt_o);
    S.gsync();
    if (tid == 0) {
      P.status[smp] = stt;
      if (P.stats) {
        tchem_gb_sample_stats sst;
        sst.n_steps = stats[S_STEPS];
        sst.n_rejected = stats[S_REJ];
        sst.n_newton_fail = stats[S_NFAIL];
        sst.n_newton_iter = stats[S_NEWTON];
        sst.n_lu = stats[S_LU];
        sst.n_solve = stats[S_SOLVE];
        sst.n_rhs = stats[S_RHS];
        sst.n_jac = stats[S_JAC];
        P.stats[smp] = sst;
      }
    }
    if (stt != TCHEM_GB_SAMPLE_NEGATIVE_DT) {
      double* out = P.state_out + static_cast<size_t>(smp) * P.state_dim;
      for (int i = tid; i < P.state_dim - 3 - m; i += NT) out[3 + m + i] = row[3 + m + i];
      if (tid == 0) {
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
    S.gsync();
  }
}

}  // namespace mixed
}  // namespace tchem_gb
