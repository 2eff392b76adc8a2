// Tensor-core TR-BDF2 form for large mechanisms (129 to 320 active species): the time advance of
// TChem::AtmosphericChemistry::runDeviceBatch (src/core/TChem_AtmosphericChemistry.cpp:42-167,
// integrator call src/core/problems/TChem_Impl_AtmosphericChemistry.hpp:138-155) for mechanisms
// whose Newton matrix is too large for registers or shared memory (300 x 300 FP32 = 360 KB).
//
// One CTA of four warps per sample, persistent over a work queue. Full Newton with the reference's
// jacobian_interval, the same TR-BDF2 step control as the plain form (fp64_core.cuh); FP64 state,
// right-hand side, Newton residual, error estimate and step control. The Newton matrix
// I - c J(y) is formed in FP32 in the CTA's slot in global memory (L2-resident) and factored by a
// blocked right-looking LU with partial pivoting:
//   * each 32-column panel is loaded into shared memory and factored on the CUDA cores (pivot
//     search by warp shuffles and one cross-warp exchange per column; row exchanges are logical,
//     through a permutation, so no matrix row moves);
//   * U12 = L11^-1 A12 on the CUDA cores, written to the matrix and, as the MMA's B operand, to
//     shared memory in the K-major canonical layout; L21 likewise as the A operand;
//   * the trailing update A22 -= L21 U12 on the tensor cores: tiles of 128 rows x up to 256
//     columns, four tcgen05.mma.kind::tf32 (K = 8 each) per tile into one of two TMEM buffers,
//     the next tile's MMAs issued before the current tile is drained (tcgen05.ld, then A22 -= P
//     in place in global memory).
// Each Newton solve runs forward and back substitution on the CUDA cores (32-row diagonal blocks
// by one warp with shuffles, the off-diagonal blocks as matrix-vector products over the CTA) in
// FP32, followed by one sweep of iterative refinement with an FP64 residual (an FP64
// Jacobian-vector product at the matrix's point), so the Newton iterates follow the FP64 form's.
// Every wait on an MMA is bounded; on expiry the kernel records kErrBarrierTimeout, stops taking
// samples, drains with a second bounded window and frees its TMEM.
#include <cuda_runtime.h>

#include <algorithm>

#include "advance.hpp"
#include "capi_internal.hpp"
#include "engine.cuh"
#include "kernels.hpp"
#include "tc_tile.cuh"

namespace tchem_gb {
namespace tcadv {

constexpr int kNT = 128;                     // threads per CTA (one warpgroup: TMEM lanes 0..127)
constexpr int kMaxM = 320;                   // largest system
constexpr int kLda = 320;                    // row stride of the global matrix (floats)
constexpr int kPW = 32;                      // panel width = K of the trailing update
constexpr int kPLd = 36;                     // pivot-row stride in shared memory (floats, 16-byte rows)
constexpr int kRowsPT = (kMaxM + kNT - 1) / kNT;  // panel rows per thread
constexpr int kMaxTrail = kMaxM - kPW;       // widest trailing matrix
constexpr int kRowTiles = (kMaxTrail + 127) / 128;
constexpr int kBTileRows = 288;              // B operand rows (trailing columns, padded to 16)
constexpr uint32_t kTmemCols = 512;          // two accumulator buffers of 256 columns

// Vector slots (FP64, kMaxM each) of the per-sample working set.
enum Vec { V_Y, V_FN, V_FG, V_F1, V_YG, V_Y1, V_RV, V_G, V_DX, V_R, V_EST, V_ATOL, V_RTOL, V_YJ, V_F, kNumVec };

}  // namespace tcadv

size_t tc_advance_smem_bytes(const MechLayout& L) {
  using namespace tcadv;
  auto up128 = [](size_t b) { return (b + 127) & ~size_t(127); };
  size_t b = 1024;                                        // mbarriers, TMEM slot, reductions, flags
  b += up128(sizeof(float) * (kPW + 8) * kPLd);           // the panel's pivot rows + pivot candidates
  b += static_cast<size_t>(kRowTiles) * 128 * kPW * 4;    // A operand (L21), K-major
  b += static_cast<size_t>(kBTileRows) * kPW * 4;         // B operand (U12), K-major
  b += up128(sizeof(double) * kNumVec * kMaxM);           // vectors
  b += up128(sizeof(double) * L.R) * 2;                   // keff, q
  b += up128(sizeof(float) * L.NF);                       // d32
  b += up128(sizeof(float) * kMaxM);                      // w32 (solve vector)
  b += up128(sizeof(int32_t) * kMaxM);                    // perm
  return b;
}

namespace tcadv {

struct Layout {
  uint32_t panel, aop, bop, vec, keff, q, d32, w32, perm, bytes;
};

__device__ __forceinline__ Layout layout(const MechLayout& L) {
  auto up128 = [](uint32_t b) { return (b + 127u) & ~127u; };
  Layout s;
  uint32_t o = 1024;
  s.panel = o;
  o += up128(sizeof(float) * (kPW + 8) * kPLd);
  s.aop = o;  // 1024-byte aligned: the operand base offsets below are multiples of 16
  o += kRowTiles * 128 * kPW * 4;
  s.bop = o;
  o += kBTileRows * kPW * 4;
  s.vec = o;
  o += up128(sizeof(double) * kNumVec * kMaxM);
  s.keff = o;
  o += up128(sizeof(double) * L.R);
  s.q = o;
  o += up128(sizeof(double) * L.R);
  s.d32 = o;
  o += up128(sizeof(float) * L.NF);
  s.w32 = o;
  o += up128(sizeof(float) * kMaxM);
  s.perm = o;
  o += up128(sizeof(int32_t) * kMaxM);
  s.bytes = o;
  return s;
}

// Shared-memory header (first 1024 bytes).
struct Header {
  uint64_t mbar[2];      // MMA completion, one per TMEM buffer
  uint32_t tmem_slot;    // address written by tcgen05.alloc
  int32_t item;          // current work item (broadcast)
  int32_t abort;         // a bounded wait expired: stop taking samples
  int32_t pad;
  double redd[2][4];     // double reductions, two rotating halves
  float redf[2][4];      // pivot candidates |a|
  int32_t redi[2][4];    // pivot candidate rows
  int32_t pphys[32];     // physical matrix row of the panel's pivot at each step
  int32_t scnt[3][4];    // non-pivot rows per (row segment, warp): the trailing-order scan
};

struct Solver {
  const AdvanceParams& P;
  unsigned char* sm;
  Header* H;
  SmemTables T;  // the mechanism's tables, read from global memory (L1/L2)
  float* A;      // this CTA's matrix slot [kMaxM][kLda]
  float* pn;     // the current panel's pivot rows [kPW][kPLd] in step order, then the pivot
                 // candidates [2][4][kPLd] (step parity, warp)
  unsigned char* aop;
  unsigned char* bop;
  double* vecs;
  double* keff;
  double* q;
  float* d32;
  float* w32;
  int32_t* perm;
  int m, R, tid, lane, warp;
  uint32_t tmem;
  uint32_t phbits = 0u;  // bit b: the parity to wait for next on TMEM buffer b (a scalar: the struct stays in registers)
  int rr = 0;  // rotating reduction half
  tchem_gb_sample_stats st{};

  __device__ double* v(int i) const { return vecs + static_cast<size_t>(i) * kMaxM; }

  // ---- block reductions (one barrier each; two rotating halves keep back-to-back reductions safe)
  __device__ double bsum(double x) {
    x = warp_sum(x);
    double* r = H->redd[rr];
    rr ^= 1;
    if (lane == 0) r[warp] = x;
    __syncthreads();
    return (r[0] + r[1]) + (r[2] + r[3]);
  }
  __device__ double bmax(double x) {
    x = warp_max(x);
    double* r = H->redd[rr];
    rr ^= 1;
    if (lane == 0) r[warp] = x;
    __syncthreads();
    return fmax(fmax(r[0], r[1]), fmax(r[2], r[3]));
  }

  // ---- FP64 right-hand side f = omega(y): src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:80-138
  __device__ void rhs(const double* y, double* f) {
    for (int r = tid; r < R; r += kNT) {
      double qq = keff[r];
      const int g1 = __ldg(T.rf_ptr + r + 1);
      for (int g = __ldg(T.rf_ptr + r); g < g1; ++g) qq *= y[__ldg(T.rf_sp + g)];
      q[r] = qq;
    }
    __syncthreads();
    for (int i = tid; i < m; i += kNT) {
      double acc = __ldg(T.emis + i);
      const int e1 = __ldg(T.pr_ptr + i + 1);
      for (int e = __ldg(T.pr_ptr + i); e < e1; ++e) acc += __ldg(T.pr_nu + e) * q[__ldg(T.pr_r + e)];
      f[i] = acc;
    }
    __syncthreads();
    ++st.n_rhs;
  }

  // ---- FP64 Jacobian-vector product out = J(xj) vv (the refinement residual), no emissions
  __device__ void jvec(const double* xj, const double* vv, double* out) {
    for (int r = tid; r < R; r += kNT) {
      const int g0 = __ldg(T.rf_ptr + r), g1 = __ldg(T.rf_ptr + r + 1);
      double dq = 0.0;
      for (int f = g0; f < g1; ++f) {
        double p = vv[__ldg(T.rf_sp + f)];
        for (int g = g0; g < g1; ++g)
          if (g != f) p *= xj[__ldg(T.rf_sp + g)];
        dq += p;
      }
      q[r] = keff[r] * dq;
    }
    __syncthreads();
    for (int i = tid; i < m; i += kNT) {
      double acc = 0.0;
      const int e1 = __ldg(T.pr_ptr + i + 1);
      for (int e = __ldg(T.pr_ptr + i); e < e1; ++e) acc += __ldg(T.pr_nu + e) * q[__ldg(T.pr_r + e)];
      out[i] = acc;
    }
    __syncthreads();
    ++st.n_rhs;  // counted like a right-hand side
  }

  // ---- FP32 Newton matrix I - c J(y) into the global slot; the permutation reset to identity
  __device__ void newton_matrix(const double* y, double coef) {
    for (int r = tid; r < R; r += kNT) {
      const int f0 = __ldg(T.rf_ptr + r), f1 = __ldg(T.rf_ptr + r + 1);
      for (int f = f0; f < f1; ++f) {
        double dv = keff[r];
        for (int g = f0; g < f1; ++g)
          if (g != f) dv *= y[__ldg(T.rf_sp + g)];
        d32[f] = static_cast<float>(dv);
      }
    }
    const int m4 = (m + 3) / 4;  // float4 columns; kLda = 320 keeps every row 16-byte aligned
    for (int e = tid; e < m * m4; e += kNT) {
      const int i = e / m4, j4 = 4 * (e - i * m4);
      float4 w = make_float4(i == j4 ? 1.f : 0.f, i == j4 + 1 ? 1.f : 0.f, i == j4 + 2 ? 1.f : 0.f,
                             i == j4 + 3 ? 1.f : 0.f);
      *reinterpret_cast<float4*>(A + static_cast<size_t>(i) * kLda + j4) = w;
    }
    for (int i = tid; i < m; i += kNT) perm[i] = i;
    __syncthreads();
    const float c = static_cast<float>(coef);
    for (int z = tid; z < P.mech.L.NZ; z += kNT) {
      const int rc = __ldg(T.jz_rc + z);
      const int i = rc >> 16, j = rc & 0xffff;
      float J = 0.f;
      const int e1 = __ldg(T.jz_ptr + z + 1);
      for (int e = __ldg(T.jz_ptr + z); e < e1; ++e) J += __ldg(T.jc_nu32 + e) * d32[__ldg(T.jc_f + e)];
      A[static_cast<size_t>(i) * kLda + j] = (i == j ? 1.f : 0.f) - c * J;
    }
    __syncthreads();
    ++st.n_jac;
  }

  // ---- tensor-core pieces -------------------------------------------------------------------
  // Thread 0: D[buffer b] = A_tile(rt) * B_tile(n0 .. n0 + N) over K = 32 (four kind::tf32 MMAs),
  // committed to mbar[b].
  __device__ void issue_tile(int b, int rt, int n0, int N) {
    if (tid == 0) {
      const uint32_t id = tc::idesc_tf32(128, N, false);
      const uint32_t a0 = tc::smem_addr(aop) + static_cast<uint32_t>(rt) * 128u * kPW * 4u;
      const uint32_t b0 = tc::smem_addr(bop) + static_cast<uint32_t>(n0) * kPW * 4u;
#pragma unroll
      for (int s = 0; s < kPW / 8; ++s)
        tc::mma_tf32(tmem + static_cast<uint32_t>(b) * 256u, tc::smem_desc(a0 + 256u * s, 128u, 32u * kPW),
                     tc::smem_desc(b0 + 256u * s, 128u, 32u * kPW), id, s > 0);
      tc::commit(&H->mbar[b]);
    }
  }

  // All threads: waits (bounded) for buffer b's MMAs; false when the wait expired anywhere.
  __device__ bool wait_tile(int b) {
    const uint32_t par = (phbits >> b) & 1u;
    const bool ok = tc::mbar_wait(&H->mbar[b], par, kSpinLimit);
    phbits ^= 1u << b;
    const bool all = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!all) {
      if (tid == 0) {
        atomicOr(P.error_word, kErrBarrierTimeout);
        H->abort = 1;
      }
      // a second bounded window for the MMAs in flight
      const bool drained = __syncthreads_and(tc::mbar_wait(&H->mbar[b], par, kSpinLimit) ? 1 : 0) != 0;
      if (!drained && tid == 0) atomicOr(P.error_word, kErrMmaInFlight);
    }
    tc::fence_after_sync();
    return all;
  }

  // All threads: A22[rows of tile rt][n0 .. n0 + N) -= P (buffer b), thread = TMEM lane = row.
  __device__ void drain_tile(int b, int rt, int p1, int n0, int N) {
    const int lr = p1 + 128 * rt + tid;  // logical row
    float* row = lr < m ? A + static_cast<size_t>(perm[lr]) * kLda : nullptr;
    // 64 columns at a time: the row segment's global loads are all issued before the TMEM reads
    for (int c0 = 0; c0 < N; c0 += 64) {
      const int base = p1 + n0 + c0;
      float4 g[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int col = base + 4 * q;
        g[q] = (row != nullptr && 4 * q < N - c0 && col + 4 <= m) ? *reinterpret_cast<const float4*>(row + col)
                                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int sc = 0; sc < 4; ++sc) {
        if (16 * sc < N - c0) {  // warp-uniform
          float pv[16];
          tc::tmem_ld16(tmem + static_cast<uint32_t>(b) * 256u, warp, c0 + 16 * sc, pv);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            float4& a = g[4 * sc + q];
            a.x -= pv[4 * q];
            a.y -= pv[4 * q + 1];
            a.z -= pv[4 * q + 2];
            a.w -= pv[4 * q + 3];
            const int col = base + 16 * sc + 4 * q;
            if (row == nullptr || col >= m) continue;
            if (col + 4 <= m) {
              *reinterpret_cast<float4*>(row + col) = a;
            } else {  // the ragged end of the row
              const float* pq = pv + 4 * q;
              for (int z = 0; col + z < m; ++z) row[col + z] -= pq[z];
            }
          }
        }
      }
    }
  }

  // ---- blocked LU with partial pivoting, in place, rows addressed through perm -------------
  // Returns false on a zero or non-finite pivot, or when an MMA wait expired (H->abort).
  __device__ bool lu_factor() {
    for (int k0 = 0; k0 < m; k0 += kPW) {
      const int kb = min(kPW, m - k0), p1 = k0 + kb, np = m - k0;
      // The panel (logical rows k0 .. m-1, columns k0 .. k0 + 31) in registers, panel row
      // r = tid + 128 s held by thread tid. Implicit pivoting: the pivot row of each step is
      // published to shared memory (pn row c = L11 row c left of the diagonal, U11 row c from it)
      // and leaves the active set; the other rows are updated in registers. k0 is a multiple of
      // 32 and kLda of 4, so the float4 loads are aligned and stay inside the row.
      float a[kRowsPT][kPW];
      bool act[kRowsPT];
      int prow[kRowsPT];
#pragma unroll
      for (int s = 0; s < kRowsPT; ++s) {
        const int r = tid + kNT * s;
        act[s] = r < np;
        prow[s] = act[s] ? perm[k0 + r] : 0;
#pragma unroll
        for (int q = 0; q < kPW / 4; ++q) {
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (act[s]) v = *reinterpret_cast<const float4*>(A + static_cast<size_t>(prow[s]) * kLda + k0 + 4 * q);
          a[s][4 * q] = 4 * q < kb ? v.x : 0.f;
          a[s][4 * q + 1] = 4 * q + 1 < kb ? v.y : 0.f;
          a[s][4 * q + 2] = 4 * q + 2 < kb ? v.z : 0.f;
          a[s][4 * q + 3] = 4 * q + 3 < kb ? v.w : 0.f;
        }
      }
#pragma unroll
      for (int c = 0; c < kPW; ++c) {
        if (c < kb) {  // uniform
          // Pivot with one barrier: a packed key per row (|a| with its low 9 mantissa bits replaced
          // by 511 - panel row, so one max picks the largest magnitude to a relative 2^-14, ties to
          // the lowest row), one redux per warp; each warp's winning lane writes its row to the
          // warp's candidate slot (double-buffered by step parity) and lane 0 the warp's key.
          uint32_t key = 0u;
#pragma unroll
          for (int s = 0; s < kRowsPT; ++s) {
            const uint32_t kb9 = (__float_as_uint(a[s][c]) & 0x7fffffffu & ~511u) |
                                 (511u - static_cast<uint32_t>(tid + kNT * s));
            key = max(key, act[s] ? kb9 : 0u);
          }
          const uint32_t wkey = __reduce_max_sync(kFullMask, key);
          const int par = c & 1;
          float* cand = pn + (kPW + 4 * par + warp) * kPLd;
          if (key == wkey && wkey != 0u) {
            const int so = static_cast<int>(511u - (wkey & 511u)) / kNT;
#pragma unroll
            for (int s = 0; s < kRowsPT; ++s)
              if (s == so) {
#pragma unroll
                for (int q = 0; q < kPW / 4; ++q)
                  *reinterpret_cast<float4*>(cand + 4 * q) =
                      make_float4(a[s][4 * q], a[s][4 * q + 1], a[s][4 * q + 2], a[s][4 * q + 3]);
              }
          }
          uint32_t* keys = reinterpret_cast<uint32_t*>(H->redi[par]);
          if (lane == 0) keys[warp] = wkey;
          __syncthreads();
          uint32_t best = keys[0];
          int bw = 0;
#pragma unroll
          for (int w = 1; w < 4; ++w)
            if (keys[w] > best) {
              best = keys[w];
              bw = w;
            }
          const uint32_t mag = best & ~511u;
          if (mag == 0u || mag >= 0x7f800000u) return false;  // zero column, inf or nan (uniform)
          const int bi = static_cast<int>(511u - (best & 511u));  // the pivot's panel row
          const float* prow_s = pn + (kPW + 4 * par + bw) * kPLd;
          float u[kPW];
#pragma unroll
          for (int q = 0; q < kPW / 4; ++q) {
            const float4 v = *reinterpret_cast<const float4*>(prow_s + 4 * q);
            u[4 * q] = v.x;
            u[4 * q + 1] = v.y;
            u[4 * q + 2] = v.z;
            u[4 * q + 3] = v.w;
          }
          if ((bi & (kNT - 1)) == tid) {  // the owner records the step and drops the row
            const int so = bi / kNT;
#pragma unroll
            for (int s = 0; s < kRowsPT; ++s)
              if (s == so) {
#pragma unroll
                for (int q = 0; q < kPW / 4; ++q)
                  *reinterpret_cast<float4*>(pn + c * kPLd + 4 * q) =
                      make_float4(a[s][4 * q], a[s][4 * q + 1], a[s][4 * q + 2], a[s][4 * q + 3]);
                act[s] = false;
                H->pphys[c] = prow[s];
              }
          }
          const float inv = 1.f / u[c];
#pragma unroll
          for (int s = 0; s < kRowsPT; ++s) {
            if (act[s]) {
              const float l = a[s][c] * inv;
              a[s][c] = l;
#pragma unroll
              for (int j = c + 1; j < kPW; ++j) a[s][j] = fmaf(-l, u[j], a[s][j]);
            }
          }
        }
      }
      __syncthreads();  // pivot rows (pn) and pphys complete
      // factored rows back to the matrix (physical rows): L and U11 of the pivot rows, L21
#pragma unroll
      for (int s = 0; s < kRowsPT; ++s) {
        if (tid + kNT * s < np) {
          float* dst = A + static_cast<size_t>(prow[s]) * kLda + k0;
#pragma unroll
          for (int q = 0; q < kPW / 4; ++q) {
            if (4 * q + 4 <= kb) {
              *reinterpret_cast<float4*>(dst + 4 * q) =
                  make_float4(a[s][4 * q], a[s][4 * q + 1], a[s][4 * q + 2], a[s][4 * q + 3]);
            } else {
#pragma unroll
              for (int z = 0; z < 4; ++z)
                if (4 * q + z < kb) dst[4 * q + z] = a[s][4 * q + z];
            }
          }
        }
      }
      // trailing order: the non-pivot rows by increasing panel row (an exclusive scan of the
      // still-active flags over r = tid + 128 s)
      int qpos[kRowsPT];
#pragma unroll
      for (int s = 0; s < kRowsPT; ++s) {
        const unsigned bal = __ballot_sync(kFullMask, act[s]);
        qpos[s] = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) H->scnt[s][warp] = __popc(bal);
      }
      __syncthreads();
      {
        int base = 0;
#pragma unroll
        for (int s = 0; s < kRowsPT; ++s) {
          int off = base;
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            if (w < warp) off += H->scnt[s][w];
            base += H->scnt[s][w];
          }
          qpos[s] += off;
        }
      }
      // the new logical order: the kb pivots, then the trailing rows
      if (tid < kb) perm[k0 + tid] = H->pphys[tid];
#pragma unroll
      for (int s = 0; s < kRowsPT; ++s)
        if (act[s]) perm[p1 + qpos[s]] = prow[s];
      __syncthreads();  // the new order before U12 reads the pivot rows through it
      const int W = m - p1;  // trailing width
      if (W <= 0) break;
      const int N0 = W <= 256 ? ((W + 15) & ~15) : (((W + 1) / 2 + 15) & ~15);
      const int N1 = W <= 256 ? 0 : ((W - N0 + 15) & ~15);
      const int Wp = N0 + N1;
      // U12 = L11^-1 A12 (one column per thread), to the matrix and the B operand
      for (int j = tid; j < Wp; j += kNT) {
        float u[kPW];
        const bool in = j < W;
#pragma unroll
        for (int i = 0; i < kPW; ++i)
          u[i] = (in && i < kb) ? A[static_cast<size_t>(perm[k0 + i]) * kLda + p1 + j] : 0.f;
#pragma unroll
        for (int i = 1; i < kPW; ++i) {
          float acc = u[i];
#pragma unroll
          for (int q = 0; 4 * q < i; ++q) {  // L11 row i, columns 0 .. i-1, as float4 reads
            const float4 v = *reinterpret_cast<const float4*>(pn + i * kPLd + 4 * q);
            acc = fmaf(-v.x, u[4 * q], acc);
            if (4 * q + 1 < i) acc = fmaf(-v.y, u[4 * q + 1], acc);
            if (4 * q + 2 < i) acc = fmaf(-v.z, u[4 * q + 2], acc);
            if (4 * q + 3 < i) acc = fmaf(-v.w, u[4 * q + 3], acc);
          }
          u[i] = i < kb ? acc : 0.f;
        }
#pragma unroll
        for (int i = 0; i < kPW; ++i) {
          if (in && i < kb) A[static_cast<size_t>(perm[k0 + i]) * kLda + p1 + j] = u[i];
          *reinterpret_cast<float*>(bop + tc::kmajor_offset(j, i, kPW)) = u[i];
        }
      }
      // L21 (the trailing rows' multipliers, from registers) as the A operand; rows W .. of the last
      // 128-row tile are zero
      const int nrt = (W + 127) / 128;
#pragma unroll
      for (int s = 0; s < kRowsPT; ++s)
        if (act[s]) {
#pragma unroll
          for (int c = 0; c < kPW; ++c)
            *reinterpret_cast<float*>(aop + tc::kmajor_offset(qpos[s], c, kPW)) = c < kb ? a[s][c] : 0.f;
        }
      for (int e = W * kPW + tid; e < nrt * 128 * kPW; e += kNT) {
        const int r = e / kPW, c = e - r * kPW;
        *reinterpret_cast<float*>(aop + tc::kmajor_offset(r, c, kPW)) = 0.f;
      }
      tc::fence_proxy_async();  // generic-proxy operand writes before the MMAs read them
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      // trailing update, two TMEM buffers: tile j + 1's MMAs run while tile j is drained
      const int nct = N1 > 0 ? 2 : 1;
      const int nt = nrt * nct;
      issue_tile(0, 0, 0, N0);
      for (int j = 0; j < nt; ++j) {
        if (j + 1 < nt) {
          const int ct = (j + 1) % nct;
          issue_tile((j + 1) & 1, (j + 1) / nct, ct ? N0 : 0, ct ? N1 : N0);
        }
        if (!wait_tile(j & 1)) {
          // the buffer of tile j + 1 may still be in flight: give it the second window too
          if (j + 1 < nt) {
            const int b1 = (j + 1) & 1;
            const bool d = __syncthreads_and(tc::mbar_wait(&H->mbar[b1], (phbits >> b1) & 1u, kSpinLimit) ? 1 : 0);
            if (!d && tid == 0) atomicOr(P.error_word, kErrMmaInFlight);
          }
          return false;
        }
        const int ct = j % nct;
        drain_tile(j & 1, j / nct, p1, ct ? N0 : 0, ct ? N1 : N0);
        tc::fence_before_sync();
        __syncthreads();  // buffer j & 1 drained and A22 updated before it is reused / re-read
        tc::fence_after_sync();
      }
    }
    ++st.n_lu;
    return true;
  }

  // sum over c < kb of row[c] * w32[k0 + c]: 8 float4 loads for a full block (row 16-byte aligned)
  __device__ __forceinline__ float row_dot(const float* row, int k0, int kb) const {
    float acc = 0.f;
    if (kb == kPW) {
      float4 a[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) a[q] = *reinterpret_cast<const float4*>(row + 4 * q);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        acc = fmaf(a[q].x, w32[k0 + 4 * q], acc);
        acc = fmaf(a[q].y, w32[k0 + 4 * q + 1], acc);
        acc = fmaf(a[q].z, w32[k0 + 4 * q + 2], acc);
        acc = fmaf(a[q].w, w32[k0 + 4 * q + 3], acc);
      }
    } else {
      for (int c = 0; c < kb; ++c) acc = fmaf(row[c], w32[k0 + c], acc);
    }
    return acc;
  }

  // ---- x = A^-1 b with the factors (FP32 substitutions; b and x FP64 vectors in shared memory)
  // Forward: w = L^-1 (P b), back: x = U^-1 w, by 32-row blocks. Warp 0 applies the previous
  // block to the next block's rows and then solves that block (one row per lane, shuffles) while
  // warps 1-3 apply the previous block to the remaining rows: one barrier per block.
  __device__ void diag_lower(int k0) {  // warp 0: unit-lower diagonal block at k0
    const int kb = min(kPW, m - k0), r = k0 + lane;
    float lrow[kPW];
    const float* src = A + static_cast<size_t>(perm[r < m ? r : k0]) * kLda + k0;
#pragma unroll
    for (int c = 0; c < kPW; ++c) lrow[c] = (r < m && c < kb) ? src[c] : 0.f;
    float val = r < m ? w32[r] : 0.f;
#pragma unroll
    for (int c = 0; c < kPW; ++c) {
      const float zc = __shfl_sync(kFullMask, val, c);
      if (lane > c) val = fmaf(-lrow[c], zc, val);
    }
    if (lane < kb) w32[r] = val;
  }
  __device__ void diag_upper(int k0) {  // warp 0: upper diagonal block at k0
    const int kb = min(kPW, m - k0), r = k0 + lane;
    float urow[kPW];
    const float* src = A + static_cast<size_t>(perm[r < m ? r : k0]) * kLda + k0;
#pragma unroll
    for (int c = 0; c < kPW; ++c) urow[c] = (r < m && c < kb) ? src[c] : 0.f;
    float val = r < m ? w32[r] : 0.f;
#pragma unroll
    for (int c = kPW - 1; c >= 0; --c) {
      if (c < kb) {
        if (lane == c) val = val / urow[c];
        const float xc = __shfl_sync(kFullMask, val, c);
        if (lane < c) val = fmaf(-urow[c], xc, val);
      }
    }
    if (lane < kb) w32[r] = val;
  }

  __device__ void solve(const double* b, double* x) {
    for (int i = tid; i < m; i += kNT) w32[i] = static_cast<float>(b[perm[i]]);
    __syncthreads();
    const int nb = (m + kPW - 1) / kPW;
    if (warp == 0) diag_lower(0);
    __syncthreads();
    for (int blk = 0; blk + 1 < nb; ++blk) {
      const int k0 = blk * kPW, next = k0 + kPW;  // block blk is full (32 rows): it is not the last
      if (warp == 0) {
        const int r = next + lane;
        if (r < m) w32[r] -= row_dot(A + static_cast<size_t>(perm[r]) * kLda + k0, k0, kPW);
        __syncwarp();
        diag_lower(next);
      } else {
        for (int i = next + kPW + (tid - 32); i < m; i += kNT - 32)
          w32[i] -= row_dot(A + static_cast<size_t>(perm[i]) * kLda + k0, k0, kPW);
      }
      __syncthreads();
    }
    if (warp == 0) diag_upper((nb - 1) * kPW);
    __syncthreads();
    for (int blk = nb - 1; blk > 0; --blk) {
      const int k0 = blk * kPW, kb = min(kPW, m - k0), prev = k0 - kPW;
      if (warp == 0) {
        const int r = prev + lane;
        w32[r] -= row_dot(A + static_cast<size_t>(perm[r]) * kLda + k0, k0, kb);
        __syncwarp();
        diag_upper(prev);
      } else {
        for (int i = tid - 32; i < prev; i += kNT - 32)
          w32[i] -= row_dot(A + static_cast<size_t>(perm[i]) * kLda + k0, k0, kb);
      }
      __syncthreads();
    }
    for (int i = tid; i < m; i += kNT) x[i] = static_cast<double>(w32[i]);
    __syncthreads();
    ++st.n_solve;
  }

  // ---- Newton on y - coef f(y) = rv from the guess in y (the full Newton of the FP64 form)
  // Returns 0 converged, 1 not converged / singular, 2 aborted (an MMA wait expired).
  __device__ int newton(double* y, const double* rv, double coef, int max_newton, int jac_interval, double atol,
                        double rtol) {
    double* f = v(V_F);
    double* g = v(V_G);
    double* dx = v(V_DX);
    double* r = v(V_R);
    double* yj = v(V_YJ);
    for (int it = 0; it < max_newton; ++it) {
      rhs(y, f);
      for (int i = tid; i < m; i += kNT) g[i] = -((y[i] - coef * f[i]) - rv[i]);
      if (it % jac_interval == 0) {
        for (int i = tid; i < m; i += kNT) yj[i] = y[i];
        newton_matrix(y, coef);
        if (!lu_factor()) return H->abort ? 2 : 1;
      }
      __syncthreads();
      solve(g, dx);
      // one sweep of refinement: FP64 residual of (I - c J(yj)) dx = g, correction through the factors
      jvec(yj, dx, r);
      for (int i = tid; i < m; i += kNT) r[i] = g[i] - (dx[i] - coef * r[i]);
      __syncthreads();
      solve(r, f);
      double sdx = 0.0, sy = 0.0;
      for (int i = tid; i < m; i += kNT) {
        const double d = dx[i] + f[i];
        y[i] += d;
        sdx += d * d;
        sy += y[i] * y[i];
      }
      ++st.n_newton_iter;
      const double ndx = sqrt(bsum(sdx)), ny = sqrt(bsum(sy));
      if (!isfinite(ndx) || !isfinite(ny)) return 1;
      if (ndx <= atol + rtol * ny) return 0;
    }
    return 1;
  }

  // ---- TR-BDF2 (the algorithm of fp64_core.cuh's integrate and of the oracle) ---------------
  __device__ int integrate(double t_beg, double t_end, double dt_in, double dt_min, double dt_max, int max_iters,
                           int max_newton, int jac_interval, double natol, double nrtol, double& t_out,
                           double& dt_out) {
    if (dt_in < 0.0) return TCHEM_GB_SAMPLE_NEGATIVE_DT;
    const double gamma = 2.0 - sqrt(2.0);
    const double d = 0.5 * gamma;
    const double cg = 1.0 / (gamma * (2.0 - gamma));
    const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
    const double kappa = (-3.0 * gamma * gamma + 4.0 * gamma - 2.0) / (12.0 * (2.0 - gamma));
    const double e0 = 1.0 / gamma, e1 = -1.0 / (gamma * (1.0 - gamma)), e2 = 1.0 / (1.0 - gamma);
    double* y = v(V_Y);
    double* fn = v(V_FN);
    double* fg = v(V_FG);
    double* f1 = v(V_F1);
    double* yg = v(V_YG);
    double* y1 = v(V_Y1);
    double* rv = v(V_RV);
    double* est = v(V_EST);
    const double* atol = v(V_ATOL);
    const double* rtol = v(V_RTOL);
    double t = t_beg, dt = dt_in;
    int status = TCHEM_GB_SAMPLE_OK;
    rhs(y, fn);
    for (int iter = 0; iter < max_iters && t < t_end; ++iter) {
      bool converged = false, last = false;
      for (int ntry = 0; ntry < 4; ++ntry) {
        dt = fmin(fmax(dt, dt_min), dt_max);
        last = dt >= t_end - t;
        if (last) dt = t_end - t;
        if (!(dt > 0.0)) {
          status = TCHEM_GB_SAMPLE_DT_UNDERFLOW;
          break;
        }
        const double coef = d * dt;
        for (int i = tid; i < m; i += kNT) {
          rv[i] = y[i] + coef * fn[i];
          yg[i] = y[i];
        }
        __syncthreads();
        int ok = newton(yg, rv, coef, max_newton, jac_interval, natol, nrtol);
        if (ok == 0) {
          rhs(yg, fg);
          for (int i = tid; i < m; i += kNT) {
            rv[i] = cg * yg[i] - cn * y[i];
            y1[i] = yg[i];
          }
          __syncthreads();
          ok = newton(y1, rv, coef, max_newton, jac_interval, natol, nrtol);
        }
        if (ok == 2) {
          status = TCHEM_GB_SAMPLE_NONFINITE;  // aborted: the kernel stops after this sample
          break;
        }
        if (ok == 0) {
          converged = true;
          break;
        }
        ++st.n_newton_fail;
        dt *= 0.5;
      }
      if (status != TCHEM_GB_SAMPLE_OK) break;
      if (!converged) {
        status = TCHEM_GB_SAMPLE_NEWTON_FAIL;
        break;
      }
      rhs(y1, f1);
      for (int i = tid; i < m; i += kNT) est[i] = 2.0 * kappa * dt * (e0 * fn[i] + e1 * fg[i] + e2 * f1[i]);
      __syncthreads();
      solve(est, est);  // filtered with the last Newton matrix, as the FP64 form
      double err = 0.0;
      for (int i = tid; i < m; i += kNT)
        err = fmax(err, fabs(est[i]) / (atol[i] + rtol[i] * fmax(fabs(y[i]), fabs(y1[i]))));
      err = bmax(err);
      if (!isfinite(err)) {
        status = TCHEM_GB_SAMPLE_NONFINITE;
        break;
      }
      if (err <= 1.0 || dt <= dt_min) {
        t = last ? t_end : t + dt;
        for (int i = tid; i < m; i += kNT) {
          y[i] = y1[i];
          fn[i] = f1[i];
        }
        __syncthreads();
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
      for (int i = tid; i < m; i += kNT) y[i] = 0.0;
      __syncthreads();
      t_out = t_end;
      dt_out = -1.0;
    }
    return status;
  }
};

// One sample per CTA, persistent over the work queue (the outer protocol of the other forms).
__global__ void __launch_bounds__(kNT, 1) trbdf2_tc_kernel(const __grid_constant__ AdvanceParams P) {
  extern __shared__ __align__(1024) unsigned char smem[];
  Header* H = reinterpret_cast<Header*>(smem);
  const MechLayout& L = P.mech.L;
  const Layout lay = layout(L);
  const int tid = threadIdx.x;
  Solver S{P,
           smem,
           H,
           tables_at(P.mech.blob, L),
           reinterpret_cast<float*>(P.gmat) + static_cast<size_t>(blockIdx.x) * P.gmat_stride,
           reinterpret_cast<float*>(smem + lay.panel),
           smem + lay.aop,
           smem + lay.bop,
           reinterpret_cast<double*>(smem + lay.vec),
           reinterpret_cast<double*>(smem + lay.keff),
           reinterpret_cast<double*>(smem + lay.q),
           reinterpret_cast<float*>(smem + lay.d32),
           reinterpret_cast<float*>(smem + lay.w32),
           reinterpret_cast<int32_t*>(smem + lay.perm),
           L.m,
           L.R,
           tid,
           tid & 31,
           tid >> 5,
           0u};
  if (S.warp == 0) tc::tmem_alloc(&H->tmem_slot, kTmemCols);
  if (tid == 0) {
    tc::mbar_init(&H->mbar[0], 1);
    tc::mbar_init(&H->mbar[1], 1);
    H->abort = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  S.tmem = H->tmem_slot;
  const int n_items = P.n_items_dev ? *P.n_items_dev : P.n_items;
  const int m = L.m;
  while (true) {
    if (tid == 0) H->item = H->abort ? n_items : atomicAdd(P.queue, 1);
    __syncthreads();
    const int item = H->item;
    __syncthreads();
    if (item >= n_items) break;
    const int s = P.items ? P.items[item] : item;
    const tchem_gb_tadv ta = P.tadv[s];
    if (P.t_out[s] >= ta.tend) {
      if (tid == 0) {
        P.status[s] = TCHEM_GB_SAMPLE_SKIPPED;
        if (P.stats) P.stats[s] = tchem_gb_sample_stats{};
      }
      continue;
    }
    const int gm = P.mech_of_sample ? P.mech_of_sample[s] : 0;
    const int slot = (gm >= 0 && gm < kMaxMechs) ? P.slot_of_mech[gm] : -1;
    if (slot < 0) {
      if (tid == 0) P.status[s] = TCHEM_GB_SAMPLE_BAD_MECH;
      continue;
    }
    const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
    const double p = row[1], Tk = row[2];
    {
      // rate constants once per sample, with the constant species folded in
      const double t_1 = 1.0 / Tk;
      const double conv = P.mech.conv_ppm * p * t_1;
      const double* rp = P.rate_param[slot];
      const double* xconst = row + 3 + m;
      for (int r = tid; r < L.R; r += kNT) {
        double k = rate_constant(P.mech.rate_type[r], rp + 8 * r, P.mech.conv_exp[r], Tk, t_1, p, conv);
        for (int c = P.mech.cf_ptr[r]; c < P.mech.cf_ptr[r + 1]; ++c) k *= xconst[P.mech.cf_idx[c]];
        S.keff[r] = k;
      }
    }
    for (int i = tid; i < m; i += kNT) {
      S.v(V_Y)[i] = row[3 + i];
      S.v(V_ATOL)[i] = P.tol_time[2 * i];
      S.v(V_RTOL)[i] = P.tol_time[2 * i + 1];
    }
    __syncthreads();
    S.st = tchem_gb_sample_stats{};
    double t_o = 0.0, dt_o = 0.0;
    const int st = S.integrate(ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax, ta.num_time_iterations_per_interval,
                               ta.max_num_newton_iterations, ta.jacobian_interval > 0 ? ta.jacobian_interval : 1,
                               P.tol_newton[0], P.tol_newton[1], t_o, dt_o);
    if (tid == 0) {
      P.status[s] = st;
      if (P.stats) P.stats[s] = S.st;
    }
    if (st != TCHEM_GB_SAMPLE_NEGATIVE_DT) {
      double* out = P.state_out + static_cast<size_t>(s) * P.state_dim;
      // constant species and rho, p, T pass through (src/core/TChem_AtmosphericChemistry.cpp:159-161)
      for (int i = tid; i < P.state_dim - 3 - m; i += kNT) out[3 + m + i] = row[3 + m + i];
      if (tid == 0) {
        const double rho = row[0];
        out[0] = rho;
        out[1] = p;
        out[2] = Tk;
        P.t_out[s] = t_o;
        P.dt_out[s] = dt_o;
      }
      for (int i = tid; i < m; i += kNT) out[3 + i] = S.v(V_Y)[i];
    }
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (S.warp == 0) tc::tmem_dealloc(S.tmem, kTmemCols);
}

}  // namespace tcadv

size_t tc_advance_matrix_floats() { return static_cast<size_t>(tcadv::kMaxM) * tcadv::kLda; }

int tc_advance_max_species() { return tcadv::kMaxM; }

cudaError_t launch_trbdf2_tc(const AdvanceParams& P, int grid, size_t smem, cudaStream_t stream) {
  auto k = tcadv::trbdf2_tc_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, tcadv::kNT, smem, stream>>>(P);
  return cudaGetLastError();
}

}  // namespace tchem_gb
