// Plain FP64 TR-BDF2 time advance: one warp per sample, persistent work queue.
//
// Per sample the warp runs the whole integration to t_end (or the step budget): rate
// constants once (the reference recomputes them in every RHS call,
// src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:96), then TR-BDF2 steps whose two implicit
// stages are solved by Newton with an analytic Jacobian and a dense LU with partial pivoting.
// The Newton matrix lives in shared memory (global memory for mechanisms too large for it);
// the trailing update of the LU is flattened over (row, column) pairs so all 32 lanes stay
// busy on the FP64 pipe, which bounds this form.
#include "advance.hpp"
#include "engine.cuh"
#include "fp64_core.cuh"
#include "kernels.hpp"

namespace tchem_gb {

using namespace fp64;

size_t fp64_warp_smem_bytes(const MechLayout& L, int lda, bool matrix_in_smem, bool src_section) {
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  size_t b = 0;
  if (src_section) b += up16(sizeof(double) * L.m);  // per-sample source term
  b += up16(sizeof(double) * L.m);   // x
  b += up16(sizeof(double) * L.R);   // keff
  b += up16(sizeof(double) * L.R);   // q
  b += up16(sizeof(double) * L.NF);  // d
  b += up16(sizeof(double) * L.m);   // w
  b += up16(sizeof(int32_t) * L.m);  // piv
  if (matrix_in_smem) b += up16(sizeof(double) * static_cast<size_t>(L.m) * lda);
  return b;
}

template <int NPL>
__global__ void __launch_bounds__(256, 1) trbdf2_fp64_kernel(const __grid_constant__ AdvanceParams P) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
  unsigned char* tables = smem + 16;
  const MechLayout& L = P.mech.L;
  if (!stage_to_smem(tables, P.mech.blob, static_cast<uint32_t>(L.blob_bytes), mbar)) {
    if (threadIdx.x == 0) atomicOr(P.error_word, kErrBarrierTimeout);
    return;
  }
  SmemTables T = tables_at(tables, L);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* mine = tables + L.blob_bytes + static_cast<size_t>(warp) * P.warp_smem_bytes;
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  double* src = nullptr;  // per-sample source term (E3SM external sources) in place of the emissions
  if (P.src_in) {
    src = reinterpret_cast<double*>(mine);
    mine += up16(sizeof(double) * L.m);
    T.emis = src;
  }
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
  if (P.matrix_in_smem) {
    W.A = reinterpret_cast<double*>(mine);
  } else {
    const long long gw = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp;
    W.A = P.gmat + gw * P.gmat_stride;
  }

  const int n_items = P.n_items_dev ? *P.n_items_dev : P.n_items;
  const int m = L.m;
  const NewtonSettings ns{0, 1, P.tol_newton[0], P.tol_newton[1]};
  while (true) {
    int item = 0;
    if (lane == 0) item = atomicAdd(P.queue, 1);
    item = __shfl_sync(kFullMask, item, 0);
    if (item >= n_items) break;
    const int s = P.items ? P.items[item] : item;
    const tchem_gb_tadv ta = P.tadv[s];
    if (P.t_out[s] >= ta.tend) {
      if (lane == 0) {
        P.status[s] = TCHEM_GB_SAMPLE_SKIPPED;
        if (P.stats) P.stats[s] = tchem_gb_sample_stats{};
      }
      continue;
    }
    const int gm = P.mech_of_sample ? P.mech_of_sample[s] : 0;
    const int slot = (gm >= 0 && gm < kMaxMechs) ? P.slot_of_mech[gm] : -1;
    if (slot < 0) {
      if (lane == 0) P.status[s] = TCHEM_GB_SAMPLE_BAD_MECH;
      continue;
    }
    const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
    const double p = row[1], Tk = row[2];
    if (P.keff_in) {
      for (int r = lane; r < L.R; r += 32) W.keff[r] = P.keff_in[static_cast<size_t>(s) * L.R + r];
    } else {
      compute_keff(P.mech, P.rate_param[slot], Tk, p, row + 3 + m, W.keff, lane);
    }
    if (P.src_in)
      for (int i = lane; i < m; i += 32) src[i] = P.src_in[s * P.src_stride + i];
    __syncwarp();
    if (P.k_scale) {
      for (int r = lane; r < L.R; r += 32) W.keff[r] *= P.k_scale[r];
      __syncwarp();
    }

    double y[NPL], atol[NPL], rtol[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
      const int i = lane + 32 * k;
      y[k] = (i < m) ? row[3 + i] : 0.0;
      atol[k] = (i < m) ? P.tol_time[2 * i] : 1.0;
      rtol[k] = (i < m) ? P.tol_time[2 * i + 1] : 0.0;
    }
    Ctx<NPL> c{L, T, W, lane, P.lda, tchem_gb_sample_stats{}};
    NewtonSettings nset = ns;
    nset.max_newton = ta.max_num_newton_iterations;
    nset.jac_interval = ta.jacobian_interval > 0 ? ta.jacobian_interval : 1;
    double t_o = 0.0, dt_o = 0.0;
    Tape tape{};
    if (P.tape_dt) {
      tape.dt = P.tape_dt + static_cast<size_t>(s) * P.tape_cap;
      tape.ckpt = P.tape_ckpt + static_cast<size_t>(s) * (P.tape_cap / kTapeSegment + 1) * m;
      tape.cap = P.tape_cap;
    }
    const int st = integrate(c, y, atol, rtol, ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax,
                             ta.num_time_iterations_per_interval, nset, t_o, dt_o, tape);
    if (lane == 0) {
      P.status[s] = st;
      if (P.stats) P.stats[s] = c.st;
      if (P.tape_nsteps) P.tape_nsteps[s] = c.st.n_steps;
    }
    if (st == TCHEM_GB_SAMPLE_NEGATIVE_DT) continue;
    double* out = P.state_out + static_cast<size_t>(s) * P.state_dim;
    // Constant species and rho, p, T are copied through (src/core/TChem_AtmosphericChemistry.cpp:159-161).
    for (int i = lane; i < P.state_dim - 3 - m; i += 32) out[3 + m + i] = row[3 + m + i];
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
      if (i < m) out[3 + i] = y[k];
    }
    __syncwarp();
  }
}

template <int NPL>
cudaError_t launch_fp64_npl(const AdvanceParams& P, int grid, int warps_per_block, size_t smem, cudaStream_t stream) {
  auto k = trbdf2_fp64_kernel<NPL>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  k<<<grid, warps_per_block * 32, smem, stream>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_trbdf2_fp64(const AdvanceParams& P, int grid, int warps_per_block, size_t smem,
                               cudaStream_t stream) {
  const int m = P.mech.L.m;
  if (m <= 32) return launch_fp64_npl<1>(P, grid, warps_per_block, smem, stream);
  if (m <= 64) return launch_fp64_npl<2>(P, grid, warps_per_block, smem, stream);
  if (m <= 128) return launch_fp64_npl<4>(P, grid, warps_per_block, smem, stream);
  if (m <= 256) return launch_fp64_npl<8>(P, grid, warps_per_block, smem, stream);
  if (m <= 320) return launch_fp64_npl<10>(P, grid, warps_per_block, smem, stream);
  return cudaErrorInvalidValue;
}

}  // namespace tchem_gb

namespace tchem_gb {

const void* trbdf2_fp64_kernel_ptr(int m) {
  if (m <= 32) return reinterpret_cast<const void*>(trbdf2_fp64_kernel<1>);
  if (m <= 64) return reinterpret_cast<const void*>(trbdf2_fp64_kernel<2>);
  if (m <= 128) return reinterpret_cast<const void*>(trbdf2_fp64_kernel<4>);
  if (m <= 256) return reinterpret_cast<const void*>(trbdf2_fp64_kernel<8>);
  return reinterpret_cast<const void*>(trbdf2_fp64_kernel<10>);
}

namespace {

constexpr int kUnitWarps = 4;

// Rate constants, right-hand side or Jacobian of one sample per warp, on the staged tables.
template <int KIND>
__global__ void __launch_bounds__(kUnitWarps * 32) unit_kernel(const __grid_constant__ UnitParams P) {
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
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  const size_t per_warp = up16(sizeof(double) * L.m) + 2 * up16(sizeof(double) * L.R) + up16(sizeof(double) * L.NF);
  unsigned char* mine = tables + L.blob_bytes + warp * per_warp;
  double* x = reinterpret_cast<double*>(mine);
  double* keff = reinterpret_cast<double*>(mine + up16(sizeof(double) * L.m));
  double* q = keff + (up16(sizeof(double) * L.R) / sizeof(double));
  double* d = q + (up16(sizeof(double) * L.R) / sizeof(double));
  const int s = blockIdx.x * kUnitWarps + warp;
  if (s >= P.B) return;
  const int gm = P.mech_of_sample ? P.mech_of_sample[s] : 0;
  const int slot = (gm >= 0 && gm < kMaxMechs) ? P.slot_of_mech[gm] : -1;
  if (slot < 0) {
    if (lane == 0 && P.status) P.status[s] = TCHEM_GB_SAMPLE_BAD_MECH;
    return;
  }
  const double* row = P.state + static_cast<size_t>(s) * P.state_dim;
  const double p = row[1], Tk = row[2];
  const int m = L.m;
  if constexpr (KIND == UNIT_KFORWARD) {
    const double t_1 = 1.0 / Tk;
    const double conv = P.mech.conv_ppm * p * t_1;
    for (int r = lane; r < L.R; r += 32)
      P.out[static_cast<size_t>(s) * L.R + r] =
          rate_constant(P.mech.rate_type[r], P.rate_param[slot] + 8 * r, P.mech.conv_exp[r], Tk, t_1, p, conv);
    return;
  }
  compute_keff(P.mech, P.rate_param[slot], Tk, p, row + 3 + m, keff, lane);
  for (int i = lane; i < m; i += 32) x[i] = row[3 + i];
  __syncwarp();
  if constexpr (KIND == UNIT_RHS) {
    for (int r = lane; r < L.R; r += 32) {
      double qq = keff[r];
      for (int g = T.rf_ptr[r]; g < T.rf_ptr[r + 1]; ++g) qq *= x[T.rf_sp[g]];
      q[r] = qq;
    }
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
      double acc = T.emis[i];
      for (int e = T.pr_ptr[i]; e < T.pr_ptr[i + 1]; ++e) acc += T.pr_nu[e] * q[T.pr_r[e]];
      P.out[static_cast<size_t>(s) * m + i] = acc;
    }
  } else {  // Jacobian
    for (int r = lane; r < L.R; r += 32) {
      const int f0 = T.rf_ptr[r], f1 = T.rf_ptr[r + 1];
      for (int f = f0; f < f1; ++f) {
        double dv = keff[r];
        for (int g = f0; g < f1; ++g)
          if (g != f) dv *= x[T.rf_sp[g]];
        d[f] = dv;
      }
    }
    double* J = P.out + static_cast<size_t>(s) * m * m;
    for (int e = lane; e < m * m; e += 32) J[e] = 0.0;
    __syncwarp();
    for (int z = lane; z < L.NZ; z += 32) {
      const int rc = T.jz_rc[z];
      double acc = 0.0;
      for (int e = T.jz_ptr[z]; e < T.jz_ptr[z + 1]; ++e) acc += T.jc_nu[e] * d[T.jc_f[e]];
      J[static_cast<size_t>(rc >> 16) * m + (rc & 0xffff)] = acc;
    }
  }
}

__global__ void bucket_kernel(const int32_t* mech_of_sample, int B, const GroupMap G, int n_mechs,
                              int32_t* counts, int32_t* items, int32_t* status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const int gm = mech_of_sample[s];
  if (gm < 0 || gm >= n_mechs) {
    status[s] = TCHEM_GB_SAMPLE_BAD_MECH;
    return;
  }
  const int g = G.group_of_mech[gm];
  const int pos = atomicAdd(&counts[g], 1);
  items[static_cast<size_t>(g) * B + pos] = s;
}

}  // namespace

cudaError_t launch_unit(const UnitParams& P, UnitKind kind, cudaStream_t stream) {
  const MechLayout& L = P.mech.L;
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  const size_t per_warp = up16(sizeof(double) * L.m) + 2 * up16(sizeof(double) * L.R) + up16(sizeof(double) * L.NF);
  const size_t smem = 16 + L.blob_bytes + kUnitWarps * per_warp;
  const int grid = (P.B + kUnitWarps - 1) / kUnitWarps;
  if (grid == 0) return cudaSuccess;
  const void* k = kind == UNIT_KFORWARD ? reinterpret_cast<const void*>(unit_kernel<UNIT_KFORWARD>)
                  : kind == UNIT_RHS    ? reinterpret_cast<const void*>(unit_kernel<UNIT_RHS>)
                                        : reinterpret_cast<const void*>(unit_kernel<UNIT_JACOBIAN>);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  if (kind == UNIT_KFORWARD) unit_kernel<UNIT_KFORWARD><<<grid, kUnitWarps * 32, smem, stream>>>(P);
  else if (kind == UNIT_RHS) unit_kernel<UNIT_RHS><<<grid, kUnitWarps * 32, smem, stream>>>(P);
  else unit_kernel<UNIT_JACOBIAN><<<grid, kUnitWarps * 32, smem, stream>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_bucket(const int32_t* mech_of_sample, int B, const GroupMap& G, int n_mechs,
                          int32_t* counts, int32_t* items, int32_t* status, cudaStream_t stream) {
  if (B <= 0) return cudaSuccess;
  bucket_kernel<<<(B + 255) / 256, 256, 0, stream>>>(mech_of_sample, B, G, n_mechs, counts, items, status);
  return cudaGetLastError();
}

}  // namespace tchem_gb
