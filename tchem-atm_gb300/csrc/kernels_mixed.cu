// Mixed-precision form: kernel-shape selection and launch configuration for the register-resident
// FP32-LU kernel (kernels_mixed_impl.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>

#include "kernels_mixed.hpp"
#include "kernels_mixed_impl.cuh"

namespace tchem_gb {

// Launchers defined in kernels_mixed_v*.cu (FP32 LU) and kernels_simpl_v*.cu (simplified Newton),
// one translation unit per kernel.
#define TCHEM_GB_DECLARE_SHAPE(PRE, MC, RPT)                                                    \
  cudaError_t launch_##PRE##_##MC##_##RPT(const AdvanceParams&, int, int, size_t, cudaStream_t); \
  const void* kernel_##PRE##_##MC##_##RPT();
TCHEM_GB_DECLARE_SHAPE(mixed, 24, 1)
TCHEM_GB_DECLARE_SHAPE(mixed, 32, 1)
TCHEM_GB_DECLARE_SHAPE(mixsp, 64, 2)
TCHEM_GB_DECLARE_SHAPE(mixsp, 128, 4)
TCHEM_GB_DECLARE_SHAPE(mixgj, 52, 1_g2)
TCHEM_GB_DECLARE_SHAPE(mixgj, 64, 1_g2)
TCHEM_GB_DECLARE_SHAPE(mixgj, 128, 1_g4)
TCHEM_GB_DECLARE_SHAPE(simpl, 24, 1)
TCHEM_GB_DECLARE_SHAPE(simpl, 32, 1)
TCHEM_GB_DECLARE_SHAPE(simpl, 52, 2)
TCHEM_GB_DECLARE_SHAPE(simpl, 64, 2)
TCHEM_GB_DECLARE_SHAPE(simpl, 52, 1_g2)
TCHEM_GB_DECLARE_SHAPE(simpl, 64, 1_g2)
TCHEM_GB_DECLARE_SHAPE(simpl, 128, 1_g4)
TCHEM_GB_DECLARE_SHAPE(e3mixed, 64, 2)
TCHEM_GB_DECLARE_SHAPE(e3simpl, 64, 2)
TCHEM_GB_DECLARE_SHAPE(e3simpl, 64, 1_g2)
#undef TCHEM_GB_DECLARE_SHAPE

namespace {

struct Variant {
  int MC, RPT, G;  // columns, rows per thread, warps per sample
  int max_warps;   // per CTA (the kernel's launch bounds)
  bool simplified;  // the form: TCHEM_GB_FORM_MIXED_SIMPLIFIED (else TCHEM_GB_FORM_MIXED)
  bool gj;          // Gauss-Jordan inverse (else LU)
  bool e3;          // E3SM inputs (per-sample rate constants and source terms)
  bool sp;          // static-order sparse LU (full Newton; needs the mechanism's LU program)
  const void* kernel;
  cudaError_t (*launch)(const AdvanceParams&, int, int, size_t, cudaStream_t);
};

// Kernel shapes of each form; a mechanism uses the first in table order with MC >= m and
// 32 G RPT >= m, among those with the requested threads per sample (32 G; 0: any). The E3SM time
// advance has its own instantiations (up to 64 species). In the full-Newton form, one warp per
// sample above 32 species is the static-order sparse LU (needs the mechanism's LU program); it
// comes after the Gauss-Jordan shapes, which measured faster (51 species: 5,621 against 3,248
// samples/s; 120 species: 436 against 238), so they are the default without a tuned preference.
const Variant* variants(int* n) {
  static const Variant v[] = {
      {24, 1, 1, 12, false, false, false, false, kernel_mixed_24_1(), &launch_mixed_24_1},
      {32, 1, 1, 12, false, false, false, false, kernel_mixed_32_1(), &launch_mixed_32_1},
      {52, 1, 2, 16, false, true, false, false, kernel_mixgj_52_1_g2(), &launch_mixgj_52_1_g2},
      {64, 1, 2, 12, false, true, false, false, kernel_mixgj_64_1_g2(), &launch_mixgj_64_1_g2},
      {128, 1, 4, 8, false, true, false, false, kernel_mixgj_128_1_g4(), &launch_mixgj_128_1_g4},
      {64, 2, 1, 16, false, true, false, true, kernel_mixsp_64_2(), &launch_mixsp_64_2},
      {128, 4, 1, 8, false, true, false, true, kernel_mixsp_128_4(), &launch_mixsp_128_4},
      {24, 1, 1, 12, true, true, false, false, kernel_simpl_24_1(), &launch_simpl_24_1},
      {32, 1, 1, 12, true, true, false, false, kernel_simpl_32_1(), &launch_simpl_32_1},
      {52, 2, 1, 8, true, true, false, false, kernel_simpl_52_2(), &launch_simpl_52_2},
      {64, 2, 1, 8, true, true, false, false, kernel_simpl_64_2(), &launch_simpl_64_2},
      {52, 1, 2, 16, true, true, false, false, kernel_simpl_52_1_g2(), &launch_simpl_52_1_g2},
      {64, 1, 2, 12, true, true, false, false, kernel_simpl_64_1_g2(), &launch_simpl_64_1_g2},
      {128, 1, 4, 8, true, true, false, false, kernel_simpl_128_1_g4(), &launch_simpl_128_1_g4},
      {64, 2, 1, 8, false, false, true, false, kernel_e3mixed_64_2(), &launch_e3mixed_64_2},
      {64, 2, 1, 8, true, true, true, false, kernel_e3simpl_64_2(), &launch_e3simpl_64_2},
      {64, 1, 2, 12, true, true, true, false, kernel_e3simpl_64_1_g2(), &launch_e3simpl_64_1_g2},
  };
  *n = static_cast<int>(sizeof(v) / sizeof(v[0]));
  return v;
}

const Variant* pick(const MechLayout& L, bool simplified, int threads_per_sample, bool e3, int lu_nnz) {
  int nv = 0;
  const Variant* v = variants(&nv);
  for (int i = 0; i < nv; ++i)
    if (v[i].simplified == simplified && v[i].e3 == e3 && v[i].MC >= L.m && 32 * v[i].G * v[i].RPT >= L.m &&
        (!v[i].sp || (lu_nnz > 0 && L.off_js_e >= 0)) &&
        (threads_per_sample == 0 || threads_per_sample == 32 * v[i].G))
      return &v[i];
  return nullptr;
}

}  // namespace

MixedConfig mixed_config(const MechLayout& L, int threads_per_sample, int sm_count, int max_smem_optin, int nbatch,
                         bool simplified, bool e3, int lu_nnz) {
  if (threads_per_sample != 0 && threads_per_sample != 32 && threads_per_sample != 64 && threads_per_sample != 128)
    throw std::domain_error("mixed forms: threads_per_sample must be 0, 32, 64 or 128");
  const Variant* best = pick(L, simplified, threads_per_sample, e3, lu_nnz);
  if (!best && e3)
    throw std::domain_error("E3SM time advance: the mixed forms have kernel shapes for up to 64 active species "
                            "(32 or 64 threads per sample for the simplified form, 32 for the FP32-LU form); "
                            "larger mechanisms use the plain form");
  if (!best)
    throw std::domain_error(simplified ? "simplified form: no kernel shape for this mechanism size and threads_per_sample "
                                         "(up to 64 species with 32 or 64 threads, 128 with 128 threads)"
                                       : "full-Newton FP32 form: no kernel shape for this mechanism size and "
                                         "threads_per_sample (LU up to 128 species with 32 threads; Gauss-Jordan "
                                         "up to 64 species with 64 threads, 128 with 128 threads)");
  MixedLayout ml = mixed::make_layout(L, best->MC, best->gj, e3, best->sp ? lu_nnz : 0);
  ml.simplified = simplified ? 1 : (best->gj ? 2 : 0);
  const size_t gbytes = ml.warp_bytes;
  const size_t avail = static_cast<size_t>(max_smem_optin) - 16 - L.blob_bytes;
  const int groups = static_cast<int>(std::min<size_t>(best->max_warps / best->G, avail / gbytes));
  if (groups < 1) throw std::domain_error("mixed form: shared-memory working set too large");
  const int warps = groups * best->G;
  MixedConfig mc;
  mc.kernel = best->kernel;
  mc.threads_per_sample = 32 * best->G;
  mc.ml = ml;
  mc.warps_per_block = warps;
  mc.smem = 16 + L.blob_bytes + groups * gbytes;
  cudaFuncSetAttribute(mc.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(mc.smem));
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, mc.kernel, warps * 32, mc.smem) != cudaSuccess || bps < 1)
    bps = 1;
  const int need = (std::max(nbatch, 1) + groups - 1) / groups;
  mc.grid = std::max(1, std::min(sm_count * bps, need));
  return mc;
}

cudaError_t launch_trbdf2_mixed(const AdvanceParams& P, const MechLayout& L, int grid, int warps_per_block,
                                size_t smem, int threads_per_sample, cudaStream_t stream) {
  const int lu_nnz = P.mech.lu_prog ? P.mech.lu.nnz : 0;
  const Variant* best = pick(L, P.ml.simplified == 1, threads_per_sample, P.keff_in != nullptr, lu_nnz);
  if (!best) return cudaErrorInvalidValue;
  return best->launch(P, grid, warps_per_block * 32, smem, stream);
}

}  // namespace tchem_gb
