// Static-order sparse LU of the Newton matrix I - c J (the sparse-LU shape of the full-Newton FP32
// form, kernels_mixed_impl.cuh).
//
// The reference factors the dense Newton matrix with partial pivoting inside Tines
// (src/core/problems/TChem_Impl_AtmosphericChemistry.hpp:138-155). A chemistry Jacobian is sparse
// (the 51-species / 156-reaction benchmark mechanism: 507 of 2,601 entries), so here the structure
// is analysed once per mechanism: a greedy Markowitz order on the diagonal (the remaining species
// with the smallest (row count - 1) x (column count - 1), ties to the lowest species index), the
// fill of that elimination, and a program of index lists that a warp runs per factorization
// without any pivot search. The matrix I - c J of a mass-conserving mechanism has a diagonal of
// 1 + c x (loss rate) >= 1; the kernel still tests every pivot (zero or non-finite: the Newton solve
// fails, as the dense form's does), and the FP64-residual refinement sweep of every solve absorbs
// the FP32 rounding of the factors.
//
// Entries of the filled pattern are numbered row-major in position order (position k holds
// species order[k]). The program is one int32 array with sections (offsets in SparseLuLayout):
//   diag[m]        entry of (k, k)
//   pos[m]         position of each species
//   lc_ptr[m+1], lc[]  column k of L below the diagonal: entry | (row << 16)
//   uc_ptr[m+1], uc[]  column k of U above the diagonal: entry | (row << 16)
//   up_ptr[m+1], up[]  the trailing updates of step k, two int32 each: dst | (l << 16), u
//                      (a(dst) -= a(l) * a(u) with l = (i, k), u = (k, j), dst = (i, j))
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

namespace tchem_gb {

struct SparseLuLayout {
  int32_t m = 0, nnz = 0, n_ops = 0, prog_len = 0;
  int32_t off_diag = -1, off_pos = -1, off_lc_ptr = -1, off_lc = -1, off_uc_ptr = -1, off_uc = -1, off_up_ptr = -1,
          off_up = -1;
};

struct SparseLuHost {
  SparseLuLayout lay;
  std::vector<int32_t> order;  // position -> species
  std::vector<int32_t> pos;    // species -> position
  std::vector<int32_t> entry;  // [m * m] entry of (position row, position col), -1 outside the pattern
  std::vector<int32_t> prog;
};

// Largest mechanism the program encoding covers (entries and rows in 16 bits).
constexpr int kSparseLuMaxSpecies = 128;

// nonzeros: (row, col) species pairs of the Jacobian (the diagonal is always included).
SparseLuHost build_sparse_lu(int m, const std::vector<std::pair<int, int>>& nonzeros);

}  // namespace tchem_gb
