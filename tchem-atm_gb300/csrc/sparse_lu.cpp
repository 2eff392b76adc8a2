// Static-order sparse LU: ordering, fill and the device program (see sparse_lu.hpp).
#include "sparse_lu.hpp"

#include <stdexcept>

namespace tchem_gb {

SparseLuHost build_sparse_lu(int m, const std::vector<std::pair<int, int>>& nonzeros) {
  if (m < 1 || m > kSparseLuMaxSpecies) throw std::invalid_argument("sparse LU: mechanism size out of range");
  // pattern in species space, with the diagonal
  std::vector<char> A(static_cast<size_t>(m) * m, 0);
  auto at = [&](int i, int j) -> char& { return A[static_cast<size_t>(i) * m + j]; };
  for (int i = 0; i < m; ++i) at(i, i) = 1;
  for (const auto& z : nonzeros) {
    if (z.first < 0 || z.first >= m || z.second < 0 || z.second >= m)
      throw std::invalid_argument("sparse LU: Jacobian nonzero outside the active species");
    at(z.first, z.second) = 1;
  }
  // greedy Markowitz order with symbolic elimination (fill recorded in A)
  SparseLuHost h;
  std::vector<char> done(m, 0);
  h.order.reserve(m);
  for (int step = 0; step < m; ++step) {
    int best = -1;
    long best_score = 0;
    for (int j = 0; j < m; ++j) {
      if (done[j]) continue;
      long r = 0, c = 0;
      for (int t = 0; t < m; ++t)
        if (!done[t]) {
          r += at(j, t);
          c += at(t, j);
        }
      const long score = (r - 1) * (c - 1);
      if (best < 0 || score < best_score) {
        best = j;
        best_score = score;
      }
    }
    done[best] = 1;
    h.order.push_back(best);
    for (int i = 0; i < m; ++i) {
      if (done[i] || !at(i, best)) continue;
      for (int j = 0; j < m; ++j)
        if (!done[j] && at(best, j)) at(i, j) = 1;
    }
  }
  h.pos.assign(m, 0);
  for (int k = 0; k < m; ++k) h.pos[h.order[k]] = k;
  // entries of the filled pattern, row-major in position order
  h.entry.assign(static_cast<size_t>(m) * m, -1);
  auto F = [&](int k, int l) { return at(h.order[k], h.order[l]) != 0; };
  int nnz = 0;
  for (int k = 0; k < m; ++k)
    for (int l = 0; l < m; ++l)
      if (F(k, l)) h.entry[static_cast<size_t>(k) * m + l] = nnz++;
  // entries travel as 16-bit fields (signed in the sliced-ELL slot table)
  if (nnz > 0x7fff) throw std::invalid_argument("sparse LU: too many entries for the program encoding");
  auto E = [&](int k, int l) { return h.entry[static_cast<size_t>(k) * m + l]; };

  SparseLuLayout& L = h.lay;
  L.m = m;
  L.nnz = nnz;
  std::vector<int32_t>& p = h.prog;
  L.off_diag = static_cast<int32_t>(p.size());
  for (int k = 0; k < m; ++k) p.push_back(E(k, k));
  L.off_pos = static_cast<int32_t>(p.size());
  for (int s = 0; s < m; ++s) p.push_back(h.pos[s]);
  // column k of L (rows below) and of U (rows above)
  std::vector<int32_t> lc_ptr{0}, lc, uc_ptr{0}, uc;
  for (int k = 0; k < m; ++k) {
    for (int i = k + 1; i < m; ++i)
      if (E(i, k) >= 0) lc.push_back(E(i, k) | (i << 16));
    lc_ptr.push_back(static_cast<int32_t>(lc.size()));
    for (int i = 0; i < k; ++i)
      if (E(i, k) >= 0) uc.push_back(E(i, k) | (i << 16));
    uc_ptr.push_back(static_cast<int32_t>(uc.size()));
  }
  // trailing updates of step k
  std::vector<int32_t> up_ptr{0}, up;
  for (int k = 0; k < m; ++k) {
    for (int i = k + 1; i < m; ++i) {
      if (E(i, k) < 0) continue;
      for (int j = k + 1; j < m; ++j) {
        if (E(k, j) < 0) continue;
        const int dst = E(i, j);
        if (dst < 0) throw std::logic_error("sparse LU: fill entry missing from the pattern");
        up.push_back(dst | (E(i, k) << 16));
        up.push_back(E(k, j));
      }
    }
    up_ptr.push_back(static_cast<int32_t>(up.size() / 2));
  }
  L.n_ops = static_cast<int32_t>(up.size() / 2);
  auto append = [&](const std::vector<int32_t>& v) {
    const int32_t o = static_cast<int32_t>(p.size());
    p.insert(p.end(), v.begin(), v.end());
    return o;
  };
  L.off_lc_ptr = append(lc_ptr);
  L.off_lc = append(lc);
  L.off_uc_ptr = append(uc_ptr);
  L.off_uc = append(uc);
  L.off_up_ptr = append(up_ptr);
  if (p.size() % 2) p.push_back(0);  // the update pairs start on an 8-byte boundary (int2 loads)
  L.off_up = append(up);
  L.prog_len = static_cast<int32_t>(p.size());
  return h;
}

}  // namespace tchem_gb
