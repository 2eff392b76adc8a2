// Builds and uploads the packed per-mechanism tables (layout in device_tables.hpp).
#include "device_tables.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>

namespace tchem_gb {

namespace {

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename T>
void put(std::vector<unsigned char>& blob, int32_t off, const std::vector<T>& v) {
  if (!v.empty()) std::memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
}

// Sliced-ELL layout of variable-length lists: items sorted by length (descending, stable), 32 per
// slice; slice s holds cnt[s] entry rows of 32 lanes starting at entry off[s]; short lists are
// padded with (dummy, 0). item[s * 32 + lane] is the item id, or -1 for a padding lane.
struct Sliced {
  std::vector<int32_t> item, cnt, off;
  std::vector<int16_t> idx;
  std::vector<double> val;
};

Sliced make_slices(const std::vector<std::vector<std::pair<int, double>>>& lists, const std::vector<int32_t>& ids,
                   int16_t dummy) {
  const int n = static_cast<int>(lists.size());
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return lists[a].size() > lists[b].size(); });
  Sliced s;
  const int nsl = (n + 31) / 32;
  int32_t e = 0;
  for (int sl = 0; sl < nsl; ++sl) {
    int c = 0;
    for (int l = 0; l < 32; ++l) {
      const int k = sl * 32 + l;
      s.item.push_back(k < n ? ids[order[k]] : -1);
      if (k < n) c = std::max(c, static_cast<int>(lists[order[k]].size()));
    }
    s.cnt.push_back(c);
    s.off.push_back(e);
    for (int r = 0; r < c; ++r) {
      for (int l = 0; l < 32; ++l) {
        const int k = sl * 32 + l;
        if (k < n && r < static_cast<int>(lists[order[k]].size())) {
          s.idx.push_back(static_cast<int16_t>(lists[order[k]][r].first));
          s.val.push_back(lists[order[k]][r].second);
        } else {
          s.idx.push_back(dummy);
          s.val.push_back(0.0);
        }
      }
    }
    e += 32 * c;
  }
  return s;
}

}  // namespace

HostTables build_host_tables(const KineticModel& km) {
  HostTables ht;
  const int m = km.nActive(), n = km.nSpec, R = km.nReac, S = km.maxSpecInReac, joff = S / 2;
  if (m <= 0) throw std::runtime_error("mechanism has no active species");
  if (m >= 32768 || R >= 32768) throw std::runtime_error("mechanism too large for the device tables");

  // Stoichiometry by reaction, as the reference stores it.
  ht.rx_S = S;
  ht.rx_sidx.assign(km.reacSidx.begin(), km.reacSidx.end());
  ht.rx_nu.assign(km.reacNuki.begin(), km.reacNuki.end());
  ht.rx_n.resize(static_cast<size_t>(R) * 2);
  for (int r = 0; r < R; ++r) {
    ht.rx_n[2 * r] = km.reacNreac[r];
    ht.rx_n[2 * r + 1] = km.reacNprod[r];
  }

  // Rate parameters per reaction.
  ht.rate_type.assign(R, RATE_ZERO);
  ht.rate_param.assign(static_cast<size_t>(R) * 8, 0.0);
  ht.conv_exp.assign(km.convExponent.begin(), km.convExponent.end());
  for (const auto& a : km.arrhenius) {
    ht.rate_type[a.reaction_index] = RATE_ARRHENIUS;
    double* p = &ht.rate_param[static_cast<size_t>(a.reaction_index) * 8];
    p[0] = a.A; p[1] = a.B; p[2] = a.C; p[3] = a.D; p[4] = a.E;
  }
  for (size_t i = 0; i < km.reacPfal.size(); ++i) {
    const int r = km.reacPfal[i];
    ht.rate_type[r] = RATE_TROE;
    for (int k = 0; k < 8; ++k) ht.rate_param[static_cast<size_t>(r) * 8 + k] = km.reacPpar[i * 8 + k];
  }
  for (const auto& c : km.cmaq_h2o2) {
    ht.rate_type[c.reaction_index] = RATE_CMAQ_H2O2;
    double* p = &ht.rate_param[static_cast<size_t>(c.reaction_index) * 8];
    p[0] = c.A1; p[1] = c.B1; p[2] = c.C1; p[3] = c.A2; p[4] = c.B2; p[5] = c.C2;
  }
  for (int r = 0; r < R; ++r) {
    const int t = km.reacType[r];
    if (t == KineticModel::JPL || t == KineticModel::R_JPL_ARRHENIUS || t == KineticModel::PHOTO_RATE) {
      ht.supported = false;
      ht.unsupported_reason = "reaction " + std::to_string(r) +
                              " uses a JPL, R_JPL_ARRHENIUS or PHOTO_RATE rate: the box-model time advance "
                              "evaluates ARRHENIUS, TROE and CMAQ_H2O2 rates only";
    }
  }

  // E3SM rate tables.
  ht.e3_type.assign(R, E3_NONE);
  ht.e3_param.assign(static_cast<size_t>(R) * kE3smParams, 0.0);
  auto e3p = [&](int r) { return &ht.e3_param[static_cast<size_t>(r) * kE3smParams]; };
  for (const auto& a : km.arrhenius) {
    ht.e3_type[a.reaction_index] = E3_ARRHENIUS;
    double* p = e3p(a.reaction_index);
    p[0] = a.A; p[1] = a.B; p[2] = a.C; p[3] = a.D; p[4] = a.E;
  }
  for (size_t i = 0; i < km.reacPfal.size(); ++i) {
    ht.e3_type[km.reacPfal[i]] = E3_TROE;
    for (int k = 0; k < 8; ++k) e3p(km.reacPfal[i])[k] = km.reacPpar[i * 8 + k];
  }
  for (const auto& c : km.cmaq_h2o2) {
    ht.e3_type[c.reaction_index] = E3_CMAQ_H2O2;
    double* p = e3p(c.reaction_index);
    p[0] = c.A1; p[1] = c.B1; p[2] = c.C1; p[3] = c.A2; p[4] = c.B2; p[5] = c.C2;
  }
  for (const auto& j : km.jpl) {
    ht.e3_type[j.reaction_index] = E3_JPL;
    double* p = e3p(j.reaction_index);
    p[0] = j.k0_A; p[1] = j.k0_B; p[2] = j.k0_C; p[3] = j.kinf_A; p[4] = j.kinf_B; p[5] = j.kinf_C; p[6] = j.Fc;
  }
  for (const auto& j : km.r_jpl_arrhenius) {
    ht.e3_type[j.reaction_index] = E3_RJPL;
    double* p = e3p(j.reaction_index);
    p[0] = j.k0_A; p[1] = j.k0_B; p[2] = j.k0_C; p[3] = j.kinf_A; p[4] = j.kinf_B; p[5] = j.kinf_C; p[6] = j.Fc;
    p[7] = j.A; p[8] = j.B; p[9] = j.C;
  }
  // Adjust factors grouped by reaction, file order kept within each reaction: applying them per
  // reaction in parallel gives the products of the reference's serial pass, bit for bit.
  {
    std::vector<std::vector<int32_t>> per_r(R);
    for (const auto& a : km.adjust_reaction) per_r[a.reaction_index].push_back(a.species_index);
    ht.e3_adj_ptr.assign(R + 1, 0);
    for (int r = 0; r < R; ++r) {
      ht.e3_adj_ptr[r] = static_cast<int32_t>(ht.e3_adj_sp.size());
      ht.e3_adj_sp.insert(ht.e3_adj_sp.end(), per_r[r].begin(), per_r[r].end());
    }
    ht.e3_adj_ptr[R] = static_cast<int32_t>(ht.e3_adj_sp.size());
  }
  for (const auto& a : km.adjust_reaction) {
    if (a.species_index < m) {
      ht.e3sm_state_free = false;
      ht.e3sm_reason = "adjust_reaction of reaction " + std::to_string(a.reaction_index) + " names the active species " +
                       km.speciesNames[a.species_index];
    }
  }
  for (const auto& o : km.prod_O1D) {
    const int32_t idx[7] = {o.reaction_indices[0], o.reaction_indices[1], o.reaction_indices[2],
                            o.photolysis_reaction_index, o.species_index_1, o.species_index_2, o.species_index_3};
    bool in_range = true;
    for (int k = 0; k < 7; ++k) in_range = in_range && idx[k] >= 0 && idx[k] < (k < 4 ? R : n);
    if (!in_range) {
      ht.e3sm_valid = false;
      ht.e3sm_invalid_reason = "modifier_prod_O1D: a reaction or species index is out of range";
      continue;
    }
    ht.e3_o1d.insert(ht.e3_o1d.end(), idx, idx + 7);
    const double par[6] = {o.A1, o.C1, o.A2, o.C2, o.A3, o.C3};
    ht.e3_o1d_par.insert(ht.e3_o1d_par.end(), par, par + 6);
    for (int k = 4; k < 7; ++k)
      if (idx[k] < m) {
        ht.e3sm_state_free = false;
        ht.e3sm_reason = "modifier_prod_O1D names the active species " + km.speciesNames[idx[k]];
      }
  }
  ht.M_index = km.M_index;
  if ((!km.jpl.empty() || !km.r_jpl_arrhenius.empty()) && km.M_index < m) {
    ht.e3sm_state_free = false;
    ht.e3sm_reason = "the JPL rate forms read [M] and M is an active species";
  }
  if (!ht.e3sm_state_free)
    ht.e3sm_reason += ": the E3SM time advance evaluates rate constants once per sample and needs them to depend "
                      "on constant species only";

  // Factor slots (rate of progress) and constant-species factors.
  std::vector<int32_t> rf_ptr(R + 1, 0);
  std::vector<int16_t> rf_sp;
  ht.cf_ptr.assign(R + 1, 0);
  int max_factors = 0;
  for (int r = 0; r < R; ++r) {
    rf_ptr[r] = static_cast<int32_t>(rf_sp.size());
    ht.cf_ptr[r] = static_cast<int32_t>(ht.cf_idx.size());
    for (int j = 0; j < km.reacNreac[r]; ++j) {
      const int s = km.sidx(r, j);
      const int pw = std::abs(static_cast<int>(km.nuki(r, j)));
      for (int k = 0; k < pw; ++k) {
        if (s < m) rf_sp.push_back(static_cast<int16_t>(s));
        else ht.cf_idx.push_back(s - m);
      }
    }
    max_factors = std::max(max_factors, static_cast<int>(rf_sp.size()) - rf_ptr[r]);
  }
  rf_ptr[R] = static_cast<int32_t>(rf_sp.size());
  ht.cf_ptr[R] = static_cast<int32_t>(ht.cf_idx.size());

  // Per reaction, the (species, nu) entries in the reference's scatter order: reactant slots,
  // then product slots; constant species and zero coefficients are skipped.
  std::vector<std::vector<std::pair<int, double>>> rxn_entries(R);
  for (int r = 0; r < R; ++r) {
    for (int j = 0; j < km.reacNreac[r]; ++j) {
      const int s = km.sidx(r, j);
      const double nu = km.nuki(r, j);
      if (s < m && nu != 0.0) rxn_entries[r].push_back({s, nu});
    }
    for (int j = 0; j < km.reacNprod[r]; ++j) {
      const int s = km.sidx(r, j + joff);
      const double nu = km.nuki(r, j + joff);
      if (s < m && nu != 0.0) rxn_entries[r].push_back({s, nu});
    }
  }

  // Net production CSR over active species, reactions in ascending order.
  std::vector<std::vector<std::pair<int, double>>> per_species(m);
  for (int r = 0; r < R; ++r)
    for (const auto& e : rxn_entries[r]) per_species[e.first].push_back({r, e.second});
  std::vector<int32_t> pr_ptr(m + 1, 0);
  std::vector<int16_t> pr_r;
  std::vector<double> pr_nu;
  for (int k = 0; k < m; ++k) {
    pr_ptr[k] = static_cast<int32_t>(pr_r.size());
    for (const auto& e : per_species[k]) {
      pr_r.push_back(static_cast<int16_t>(e.first));
      pr_nu.push_back(e.second);
    }
  }
  pr_ptr[m] = static_cast<int32_t>(pr_r.size());

  // Jacobian nonzeros (row-major) with their contributions.
  std::map<std::pair<int, int>, std::vector<std::pair<int, double>>> jac;
  for (int r = 0; r < R; ++r)
    for (int f = rf_ptr[r]; f < rf_ptr[r + 1]; ++f)
      for (const auto& e : rxn_entries[r]) jac[{e.first, rf_sp[f]}].push_back({f, e.second});
  std::vector<int32_t> jz_rc, jz_ptr;
  std::vector<int16_t> jc_f;
  std::vector<double> jc_nu;
  std::vector<float> jc_nu32;
  for (const auto& kv : jac) {
    jz_rc.push_back((kv.first.first << 16) | kv.first.second);
    jz_ptr.push_back(static_cast<int32_t>(jc_f.size()));
    for (const auto& c : kv.second) {
      jc_f.push_back(static_cast<int16_t>(c.first));
      jc_nu.push_back(c.second);
      jc_nu32.push_back(static_cast<float>(c.second));
    }
  }
  jz_ptr.push_back(static_cast<int32_t>(jc_f.size()));

  std::vector<double> emis(m, 0.0);
  for (const auto& e : km.emission)
    if (e.species_index < m) emis[e.species_index] = e.emission_rate;  // last entry wins, as the reference's assignment

  MechLayout& L = ht.L;
  L.m = m; L.n = n; L.nconst = n - m; L.R = R;
  L.NF = static_cast<int32_t>(rf_sp.size());
  L.NP = static_cast<int32_t>(pr_r.size());
  L.NZ = static_cast<int32_t>(jz_rc.size());
  L.NC = static_cast<int32_t>(jc_f.size());
  L.max_factors = max_factors;
  size_t off = 0;
  auto sec = [&](size_t bytes) { const int32_t o = static_cast<int32_t>(off); off = align16(off + bytes); return o; };
  L.off_emis = sec(sizeof(double) * m);
  L.off_rf_ptr = sec(sizeof(int32_t) * (R + 1));
  L.off_pr_ptr = sec(sizeof(int32_t) * (m + 1));
  L.off_pr_nu = sec(sizeof(double) * pr_nu.size());
  L.off_jz_rc = sec(sizeof(int32_t) * jz_rc.size());
  L.off_jz_ptr = sec(sizeof(int32_t) * jz_ptr.size());
  L.off_jc_nu = sec(sizeof(double) * jc_nu.size());
  L.off_jc_nu32 = sec(sizeof(float) * jc_nu32.size());
  L.off_rf_sp = sec(sizeof(int16_t) * rf_sp.size());
  L.off_pr_r = sec(sizeof(int16_t) * pr_r.size());
  L.off_jc_f = sec(sizeof(int16_t) * jc_f.size());
  L.off_js_e = -1;
  L.blob_bytes = static_cast<int32_t>(align16(off));
  ht.blob.assign(L.blob_bytes, 0);
  put(ht.blob, L.off_emis, emis);
  put(ht.blob, L.off_rf_ptr, rf_ptr);
  put(ht.blob, L.off_rf_sp, rf_sp);
  put(ht.blob, L.off_pr_ptr, pr_ptr);
  put(ht.blob, L.off_pr_r, pr_r);
  put(ht.blob, L.off_pr_nu, pr_nu);
  put(ht.blob, L.off_jz_rc, jz_rc);
  put(ht.blob, L.off_jz_ptr, jz_ptr);
  put(ht.blob, L.off_jc_f, jc_f);
  put(ht.blob, L.off_jc_nu, jc_nu);
  put(ht.blob, L.off_jc_nu32, jc_nu32);

  // Mixed-form blob: the same rate-of-progress program plus sliced-ELL programs.
  {
    std::vector<std::vector<std::pair<int, double>>> jlists;
    std::vector<int32_t> jids;
    for (const auto& kv : jac) {
      jids.push_back((kv.first.first << 16) | kv.first.second);
      jlists.push_back(kv.second);
    }
    std::vector<int32_t> wids(m);
    for (int k = 0; k < m; ++k) wids[k] = k;
    const Sliced js = make_slices(jlists, jids, static_cast<int16_t>(L.NF));
    // sparse-LU entry of every Jacobian slot (padding lanes: 0, never written)
    std::vector<int16_t> js_e;
    if (m <= kSparseLuMaxSpecies) {
      std::vector<std::pair<int, int>> nz;
      for (const auto& kv : jac) nz.push_back(kv.first);
      try {
        ht.slu = build_sparse_lu(m, nz);
      } catch (const std::exception&) {
        ht.slu = SparseLuHost{};  // no program: the sparse-LU shapes are not offered
      }
      if (ht.slu.lay.m == m)
        for (int32_t rc : js.item) {
          int e = 0;
          if (rc >= 0) e = ht.slu.entry[static_cast<size_t>(ht.slu.pos[rc >> 16]) * m + ht.slu.pos[rc & 0xffff]];
          js_e.push_back(static_cast<int16_t>(e));
        }
    }
    const Sliced ws = make_slices(per_species, wids, static_cast<int16_t>(R));
    std::vector<float> jse_nu32(js.val.begin(), js.val.end());
    MechLayout& X = ht.Lx;
    X = L;
    X.NJS = static_cast<int32_t>(js.cnt.size());
    X.NJE = static_cast<int32_t>(js.idx.size());
    X.NWS = static_cast<int32_t>(ws.cnt.size());
    X.NWE = static_cast<int32_t>(ws.idx.size());
    size_t o = 0;
    auto sx = [&](size_t bytes) { const int32_t r = static_cast<int32_t>(o); o = align16(o + bytes); return r; };
    X.off_emis = sx(sizeof(double) * m);
    X.off_rf_ptr = sx(sizeof(int32_t) * (R + 1));
    X.off_wse_nu = sx(sizeof(double) * ws.val.size());
    X.off_js_rc = sx(sizeof(int32_t) * js.item.size());
    X.off_js_cnt = sx(sizeof(int32_t) * js.cnt.size());
    X.off_js_off = sx(sizeof(int32_t) * js.off.size());
    X.off_jse_nu32 = sx(sizeof(float) * jse_nu32.size());
    X.off_ws_sp = sx(sizeof(int32_t) * ws.item.size());
    X.off_ws_cnt = sx(sizeof(int32_t) * ws.cnt.size());
    X.off_ws_off = sx(sizeof(int32_t) * ws.off.size());
    X.off_rf_sp = sx(sizeof(int16_t) * rf_sp.size());
    X.off_jse_f = sx(sizeof(int16_t) * js.idx.size());
    X.off_wse_r = sx(sizeof(int16_t) * ws.idx.size());
    X.off_js_e = js_e.empty() ? -1 : sx(sizeof(int16_t) * js_e.size());
    // CSR sections are not part of the mixed blob
    X.off_pr_ptr = X.off_pr_r = X.off_pr_nu = X.off_jz_rc = X.off_jz_ptr = X.off_jc_f = X.off_jc_nu = X.off_jc_nu32 = -1;
    X.blob_bytes = static_cast<int32_t>(align16(o));
    ht.blob_x.assign(X.blob_bytes, 0);
    put(ht.blob_x, X.off_emis, emis);
    put(ht.blob_x, X.off_rf_ptr, rf_ptr);
    put(ht.blob_x, X.off_rf_sp, rf_sp);
    put(ht.blob_x, X.off_js_rc, js.item);
    put(ht.blob_x, X.off_js_cnt, js.cnt);
    put(ht.blob_x, X.off_js_off, js.off);
    put(ht.blob_x, X.off_jse_f, js.idx);
    put(ht.blob_x, X.off_jse_nu32, jse_nu32);
    put(ht.blob_x, X.off_ws_sp, ws.item);
    put(ht.blob_x, X.off_ws_cnt, ws.cnt);
    put(ht.blob_x, X.off_ws_off, ws.off);
    put(ht.blob_x, X.off_wse_r, ws.idx);
    put(ht.blob_x, X.off_wse_nu, ws.val);
    if (!js_e.empty()) put(ht.blob_x, X.off_js_e, js_e);
  }

  // Structural signature: everything except the rate parameters.
  auto mix = [&](int64_t v) { ht.signature.push_back(v); };
  mix(m); mix(n); mix(R);
  for (unsigned char b : ht.blob) mix(b);
  for (int32_t v : ht.cf_ptr) mix(v);
  for (int32_t v : ht.cf_idx) mix(v);
  for (int32_t v : ht.conv_exp) mix(v);
  for (int32_t v : ht.rate_type) mix(v);
  return ht;
}

DeviceTables* upload_tables(const HostTables& ht, int device) {
  const MechLayout& L = ht.L;
  const size_t R = static_cast<size_t>(L.R);
  size_t off = 0;
  auto sec = [&](size_t bytes) { const size_t o = off; off = (off + bytes + 255) & ~size_t(255); return o; };
  const size_t o_blob = sec(L.blob_bytes);
  const size_t o_blob_x = sec(ht.Lx.blob_bytes);
  const size_t o_type = sec(sizeof(int32_t) * R);
  const size_t o_param = sec(sizeof(double) * R * 8);
  const size_t o_conv = sec(sizeof(int32_t) * R);
  const size_t o_cfp = sec(sizeof(int32_t) * (R + 1));
  const size_t o_cfi = sec(sizeof(int32_t) * std::max<size_t>(1, ht.cf_idx.size()));
  const size_t o_rxs = sec(sizeof(int32_t) * ht.rx_sidx.size());
  const size_t o_rxnu = sec(sizeof(double) * ht.rx_nu.size());
  const size_t o_rxn = sec(sizeof(int32_t) * ht.rx_n.size());
  const size_t o_e3t = sec(sizeof(int32_t) * R);
  const size_t o_e3p = sec(sizeof(double) * R * kE3smParams);
  const size_t o_e3ap = sec(sizeof(int32_t) * (R + 1));
  const size_t o_e3a = sec(sizeof(int32_t) * std::max<size_t>(1, ht.e3_adj_sp.size()));
  const size_t o_e3o = sec(sizeof(int32_t) * std::max<size_t>(1, ht.e3_o1d.size()));
  const size_t o_e3op = sec(sizeof(double) * std::max<size_t>(1, ht.e3_o1d_par.size()));
  const size_t o_lu = sec(sizeof(int32_t) * std::max<size_t>(1, ht.slu.prog.size()));
  std::vector<unsigned char> host(off, 0);
  std::memcpy(host.data() + o_blob, ht.blob.data(), ht.blob.size());
  std::memcpy(host.data() + o_blob_x, ht.blob_x.data(), ht.blob_x.size());
  std::memcpy(host.data() + o_type, ht.rate_type.data(), sizeof(int32_t) * R);
  std::memcpy(host.data() + o_param, ht.rate_param.data(), sizeof(double) * R * 8);
  std::memcpy(host.data() + o_conv, ht.conv_exp.data(), sizeof(int32_t) * R);
  std::memcpy(host.data() + o_cfp, ht.cf_ptr.data(), sizeof(int32_t) * (R + 1));
  if (!ht.cf_idx.empty()) std::memcpy(host.data() + o_cfi, ht.cf_idx.data(), sizeof(int32_t) * ht.cf_idx.size());
  std::memcpy(host.data() + o_rxs, ht.rx_sidx.data(), sizeof(int32_t) * ht.rx_sidx.size());
  std::memcpy(host.data() + o_rxnu, ht.rx_nu.data(), sizeof(double) * ht.rx_nu.size());
  std::memcpy(host.data() + o_rxn, ht.rx_n.data(), sizeof(int32_t) * ht.rx_n.size());
  std::memcpy(host.data() + o_e3t, ht.e3_type.data(), sizeof(int32_t) * R);
  std::memcpy(host.data() + o_e3p, ht.e3_param.data(), sizeof(double) * R * kE3smParams);
  std::memcpy(host.data() + o_e3ap, ht.e3_adj_ptr.data(), sizeof(int32_t) * (R + 1));
  if (!ht.e3_adj_sp.empty())
    std::memcpy(host.data() + o_e3a, ht.e3_adj_sp.data(), sizeof(int32_t) * ht.e3_adj_sp.size());
  if (!ht.e3_o1d.empty()) std::memcpy(host.data() + o_e3o, ht.e3_o1d.data(), sizeof(int32_t) * ht.e3_o1d.size());
  if (!ht.e3_o1d_par.empty())
    std::memcpy(host.data() + o_e3op, ht.e3_o1d_par.data(), sizeof(double) * ht.e3_o1d_par.size());
  if (!ht.slu.prog.empty())
    std::memcpy(host.data() + o_lu, ht.slu.prog.data(), sizeof(int32_t) * ht.slu.prog.size());

  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) throw std::runtime_error("cudaSetDevice failed");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, off);
  if (e != cudaSuccess) {
    cudaSetDevice(prev);
    throw std::runtime_error(std::string("cudaMalloc for mechanism tables: ") + cudaGetErrorString(e));
  }
  e = cudaMemcpy(p, host.data(), off, cudaMemcpyHostToDevice);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaFree(p);
    throw std::runtime_error(std::string("cudaMemcpy for mechanism tables: ") + cudaGetErrorString(e));
  }
  auto* t = new DeviceTables();
  t->device = device;
  t->allocation = p;
  unsigned char* b = static_cast<unsigned char*>(p);
  t->dev.L = L;
  t->dev.blob = b + o_blob;
  t->dev.rate_type = reinterpret_cast<const int32_t*>(b + o_type);
  t->dev.rate_param = reinterpret_cast<const double*>(b + o_param);
  t->dev.conv_exp = reinterpret_cast<const int32_t*>(b + o_conv);
  t->dev.cf_ptr = reinterpret_cast<const int32_t*>(b + o_cfp);
  t->dev.cf_idx = reinterpret_cast<const int32_t*>(b + o_cfi);
  t->dev.conv_ppm = CONV_PPM;
  t->dev.rx_sidx = reinterpret_cast<const int32_t*>(b + o_rxs);
  t->dev.rx_nu = reinterpret_cast<const double*>(b + o_rxnu);
  t->dev.rx_n = reinterpret_cast<const int32_t*>(b + o_rxn);
  t->dev.rx_S = ht.rx_S;
  t->dev.e3_type = reinterpret_cast<const int32_t*>(b + o_e3t);
  t->dev.e3_param = reinterpret_cast<const double*>(b + o_e3p);
  t->dev.e3_adj_ptr = reinterpret_cast<const int32_t*>(b + o_e3ap);
  t->dev.e3_adj_sp = reinterpret_cast<const int32_t*>(b + o_e3a);
  t->dev.e3_o1d = reinterpret_cast<const int32_t*>(b + o_e3o);
  t->dev.e3_o1d_par = reinterpret_cast<const double*>(b + o_e3op);
  t->dev.e3_no1d = static_cast<int32_t>(ht.e3_o1d.size() / 7);
  t->dev.M_index = ht.M_index;
  t->dev.lu_prog = ht.slu.prog.empty() ? nullptr : reinterpret_cast<const int32_t*>(b + o_lu);
  t->dev.lu = ht.slu.lay;
  t->dev_x = t->dev;
  t->dev_x.L = ht.Lx;
  t->dev_x.blob = b + o_blob_x;
  return t;
}

void destroy_device_tables(DeviceTables* t) {
  if (!t) return;
  if (t->allocation) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(t->device);
    cudaFree(t->allocation);
    cudaSetDevice(prev);
  }
  delete t;
}

}  // namespace tchem_gb
