// C ABI: mechanism and scenario entry points (host only).
#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>

#include "mech_host.hpp"
#include "yaml_lite.hpp"

namespace tchem_gb {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }

void destroy_device_tables(DeviceTables* t);  // defined with the device code

}  // namespace tchem_gb

using tchem_gb::set_last_error;

void tchem_gb_mech::build_view() {
  const auto& k = km;
  arrhenius_reaction.clear();
  arrhenius_param.clear();
  for (const auto& a : k.arrhenius) {
    arrhenius_reaction.push_back(a.reaction_index);
    const double p[5] = {a.E, a.A, a.B, a.C, a.D};
    arrhenius_param.insert(arrhenius_param.end(), p, p + 5);
  }
  cmaq_reaction.clear();
  cmaq_param.clear();
  for (const auto& c : k.cmaq_h2o2) {
    cmaq_reaction.push_back(c.reaction_index);
    const double p[6] = {c.A1, c.B1, c.C1, c.A2, c.B2, c.C2};
    cmaq_param.insert(cmaq_param.end(), p, p + 6);
  }
  emission_species.clear();
  emission_rate.clear();
  for (const auto& e : k.emission) {
    emission_species.push_back(e.species_index);
    emission_rate.push_back(e.emission_rate);
  }
  reacPfal.assign(k.reacPfal.begin(), k.reacPfal.end());

  view.nSpec = k.nSpec;
  view.nConstSpec = k.nConstSpec;
  view.nReac = k.nReac;
  view.maxSpecInReac = k.maxSpecInReac;
  view.M_index = k.M_index;
  view.CONV_PPM = k.CONV_PPM_;
  view.reacNreac = k.reacNreac.data();
  view.reacNprod = k.reacNprod.data();
  view.reacSidx = k.reacSidx.data();
  view.reacNuki = k.reacNuki.data();
  view.convExponent = k.convExponent.data();
  view.reacType = k.reacType.data();
  view.nArrhenius = static_cast<int32_t>(arrhenius_reaction.size());
  view.arrhenius_reaction = arrhenius_reaction.data();
  view.arrhenius_param = arrhenius_param.data();
  view.nTroe = static_cast<int32_t>(reacPfal.size());
  view.reacPfal = reacPfal.data();
  view.reacPpar = k.reacPpar.data();
  view.nCMAQ_H2O2 = static_cast<int32_t>(cmaq_reaction.size());
  view.cmaq_reaction = cmaq_reaction.data();
  view.cmaq_param = cmaq_param.data();
  view.nEmission = static_cast<int32_t>(emission_species.size());
  view.emission_species = emission_species.data();
  view.emission_rate = emission_rate.data();

  jpl_reaction.clear();
  jpl_param.clear();
  for (const auto& j : k.jpl) {
    jpl_reaction.push_back(j.reaction_index);
    const double p[7] = {j.k0_A, j.k0_B, j.k0_C, j.kinf_A, j.kinf_B, j.kinf_C, j.Fc};
    jpl_param.insert(jpl_param.end(), p, p + 7);
  }
  rjpl_reaction.clear();
  rjpl_param.clear();
  for (const auto& j : k.r_jpl_arrhenius) {
    rjpl_reaction.push_back(j.reaction_index);
    const double p[10] = {j.k0_A, j.k0_B, j.k0_C, j.kinf_A, j.kinf_B, j.kinf_C, j.Fc, j.A, j.B, j.C};
    rjpl_param.insert(rjpl_param.end(), p, p + 10);
  }
  adjust_pair.clear();
  for (const auto& a : k.adjust_reaction) {
    adjust_pair.push_back(a.reaction_index);
    adjust_pair.push_back(a.species_index);
  }
  o1d_index.clear();
  o1d_param.clear();
  for (const auto& o : k.prod_O1D) {
    const int32_t idx[7] = {o.reaction_indices[0], o.reaction_indices[1], o.reaction_indices[2],
                            o.photolysis_reaction_index, o.species_index_1, o.species_index_2, o.species_index_3};
    o1d_index.insert(o1d_index.end(), idx, idx + 7);
    const double p[6] = {o.A1, o.C1, o.A2, o.C2, o.A3, o.C3};
    o1d_param.insert(o1d_param.end(), p, p + 6);
  }
  e3sm_view.nJPL = static_cast<int32_t>(jpl_reaction.size());
  e3sm_view.jpl_reaction = jpl_reaction.data();
  e3sm_view.jpl_param = jpl_param.data();
  e3sm_view.nRJPL = static_cast<int32_t>(rjpl_reaction.size());
  e3sm_view.rjpl_reaction = rjpl_reaction.data();
  e3sm_view.rjpl_param = rjpl_param.data();
  e3sm_view.nAdjust = static_cast<int32_t>(k.adjust_reaction.size());
  e3sm_view.adjust_pair = adjust_pair.data();
  e3sm_view.nProdO1D = static_cast<int32_t>(k.prod_O1D.size());
  e3sm_view.o1d_index = o1d_index.data();
  e3sm_view.o1d_param = o1d_param.data();
}

tchem_gb_mech::~tchem_gb_mech() {
  for (auto* t : device_tables)
    if (t) tchem_gb::destroy_device_tables(t);
}

extern "C" {

const char* tchem_gb_last_error(void) { return tchem_gb::g_last_error.c_str(); }

int tchem_gb_abi_version(void) { return TCHEM_GB_ABI_VERSION; }

int tchem_gb_mech_create_from_file(const char* yaml_path, const char* echo_path, tchem_gb_mech** out) {
  if (!yaml_path || !out) {
    set_last_error("tchem_gb_mech_create_from_file: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *out = nullptr;
  try {
    std::unique_ptr<tchem_gb_mech> m(new tchem_gb_mech());
    if (echo_path) {
      std::ofstream echo(echo_path);
      if (!echo) throw std::runtime_error(std::string("cannot open echo file ") + echo_path);
      m->km = tchem_gb::KineticModel::fromYamlFile(yaml_path, &echo);
    } else {
      m->km = tchem_gb::KineticModel::fromYamlFile(yaml_path, nullptr);
    }
    m->build_view();
    *out = m.release();
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

int tchem_gb_mech_create_from_string(const char* yaml_text, tchem_gb_mech** out) {
  if (!yaml_text || !out) {
    set_last_error("tchem_gb_mech_create_from_string: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *out = nullptr;
  try {
    std::unique_ptr<tchem_gb_mech> m(new tchem_gb_mech());
    m->km = tchem_gb::KineticModel::fromYamlString(yaml_text, nullptr);
    m->build_view();
    *out = m.release();
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

void tchem_gb_mech_destroy(tchem_gb_mech* mech) { delete mech; }

int tchem_gb_mech_host_view(const tchem_gb_mech* mech, tchem_gb_kmcd_view* view) {
  if (!mech || !view) {
    set_last_error("tchem_gb_mech_host_view: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *view = mech->view;
  return TCHEM_GB_OK;
}

int tchem_gb_mech_e3sm_view(const tchem_gb_mech* mech, tchem_gb_e3sm_view* view) {
  if (!mech || !view) {
    set_last_error("tchem_gb_mech_e3sm_view: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *view = mech->e3sm_view;
  return TCHEM_GB_OK;
}

int tchem_gb_mech_species_name(const tchem_gb_mech* mech, int i, char* buf, int buflen) {
  if (!mech || !buf || buflen <= 0 || i < 0 || i >= mech->km.nSpec) {
    set_last_error("tchem_gb_mech_species_name: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  std::strncpy(buf, mech->km.speciesNames[i].c_str(), static_cast<size_t>(buflen) - 1);
  buf[buflen - 1] = '\0';
  return TCHEM_GB_OK;
}

int tchem_gb_mech_sparse_lu(const tchem_gb_mech* mech, int32_t* info, int32_t* prog, int prog_cap) {
  if (!mech || !info || prog_cap < 0) {
    set_last_error("tchem_gb_mech_sparse_lu: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  auto* mm = const_cast<tchem_gb_mech*>(mech);
  {
    std::lock_guard<std::mutex> lk(mm->mu);
    try {
      if (!mm->host_tables) mm->host_tables.reset(new tchem_gb::HostTables(tchem_gb::build_host_tables(mm->km)));
    } catch (const std::exception& e) {
      set_last_error(e.what());
      return TCHEM_GB_ERR_ARG;
    }
  }
  const tchem_gb::SparseLuHost& h = mm->host_tables->slu;
  if (h.lay.m == 0) {
    set_last_error("tchem_gb_mech_sparse_lu: no sparse LU program for this mechanism (more than 128 active species)");
    return TCHEM_GB_ERR_UNSUPPORTED;
  }
  const tchem_gb::SparseLuLayout& L = h.lay;
  const int32_t v[12] = {L.m, L.nnz, L.n_ops, L.prog_len, L.off_diag, L.off_pos,
                         L.off_lc_ptr, L.off_lc, L.off_uc_ptr, L.off_uc, L.off_up_ptr, L.off_up};
  std::memcpy(info, v, sizeof(v));
  if (prog) std::memcpy(prog, h.prog.data(), sizeof(int32_t) * std::min<size_t>(prog_cap, h.prog.size()));
  return TCHEM_GB_OK;
}

int tchem_gb_scenario_batch_size(const char* yaml_path, int* nbatch) {
  if (!yaml_path || !nbatch) {
    set_last_error("tchem_gb_scenario_batch_size: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    // The batch size is the length of environmental_conditions.pressure.initial_value.
    tchem_gb::KineticModel dummy;
    dummy.nSpec = 0;
    std::vector<double> state;
    tchem_gb::setScenarioConditions(yaml_path, dummy, state, *nbatch);
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

int tchem_gb_scenario_read(const char* yaml_path, const tchem_gb_mech* mech, double* state_host, int nbatch) {
  if (!yaml_path || !mech || !state_host) {
    set_last_error("tchem_gb_scenario_read: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    std::vector<double> state;
    int nb = 0;
    tchem_gb::setScenarioConditions(yaml_path, mech->km, state, nb);
    if (nb != nbatch) {
      set_last_error("tchem_gb_scenario_read: scenario holds " + std::to_string(nb) + " samples, caller passed " +
                     std::to_string(nbatch));
      return TCHEM_GB_ERR_ARG;
    }
    std::memcpy(state_host, state.data(), state.size() * sizeof(double));
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

int tchem_gb_scenario_photolysis_rates(const char* yaml_path, int nbatch, double* photo_host, int* n_photo) {
  if (!yaml_path || !n_photo || nbatch < 0) {
    set_last_error("tchem_gb_scenario_photolysis_rates: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    std::vector<double> photo;
    tchem_gb::setScenarioPhotolysisRates(yaml_path, nbatch, photo, *n_photo);
    if (photo_host && !photo.empty()) std::memcpy(photo_host, photo.data(), photo.size() * sizeof(double));
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

int tchem_gb_scenario_external_forcing(const char* yaml_path, const tchem_gb_mech* mech, int nbatch,
                                       double* ext_host, int* count) {
  if (!yaml_path || !mech || !ext_host || nbatch < 0) {
    set_last_error("tchem_gb_scenario_external_forcing: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    std::vector<double> ext;
    int c = 0;
    tchem_gb::setScenarioExternalForcing(yaml_path, mech->km, nbatch, ext, c);
    if (!ext.empty()) std::memcpy(ext_host, ext.data(), ext.size() * sizeof(double));
    if (count) *count = c;
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

namespace {

// yaml-cpp's Node::as<T>(fallback): the fallback when the key is absent or does not convert.
double num_or(const tchem_gb::yaml::Node* n, const char* key, double fallback) {
  const tchem_gb::yaml::Node* v = n ? n->get(key) : nullptr;
  if (!v || !v->is_scalar()) return fallback;
  try {
    size_t used = 0;
    const double x = std::stod(v->scalar, &used);
    return used == v->scalar.size() ? x : fallback;
  } catch (...) {
    return fallback;
  }
}

int32_t int_or(const tchem_gb::yaml::Node* n, const char* key, int32_t fallback) {
  const tchem_gb::yaml::Node* v = n ? n->get(key) : nullptr;
  if (!v || !v->is_scalar()) return fallback;
  try {
    size_t used = 0;
    const long x = std::stol(v->scalar, &used);
    return used == v->scalar.size() ? static_cast<int32_t>(x) : fallback;
  } catch (...) {
    return fallback;
  }
}

int32_t bool_or(const tchem_gb::yaml::Node* n, const char* key, int32_t fallback) {
  const tchem_gb::yaml::Node* v = n ? n->get(key) : nullptr;
  if (!v || !v->is_scalar()) return fallback;
  std::string s = v->scalar;
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  if (s == "true" || s == "yes" || s == "y" || s == "on") return 1;
  if (s == "false" || s == "no" || s == "n" || s == "off") return 0;
  return fallback;
}

}  // namespace

int tchem_gb_numerics_read(const char* yaml_path, tchem_gb_numerics* out) {
  if (!yaml_path || !out) {
    set_last_error("tchem_gb_numerics_read: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    const tchem_gb::yaml::NodePtr root = tchem_gb::yaml::parse_file(yaml_path);
    const tchem_gb::yaml::Node* si = root ? root->get("solver_info") : nullptr;
    tchem_gb_numerics n{};
    n.atol_newton = num_or(si, "atol_newton", 1e-10);
    n.rtol_newton = num_or(si, "rtol_newton", 1e-6);
    n.dtmin = num_or(si, "dtmin", 1e-8);
    n.atol_time = num_or(si, "atol_time", 1e-12);
    n.rtol_time = num_or(si, "rtol_time", 1e-4);
    n.max_newton_iterations = int_or(si, "max_newton_iterations", 100);
    n.max_num_time_iterations = int_or(si, "max_num_time_iterations", 1000);
    n.team_size = int_or(si, "team_size", -1);
    n.vector_size = int_or(si, "vector_size", -1);
    n.verbose = bool_or(si, "verbose", 0);
    *out = n;
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(std::string("tchem_gb_numerics_read: ") + e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

}  // extern "C"
