// C ABI: aerosol model (SIMPOL.1 phase transfer) entry points (host only).
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "aero_host.hpp"
#include "aerosol_model.hpp"
#include "mech_host.hpp"

void tchem_gb_aero::build_view() {
  simpol_index.clear();
  simpol_param.clear();
  for (const auto& s : am.simpol) {
    const int32_t idx[3] = {s.aerosol_sp_index, s.gas_sp_index, s.compute_alpha ? 1 : 0};
    simpol_index.insert(simpol_index.end(), idx, idx + 3);
    const double par[7] = {s.B1, s.B2, s.B3, s.B4, s.diffusion_coeff, s.N_star, s.molecular_weight};
    simpol_param.insert(simpol_param.end(), par, par + 7);
  }
  view.nSpec = am.nSpec;
  view.nSpec_gas = am.nSpec_gas;
  view.nConstSpec_gas = am.nConstSpec_gas;
  view.nParticles = am.nParticles;
  view.nSimpol = static_cast<int32_t>(am.simpol.size());
  view.molecular_weights = am.molecular_weights.data();
  view.aerosol_density = am.aerosol_density.data();
  view.aerosol_kappa = am.aerosol_kappa.data();
  view.simpol_index = simpol_index.data();
  view.simpol_param = simpol_param.data();
}

tchem_gb_aero::~tchem_gb_aero() {
  for (auto* t : device_tables)
    if (t) tchem_gb::destroy_aero_device_tables(t);
}

using tchem_gb::set_last_error;

namespace {

template <typename F>
int create(const char* src, const tchem_gb_mech* gas, tchem_gb_aero** out, const char* who, F parse) {
  if (!src || !gas || !out) {
    set_last_error(std::string(who) + ": null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *out = nullptr;
  try {
    std::unique_ptr<tchem_gb_aero> a(new tchem_gb_aero());
    a->am = parse(src, gas->km);
    a->build_view();
    *out = a.release();
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

}  // namespace

extern "C" {

int tchem_gb_aero_create_from_file(const char* yaml_path, const tchem_gb_mech* gas, tchem_gb_aero** out) {
  return create(yaml_path, gas, out, "tchem_gb_aero_create_from_file",
                [](const char* p, const tchem_gb::KineticModel& km) { return tchem_gb::AerosolModel::fromYamlFile(p, km); });
}

int tchem_gb_aero_create_from_string(const char* yaml_text, const tchem_gb_mech* gas, tchem_gb_aero** out) {
  return create(yaml_text, gas, out, "tchem_gb_aero_create_from_string", [](const char* t, const tchem_gb::KineticModel& km) {
    return tchem_gb::AerosolModel::fromYamlString(t, km);
  });
}

void tchem_gb_aero_destroy(tchem_gb_aero* aero) { delete aero; }

int tchem_gb_aero_host_view(const tchem_gb_aero* aero, tchem_gb_aero_view* view) {
  if (!aero || !view) {
    set_last_error("tchem_gb_aero_host_view: null argument");
    return TCHEM_GB_ERR_ARG;
  }
  *view = aero->view;
  return TCHEM_GB_OK;
}

int tchem_gb_aero_set_number_of_particles(tchem_gb_aero* aero, int n_particles) {
  if (!aero || n_particles < 1) {
    set_last_error("tchem_gb_aero_set_number_of_particles: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  aero->am.nParticles = n_particles;
  aero->build_view();
  return TCHEM_GB_OK;
}

int tchem_gb_aero_species_name(const tchem_gb_aero* aero, int i, char* buf, int buflen) {
  if (!aero || !buf || buflen <= 0 || i < 0 || i >= aero->am.nSpec) {
    set_last_error("tchem_gb_aero_species_name: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  std::strncpy(buf, aero->am.speciesNames[i].c_str(), static_cast<size_t>(buflen) - 1);
  buf[buflen - 1] = '\0';
  return TCHEM_GB_OK;
}

int tchem_gb_aero_scenario_particles(const char* yaml_path, const tchem_gb_aero* aero, int nbatch, double* num_conc,
                                     double* state, int dim, int* found) {
  if (!yaml_path || !aero || nbatch < 0 || !num_conc || !state || !found) {
    set_last_error("tchem_gb_aero_scenario_particles: bad argument");
    return TCHEM_GB_ERR_ARG;
  }
  try {
    std::vector<double> nc;
    *found = tchem_gb::setScenarioParticles(yaml_path, aero->am, nbatch, nc, state, dim) ? 1 : 0;
    if (*found && !nc.empty()) std::memcpy(num_conc, nc.data(), nc.size() * sizeof(double));
    return TCHEM_GB_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TCHEM_GB_ERR_PARSE;
  }
}

}  // extern "C"
