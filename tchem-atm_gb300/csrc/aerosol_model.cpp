// Aerosol model parser and particle scenario reader (layout and rules in aerosol_model.hpp).
#include "aerosol_model.hpp"

#include <cstdio>
#include <map>
#include <stdexcept>

#include "yaml_lite.hpp"

namespace tchem_gb {

namespace {

using yaml::Node;

const Node* need(const Node* n, const char* key, const std::string& ctx) {
  const Node* c = n ? n->get(key) : nullptr;
  if (!c) throw std::runtime_error(std::string("aerosol model: missing '") + key + "' in " + ctx);
  return c;
}

AerosolModel build(const Node& root, const KineticModel& gas) {
  AerosolModel am;
  am.nSpec_gas = gas.nActive();
  am.nConstSpec_gas = gas.nConstSpec;
  const Node* items = root.get("NCAR-version");
  if (!items || !items->is_seq()) throw std::runtime_error("we do not have a parser for this file.");

  std::map<std::string, const Node*> gas_info;  // CHEM_SPEC items without a phase
  for (const auto& item : items->seq) {
    const Node* type = item->get("type");
    if (!type) continue;
    const std::string t = type->as_string();
    if (t == "CHEM_SPEC") {
      const std::string name = need(item.get(), "name", "CHEM_SPEC")->as_string();
      if (const Node* phase = item->get("phase")) {
        if (phase->as_string() == "AEROSOL") {
          if (am.speciesIndex(name) < 0) am.speciesNames.push_back(name);
          else throw std::runtime_error("aerosol model: duplicate aerosol species " + name);
          am.molecular_weights.push_back(need(item.get(), "molecular weight [kg mol-1]", name)->as_double());
          am.aerosol_density.push_back(need(item.get(), "density [kg m-3]", name)->as_double());
          am.aerosol_kappa.push_back(need(item.get(), "kappa", name)->as_double());
        }
      } else {
        gas_info.emplace(name, item.get());  // the first entry of a name is kept
      }
    } else if (t == "AERO_REP_SINGLE_PARTICLE") {
      am.nParticles = static_cast<int>(need(item.get(), "maximum computational particles", t)->as_int());
    }
  }
  am.nSpec = static_cast<int>(am.speciesNames.size());

  for (const auto& item : items->seq) {
    const Node* type = item->get("type");
    if (!type || type->as_string() != "MECHANISM") continue;
    const Node* reactions = item->get("reactions");
    if (!reactions) continue;
    for (const auto& r : reactions->seq) {
      const std::string rt = need(r.get(), "type", "reaction")->as_string();
      if (rt != "SIMPOL_PHASE_TRANSFER") {
        std::fprintf(stderr, "Warning : TChem (amd) did not parse this reaction type %s \n", rt.c_str());
        continue;
      }
      SimpolParam s{};
      const Node* B = need(r.get(), "B", rt);
      if (B->size() < 4) throw std::runtime_error("aerosol model: SIMPOL_PHASE_TRANSFER needs four B values");
      s.B1 = B->seq[0]->as_double();
      s.B2 = B->seq[1]->as_double();
      s.B3 = B->seq[2]->as_double();
      s.B4 = B->seq[3]->as_double();
      const std::string aero = need(r.get(), "aerosol-phase species", rt)->as_string();
      const int ai = am.speciesIndex(aero);
      if (ai < 0) throw std::runtime_error("species does not exit " + aero + " in reactants of SIMPOL_PHASE_TRANSFER");
      s.aerosol_sp_index = ai + am.nSpec_gas;
      const std::string gname = need(r.get(), "gas-phase species", rt)->as_string();
      const int gi = gas.speciesIndex(gname);
      if (gi < 0) throw std::runtime_error("species does not exit " + gname + " in reactants of SIMPOL_PHASE_TRANSFER");
      s.gas_sp_index = gi;
      auto it = gas_info.find(gname);
      if (it == gas_info.end())
        throw std::runtime_error("aerosol model: gas species " + gname + " has no CHEM_SPEC entry with its SIMPOL inputs");
      s.diffusion_coeff = need(it->second, "diffusion coeff [m2 s-1]", gname)->as_double();
      if (const Node* ns = it->second->get("N star")) {
        s.N_star = ns->as_double();
        s.compute_alpha = true;
      } else {
        s.N_star = 999;
        s.compute_alpha = false;
      }
      s.molecular_weight = need(it->second, "molecular weight [kg mol-1]", gname)->as_double();
      am.simpol.push_back(s);
    }
  }
  return am;
}

}  // namespace

int AerosolModel::speciesIndex(const std::string& name) const {
  for (size_t i = 0; i < speciesNames.size(); ++i)
    if (speciesNames[i] == name) return static_cast<int>(i);
  return -1;
}

AerosolModel AerosolModel::fromYamlFile(const std::string& path, const KineticModel& gas) {
  yaml::NodePtr root = yaml::parse_file(path);
  return build(*root, gas);
}

AerosolModel AerosolModel::fromYamlString(const std::string& text, const KineticModel& gas) {
  yaml::NodePtr root = yaml::parse_string(text);
  return build(*root, gas);
}

bool setScenarioParticles(const std::string& path, const AerosolModel& am, int nBatch, std::vector<double>& num_conc,
                          double* state, int dim) {
  yaml::NodePtr root = yaml::parse_file(path);
  const Node* particles = root->get("particles");
  if (!particles) return false;
  if (am.nParticles < 1) throw std::runtime_error("aerosol model: the number of particles is not set");
  const Node* nc = need(need(particles, "num_concentration", "particles"), "initial_value", "num_concentration");
  if (static_cast<int>(nc->size()) < nBatch)
    throw std::runtime_error("particles: num_concentration has fewer values than samples");
  num_conc.assign(static_cast<size_t>(nBatch) * am.nParticles, 0.0);
  for (int b = 0; b < nBatch; ++b)
    for (int i = 0; i < am.nParticles; ++i) num_conc[static_cast<size_t>(b) * am.nParticles + i] = nc->seq[b]->as_double();
  const int first = 3 + am.nSpec_gas + am.nConstSpec_gas;
  if (first + am.nSpec * am.nParticles > dim) throw std::runtime_error("particles: state rows too short");
  if (const Node* init = particles->get("initial_state")) {
    for (const auto& kv : init->map) {
      const int k = am.speciesIndex(kv.first);
      if (k < 0) throw std::runtime_error("species does not exit " + kv.first + " in the aerosol model");
      const Node* vals = need(kv.second.get(), "initial_value", kv.first);
      if (static_cast<int>(vals->size()) < nBatch)
        throw std::runtime_error("particles: " + kv.first + " has fewer values than samples");
      for (int b = 0; b < nBatch; ++b)
        for (int i = 0; i < am.nParticles; ++i)
          state[static_cast<size_t>(b) * dim + first + am.nSpec * i + k] =
              vals->seq[b]->as_double() / num_conc[static_cast<size_t>(b) * am.nParticles + i];
    }
  }
  return true;
}

}  // namespace tchem_gb
