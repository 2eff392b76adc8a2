// Host-side kinetic model builder; see kinetic_model.hpp for the rules restated here.
#include "kinetic_model.hpp"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <sstream>
#include <stdexcept>

#include "yaml_lite.hpp"

namespace tchem_gb {

namespace {

using yaml::Node;

// printf-style writer for the mechanism echo (the kmod.echo file format of
// src/core/TChem_KineticModelData.cpp:148-155, 287-299, 949-973).
void echo_printf(std::ostream* os, const char* fmt, ...) {
  if (!os) return;
  va_list args;
  va_start(args, fmt);
  const int len = std::vsnprintf(nullptr, 0, fmt, args);
  va_end(args);
  std::vector<char> buf(static_cast<size_t>(len) + 1);
  va_start(args, fmt);
  std::vsnprintf(buf.data(), buf.size(), fmt, args);
  va_end(args);
  (*os) << buf.data();
}

[[noreturn]] void model_error(const std::string& msg) {
  throw std::runtime_error("Yaml : Error when interpreting kinetic model  !!! " + msg);
}

const Node* req(const Node* n, const char* key, const std::string& ctx) {
  const Node* c = n ? n->get(key) : nullptr;
  if (!c) model_error(std::string("missing '") + key + "' in " + ctx);
  return c;
}

double opt_double(const Node* coef, const char* key, double dflt) {
  const Node* c = coef ? coef->get(key) : nullptr;
  return c ? c->as_double() : dflt;
}

bool time_unit_is_min(const Node& reaction) {
  const Node* tu = reaction.get("time_unit");
  return tu && tu->as_string() == "min";
}

std::string truncate_name(const std::string& s) {
  return s.size() > static_cast<size_t>(LENGTHOFSPECNAME) ? s.substr(0, LENGTHOFSPECNAME) : s;
}

KineticModel build(const Node& root, std::ostream* echo) {
  KineticModel km;
  if (!root.get("NCAR-version")) throw std::runtime_error("we do not have a parser for this file");

  const Node* species = root.get("species");
  const Node* reactions = root.get("reactions");
  const Node* const_species = root.get("constant_species");
  km.nConstSpec = const_species ? static_cast<int>(const_species->size()) : 0;
  km.nSpec = (species ? static_cast<int>(species->size()) : 0) + km.nConstSpec;
  km.nReac = reactions ? static_cast<int>(reactions->size()) : 0;

  // Species map: std::map::insert keeps the first index of a repeated name.
  std::map<std::string, int> species_indx;
  int sp_i = 0;
  auto add_species = [&](const Node& sp) {
    const std::string name = req(&sp, "name", "species entry")->as_string();
    species_indx.insert({name, sp_i});
    km.speciesNames.push_back(truncate_name(name));
    ++sp_i;
  };
  if (species)
    for (const auto& sp : species->seq) add_species(*sp);
  if (const_species)
    for (const auto& sp : const_species->seq) add_species(*sp);

  {
    auto it = species_indx.find("M");
    if (it == species_indx.end())
      model_error("M species does not exit; Note: Name of M species is hard-coded to M");
    km.M_index = it->second;
  }

  echo_printf(echo, "kmod.list : # of species                                      : %d\n", km.nSpec);
  echo_printf(echo, "kmod.list : # of species with constant concentration          : %d\n", km.nConstSpec);
  echo_printf(echo, "kmod.list : # of reactions                                    : %d\n", km.nReac);
  echo_printf(echo, "No. \t Species\n");
  for (int i = 0; i < km.nSpec; i++) echo_printf(echo, "%-3d\t%-32s\n", i + 1, km.speciesNames[i].c_str());
  echo_printf(echo, "-------------------------------------------------------------------------\n");

  const int R = km.nReac;
  km.isRev.assign(R, 1);
  km.reacNrp.assign(R, 0);
  km.reacNreac.assign(R, 0);
  km.reacNprod.assign(R, 0);
  km.convExponent.assign(R, 0);
  km.reacType.assign(R, 0);

  std::vector<std::map<int, double>> reactantsInfo(R), productsInfo(R);
  int countArrhenius = 0, countTroe = 0, countCMAQ = 0, countJPL = 0, countRJPL = 0, countAdjust = 0, countPhoto = 0;
  km.maxSpecInReac = 0;

  for (int r = 0; r < R; ++r) {
    const Node& reaction = *reactions->seq[r];
    const Node* reactants = reaction.get("reactants");
    if (!reactants) model_error("Reactions No " + std::to_string(r) + " does not have reactants");
    km.reacNreac[r] = static_cast<int>(reactants->size());
    for (const auto& kv : reactants->map) {
      auto it = species_indx.find(kv.first);
      if (it == species_indx.end())
        model_error("species does not exit " + kv.first + " in reactants of reaction No " + std::to_string(r));
      reactantsInfo[r].insert({it->second, kv.second->as_double()});
    }
    const Node* products = reaction.get("products");
    if (!products) model_error("Reactions No " + std::to_string(r) + " does not have products");
    km.reacNprod[r] = static_cast<int>(products->size());
    for (const auto& kv : products->map) {
      auto it = species_indx.find(kv.first);
      if (it != species_indx.end()) {
        productsInfo[r].insert({it->second, kv.second->as_double()});
      } else {
        // Only a warning in the reference: the product is dropped.
        std::fprintf(stderr, "Yaml : Warning when interpreting kinetic model  !!!species does not exit %s in products of reaction No %d\n",
                     kv.first.c_str(), r);
      }
    }
    km.reacNrp[r] = km.reacNreac[r] + km.reacNprod[r];
    km.maxSpecInReac = std::max(km.maxSpecInReac, std::max(km.reacNreac[r], km.reacNprod[r]));

    const std::string type = req(&reaction, "type", "reaction")->as_string();
    if (type == "ARRHENIUS") { ++countArrhenius; km.reacType[r] = KineticModel::ARRHENIUS; }
    else if (type == "TROE") { ++countTroe; km.reacType[r] = KineticModel::TROE; }
    else if (type == "CMAQ_H2O2") { ++countCMAQ; km.reacType[r] = KineticModel::CMAQ_H2O2; }
    else if (type == "JPL") { ++countJPL; km.reacType[r] = KineticModel::JPL; }
    else if (type == "R_JPL_ARRHENIUS") { ++countRJPL; km.reacType[r] = KineticModel::R_JPL_ARRHENIUS; }
    else if (type == "PHOTO_RATE") { ++countPhoto; km.reacType[r] = KineticModel::PHOTO_RATE; }
    else throw std::runtime_error("Error: reaction type does not exit; Reaction No: " + std::to_string(r) + " type " + type);
    if (const Node* adj = reaction.get("adjust_reaction")) countAdjust += static_cast<int>(adj->size());
  }
  km.maxSpecInReac *= 2;
  km.countPhotoRate = countPhoto;

  echo_printf(echo, "kmod.list : Max # of species in a reaction                    : %d\n", km.maxSpecInReac);
  echo_printf(echo, "kmod.list :  # of arrhenius type reactions                    : %d\n", countArrhenius);
  echo_printf(echo, "kmod.list :  # of CMAQ_H2O2 type reactions                    : %d\n", countCMAQ);
  echo_printf(echo, "kmod.list :  # of Troe type reactions                         : %d\n", countTroe);
  echo_printf(echo, "kmod.list :  # of JPL-Troe type reactions                     : %d\n", countJPL);
  echo_printf(echo, "kmod.list :  # of Ratio JPL arrhenius type reactions          : %d\n", countRJPL);
  echo_printf(echo, "kmod.list :  # of adjustment pairs                            : %d\n", countAdjust);
  echo_printf(echo, "kmod.list :  # of Photolysis rates                            : %d\n", countPhoto);

  // Stoichiometry tables. Slots a product count reserves for a dropped (unknown) product keep
  // species index 0 and coefficient 0, so they contribute nothing.
  const int S = km.maxSpecInReac;
  km.reacSidx.assign(static_cast<size_t>(R) * S, 0);
  km.reacNuki.assign(static_cast<size_t>(R) * S, 0.0);
  for (int r = 0; r < R; ++r) {
    int c = 0;
    for (const auto& kv : reactantsInfo[r]) {
      km.reacSidx[r * S + c] = kv.first;
      km.reacNuki[r * S + c] = -kv.second;
      ++c;
    }
    c = S / 2;
    for (const auto& kv : productsInfo[r]) {
      km.reacSidx[r * S + c] = kv.first;
      km.reacNuki[r * S + c] = kv.second;
      ++c;
    }
  }

  // Rate parameters, per type, in reaction order.
  for (int r = 0; r < R; ++r) {
    const Node& reaction = *reactions->seq[r];
    const Node* coef = reaction.get("coefficients");
    const bool per_min = time_unit_is_min(reaction);
    switch (km.reacType[r]) {
      case KineticModel::ARRHENIUS: {
        double A = 1.0;
        if (coef && coef->get("A")) {
          A = coef->get("A")->as_double();
          if (per_min) A /= 60.0;
        }
        const double D = opt_double(coef, "D", 300.0);
        const double B = opt_double(coef, "B", 0.0);
        double C = 0.0;
        if (coef && coef->get("Ea")) {
          C = -coef->get("Ea")->as_double() / KBOLT;
          if (coef->get("C")) throw std::runtime_error("Ea and C are presented in Yaml input file");
        } else if (coef && coef->get("C")) {
          C = coef->get("C")->as_double();
        }
        const double E = opt_double(coef, "E", 0.0);
        km.arrhenius.push_back({r, E, A, B, C, D});
        break;
      }
      case KineticModel::CMAQ_H2O2: {
        double k1_A = 1.0, k2_A = 1.0;
        if (coef && coef->get("k1_A")) { k1_A = coef->get("k1_A")->as_double(); if (per_min) k1_A /= 60.0; }
        if (coef && coef->get("k2_A")) { k2_A = coef->get("k2_A")->as_double(); if (per_min) k2_A /= 60.0; }
        CMAQ_H2O2Param p;
        p.reaction_index = r;
        p.A1 = k1_A;
        p.B1 = opt_double(coef, "k1_B", 0.0);
        p.C1 = opt_double(coef, "k1_C", 0.0);
        p.A2 = k2_A * 1e6;  // [M]*k2
        p.B2 = opt_double(coef, "k2_B", 0.0);
        p.C2 = opt_double(coef, "k2_C", 0.0);
        km.cmaq_h2o2.push_back(p);
        break;
      }
      case KineticModel::JPL:
      case KineticModel::R_JPL_ARRHENIUS: {
        double k0_A = 1.0, kinf_A = 1.0;
        if (coef && coef->get("k0_A")) { k0_A = coef->get("k0_A")->as_double(); if (per_min) k0_A /= 60.0; }
        if (coef && coef->get("kinf_A")) { kinf_A = coef->get("kinf_A")->as_double(); if (per_min) kinf_A /= 60.0; }
        const double k0_B = opt_double(coef, "k0_B", 0.0), k0_C = opt_double(coef, "k0_C", 0.0);
        const double kinf_B = opt_double(coef, "kinf_B", 0.0), kinf_C = opt_double(coef, "kinf_C", 0.0);
        const double Fc = opt_double(coef, "Fc", 0.6);
        if (km.reacType[r] == KineticModel::JPL) {
          km.jpl.push_back({r, k0_A, k0_B, kinf_A, kinf_B, Fc, k0_C, kinf_C});
        } else {
          double A = 1.0;
          if (coef && coef->get("A")) { A = coef->get("A")->as_double(); if (per_min) A /= 60.0; }
          km.r_jpl_arrhenius.push_back({r, k0_A, k0_B, kinf_A, kinf_B, Fc, k0_C, kinf_C, A,
                                        opt_double(coef, "B", 0.0), opt_double(coef, "C", 0.0)});
        }
        break;
      }
      case KineticModel::TROE: {
        double k0_A = 1.0, kinf_A = 1.0;
        if (coef && coef->get("k0_A")) { k0_A = coef->get("k0_A")->as_double(); if (per_min) k0_A /= 60.0; }
        if (coef && coef->get("kinf_A")) { kinf_A = coef->get("kinf_A")->as_double(); if (per_min) kinf_A /= 60.0; }
        km.reacPfal.push_back(r);
        // From CAMP: [M] is included in k0_A (k0_A * 1e6).
        const double par[8] = {k0_A * 1e6,
                               opt_double(coef, "k0_B", 0.0),
                               opt_double(coef, "k0_C", 0.0),
                               kinf_A,
                               opt_double(coef, "kinf_B", 0.0),
                               opt_double(coef, "kinf_C", 0.0),
                               opt_double(coef, "Fc", 0.6),
                               opt_double(coef, "N", 1.0)};
        km.reacPpar.insert(km.reacPpar.end(), par, par + 8);
        break;
      }
      default:
        break;  // PHOTO_RATE carries no coefficients
    }
    if (const Node* adj = reaction.get("adjust_reaction")) {
      for (const auto& a : adj->seq) {
        const std::string name = a->as_string();
        auto it = species_indx.find(name);
        if (it == species_indx.end())
          model_error("species does not exit " + name + " in adjust_reaction for reaction No " + std::to_string(r));
        km.adjust_reaction.push_back({r, it->second});
      }
    }
  }

  if (const Node* mod = root.get("modifier_prod_O1D")) {
    const Node* coef = mod->get("coefficients");
    ProdO1DParam p{};
    p.A1 = opt_double(coef, "A1", 1.0); p.C1 = opt_double(coef, "C1", 0.0);
    p.A2 = opt_double(coef, "A2", 1.0); p.C2 = opt_double(coef, "C2", 0.0);
    p.A3 = opt_double(coef, "A3", 1.0); p.C3 = opt_double(coef, "C3", 0.0);
    auto find_sp = [&](const char* key) {
      const std::string name = req(mod, key, "modifier_prod_O1D")->as_string();
      auto it = species_indx.find(name);
      if (it == species_indx.end()) model_error("species does not exit " + name + " in modifier_prod_O1D");
      return it->second;
    };
    p.species_index_1 = find_sp("species_name_1");
    p.species_index_2 = find_sp("species_name_2");
    p.species_index_3 = find_sp("species_name_3");
    p.photolysis_reaction_index = static_cast<int>(req(mod, "photolysis_reaction_index", "modifier_prod_O1D")->as_int());
    int c = 0;
    if (const Node* lst = mod->get("reaction_list"))
      for (const auto& e : lst->seq) { if (c < 3) p.reaction_indices[c] = static_cast<int>(e->as_int()); ++c; }
    km.prod_O1D.push_back(p);
  }

  if (const Node* sources = root.get("sources")) {
    for (const auto& src : sources->seq) {
      const std::string type = req(src.get(), "type", "source")->as_string();
      if (type != "EMISSION")
        throw std::runtime_error("Error: source type does not exit; type " + type);
      const Node* coef = src->get("coefficients");
      const Node* rate = coef ? coef->get("emission_rate") : nullptr;
      if (!rate) throw std::runtime_error("Error EMISSION, emission_rate is not provided");
      const Node* sp = src->get("species");
      if (!sp) throw std::runtime_error("Error EMISSION, species name  is not provided");
      auto it = species_indx.find(sp->as_string());
      if (it == species_indx.end()) model_error("species does not exit " + sp->as_string());
      km.emission.push_back({it->second, rate->as_double()});
    }
  }

  for (int r = 0; r < R; ++r) {
    int nu_sum = 0;
    for (int j = 0; j < km.reacNreac[r]; ++j) nu_sum += std::abs(static_cast<int>(km.nuki(r, j)));
    km.convExponent[r] = nu_sum - 1;
  }

  echo_printf(echo, "kmod.list :  # sources e.g., EMISSION                         : %d\n",
              static_cast<int>(km.emission.size()));
  echo_printf(echo, "Reaction data : species and Arrhenius pars\n");
  for (int r = 0; r < R; ++r) {
    echo_printf(echo, "%-5d\t%1d\t%2d\t%2d | ", r + 1, km.isRev[r], km.reacNreac[r], km.reacNprod[r]);
    for (int j = 0; j < km.reacNreac[r]; j++)
      echo_printf(echo, "%f*%s | ", km.nuki(r, j), km.speciesNames[km.sidx(r, j)].c_str());
    const int joff = S / 2;
    for (int j = 0; j < km.reacNprod[r]; j++)
      echo_printf(echo, "%f*%s | ", km.nuki(r, j + joff), km.speciesNames[km.sidx(r, j + joff)].c_str());
    echo_printf(echo, "\n");
  }
  return km;
}

}  // namespace

int KineticModel::speciesIndex(const std::string& name) const {
  for (int i = 0; i < nSpec; ++i)
    if (std::strncmp(speciesNames[i].c_str(), name.c_str(), LENGTHOFSPECNAME) == 0) return i;
  return -1;
}

KineticModel KineticModel::fromYamlFile(const std::string& path, std::ostream* echo) {
  yaml::NodePtr root = yaml::parse_file(path);
  return build(*root, echo);
}

KineticModel KineticModel::fromYamlString(const std::string& text, std::ostream* echo) {
  yaml::NodePtr root = yaml::parse_string(text);
  return build(*root, echo);
}

void setScenarioConditions(const std::string& path, const KineticModel& km, std::vector<double>& state, int& nBatch) {
  yaml::NodePtr root = yaml::parse_file(path);
  const Node* env = req(root.get(), "environmental_conditions", "scenario");
  const Node* pressure = req(req(env, "pressure", "environmental_conditions"), "initial_value", "pressure");
  const Node* temperature = req(req(env, "temperature", "environmental_conditions"), "initial_value", "temperature");
  const Node* initial_state = req(root.get(), "initial_state", "scenario");
  nBatch = static_cast<int>(pressure->size());
  if (static_cast<int>(temperature->size()) != nBatch)
    throw std::runtime_error("scenario: temperature and pressure lists differ in length");
  const int dim = km.nSpec + 3;
  state.assign(static_cast<size_t>(nBatch) * dim, 0.0);
  // Species without an entry in the model are skipped (the reference's index search finds no match).
  for (int i = 0; i < nBatch; ++i) {
    const double p = pressure->seq[i]->as_double();
    const double T = temperature->seq[i]->as_double();
    state[static_cast<size_t>(i) * dim + 1] = p;
    state[static_cast<size_t>(i) * dim + 2] = T;
  }
  for (const auto& kv : initial_state->map) {
    const int idx = km.speciesIndex(kv.first);
    if (idx < 0) continue;
    const std::string units = req(kv.second.get(), "units", "initial_state")->as_string();
    const Node* vals = req(kv.second.get(), "initial_value", "initial_state");
    for (int i = 0; i < nBatch; ++i) {
      const double p = pressure->seq[i]->as_double();
      const double T = temperature->seq[i]->as_double();
      const double v = vals->seq.at(static_cast<size_t>(i))->as_double();
      double x;
      if (units == "molecules m-3") {
        const double conv = CONV_PPM * p / T;
        x = v / conv;
      } else if (units == "molecules cm-3") {
        const double conv = CONV_PPM * p / T;
        x = v / conv / 1e6;
      } else if (units == "mol m-3") {
        x = v;
      } else {
        throw std::runtime_error("unit type does not exit " + units);
      }
      state[static_cast<size_t>(i) * dim + 3 + idx] = x;
    }
  }
}

void setScenarioPhotolysisRates(const std::string& path, int nBatch, std::vector<double>& photo, int& nPhoto) {
  yaml::NodePtr root = yaml::parse_file(path);
  nPhoto = 0;
  photo.clear();
  const Node* rates = root->get("photolysis_rates");
  if (!rates) return;
  nPhoto = static_cast<int>(rates->size());
  photo.assign(static_cast<size_t>(nBatch) * nPhoto, 0.0);
  for (int r = 0; r < nPhoto; ++r) {
    const std::string key = "r_" + std::to_string(r);
    const Node* entry = rates->get(key);
    const Node* vals = entry ? entry->get("value") : nullptr;
    if (!vals || static_cast<int>(vals->size()) != nBatch)
      throw std::runtime_error("Error number of values in photo reaction is different than number of conditions (" +
                               key + ")");
    for (int b = 0; b < nBatch; ++b) photo[static_cast<size_t>(b) * nPhoto + r] = vals->seq[b]->as_double();
  }
}

void setScenarioExternalForcing(const std::string& path, const KineticModel& km, int nBatch, std::vector<double>& ext,
                                int& count) {
  yaml::NodePtr root = yaml::parse_file(path);
  const int m = km.nActive();
  ext.assign(static_cast<size_t>(nBatch) * m, 0.0);
  count = 0;
  const Node* forcing = root->get("external_forcing");
  if (!forcing) return;
  if (m == 0 || nBatch == 0) throw std::runtime_error("Number of active species and bacthes is zero.");
  for (const auto& kv : forcing->map) {
    const std::string name = req(kv.second.get(), "species_name", "external_forcing")->as_string();
    int idx = -1;  // active species only, first match on the stored (truncated) names
    for (int i = 0; i < m; ++i)
      if (std::strncmp(km.speciesNames[i].c_str(), name.c_str(), LENGTHOFSPECNAME) == 0) {
        idx = i;
        break;
      }
    if (idx < 0) throw std::runtime_error("species " + name + " does not exits in tchem species lists.");
    const Node* vals = kv.second->get("value");
    if (!vals || static_cast<int>(vals->size()) != nBatch)
      throw std::runtime_error("Error number of values in external forcing is different than number of conditions");
    for (int b = 0; b < nBatch; ++b) ext[static_cast<size_t>(b) * m + idx] = vals->seq[b]->as_double();
    ++count;
  }
}

}  // namespace tchem_gb
