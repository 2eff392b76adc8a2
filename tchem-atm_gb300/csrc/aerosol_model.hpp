// Host-side aerosol model: NCAR/CAMP-format aerosol YAML -> aerosol species and SIMPOL.1
// gas-particle phase-transfer tables.
//
// Restates the semantics of TChem::AerosolModelData (src/core/TChem_AerosolModelData.hpp:30-80,
// src/core/TChem_AerosolModelData.cpp:60-303):
//  - the file's NCAR-version entry is a list of typed items; CHEM_SPEC items with
//    phase: AEROSOL are the aerosol species, in file order (molecular weight [kg mol-1],
//    density [kg m-3], kappa); CHEM_SPEC items without a phase carry the gas species'
//    SIMPOL inputs (diffusion coeff [m2 s-1], molecular weight [kg mol-1], optional N star);
//  - AERO_REP_SINGLE_PARTICLE gives the number of particles (maximum computational particles);
//  - MECHANISM items list SIMPOL_PHASE_TRANSFER reactions (B[0..3], aerosol-phase species,
//    gas-phase species), in file order; other reaction types are skipped with a warning;
//  - the ODE vector of the aerosol problem is [active gas species, particle 0's aerosol
//    species, particle 1's, ...]: a SIMPOL entry's aerosol index is the aerosol species index
//    plus the number of active gas species; its gas index is the gas species index;
//  - a gas species without "N star" uses alpha = 0.1 (compute_alpha false, N_star = 999).
#pragma once

#include <string>
#include <vector>

#include "kinetic_model.hpp"

namespace tchem_gb {

struct SimpolParam {  // src/core/TChem_ReactionTypes.hpp:30-44
  int aerosol_sp_index;  // in the ODE vector of particle 0 (add i_part * nSpec for particle i_part)
  double B1, B2, B3, B4;
  int gas_sp_index;
  double diffusion_coeff;
  double N_star;
  bool compute_alpha;
  double molecular_weight;  // of the gas species
};

struct AerosolModel {
  int nSpec = 0;            // aerosol species per particle
  int nSpec_gas = 0;        // active gas species
  int nConstSpec_gas = 0;   // constant gas species
  int nParticles = -1;      // computational particles (-1: not given)
  std::vector<std::string> speciesNames;  // aerosol species in file order
  std::vector<double> molecular_weights, aerosol_density, aerosol_kappa;
  std::vector<SimpolParam> simpol;

  int nOde() const { return nSpec_gas + nSpec * nParticles; }
  int speciesIndex(const std::string& name) const;  // aerosol species, -1 if absent

  static AerosolModel fromYamlFile(const std::string& path, const KineticModel& gas);
  static AerosolModel fromYamlString(const std::string& text, const KineticModel& gas);
};

// Particle scenario reader (src/core/TChem_AerosolModelData.cpp:256-300): from the file's
// particles section, num_conc[nBatch][nParticles] (every particle of sample b gets
// num_concentration.initial_value[b]) and, in state rows of width dim, the aerosol species of
// particle i at 3 + nSpec_gas + nConstSpec_gas + nSpec * i + k = initial_value[b] / num_conc.
// Returns false when the file has no particles section.
bool setScenarioParticles(const std::string& path, const AerosolModel& am, int nBatch, std::vector<double>& num_conc,
                          double* state, int dim);

}  // namespace tchem_gb
