// Host-side kinetic model: NCAR-format YAML -> stoichiometry and rate-parameter tables.
//
// Restates the semantics of TChem::KineticModelData::initChemNCAR
// (src/core/TChem_KineticModelData.cpp:80-1017) and the const-data bundle
// TChem::KineticModelNCAR_ConstData (src/core/TChem_KineticModelNCAR_ConstData.hpp:30-113):
//  - species order is the `species` list followed by `constant_species` (appended last);
//  - a species named M must exist;
//  - reactants/products are keyed by species index (sorted, duplicate names merge);
//    reactant nu is stored negative in slots [0, nreac), product nu positive in slots
//    [maxSpecInReac/2, ...), with maxSpecInReac = 2 * max over reactions of max(nreac, nprod);
//  - unknown product names only warn and are dropped;
//  - ARRHENIUS: A, B, C (or Ea -> C = -Ea/KBOLT), D = 300, E defaults; time_unit: min divides A by 60;
//  - TROE: k0_A is multiplied by 1e6, Fc defaults to 0.6, N to 1;
//  - CMAQ_H2O2: k2_A is multiplied by 1e6;
//  - convExponent = sum over reactant |nu| - 1.
// Error handling follows TCHEM_CHECK_ERROR (src/core/TChem_Util.hpp:108-114): the reference
// prints and exits; here a std::runtime_error with the same message is thrown.
#pragma once

#include <array>
#include <ostream>
#include <string>
#include <vector>

namespace tchem_gb {

// Conversion prefactor molecules cm^-3 per ppm at p/T = 1 (src/core/TChem_Util.hpp:183).
constexpr double CONV_PPM = 7.24296358205307e+10;
// Boltzmann's constant [J/K] (src/core/TChem_Util.hpp:195).
constexpr double KBOLT = 1.3806504e-23;
// Species names are stored truncated to this length (src/core/TChem_Util.hpp:133).
constexpr int LENGTHOFSPECNAME = 18;

struct ArrheniusParam {  // src/core/TChem_Util.hpp:367-374
  int reaction_index;
  double E, A, B, C, D;
};

struct CMAQ_H2O2Param {  // src/core/TChem_Util.hpp:378-387
  int reaction_index;
  double A1, B1, C1, A2, B2, C2;
};

struct JPLParam {  // src/core/TChem_Util.hpp:391-400
  int reaction_index;
  double k0_A, k0_B, kinf_A, kinf_B, Fc, k0_C, kinf_C;
};

struct RJPLArrheniusParam {  // src/core/TChem_Util.hpp:404-419
  int reaction_index;
  double k0_A, k0_B, kinf_A, kinf_B, Fc, k0_C, kinf_C;
  double A, B, C;
};

struct EmissionParam {  // src/core/TChem_Util.hpp:423-426
  int species_index;
  double emission_rate;
};

struct AdjustReactionParam {  // src/core/TChem_Util.hpp:430-433
  int reaction_index;
  int species_index;
};

struct ProdO1DParam {  // src/core/TChem_Util.hpp:442-459
  int reaction_indices[3];
  int photolysis_reaction_index;
  int species_index_1, species_index_2, species_index_3;
  double A1, C1, A2, C2, A3, C3;
};

struct KineticModel {
  int nSpec = 0;       // all species, constant species included (appended last)
  int nConstSpec = 0;  // constant (tracer) species
  int nReac = 0;
  int maxSpecInReac = 0;
  int M_index = -1;
  double CONV_PPM_ = CONV_PPM;

  std::vector<std::string> speciesNames;  // truncated to LENGTHOFSPECNAME characters
  std::vector<int> isRev, reacNrp, reacNreac, reacNprod, convExponent;
  std::vector<int> reacSidx;      // [nReac][maxSpecInReac], row-major
  std::vector<double> reacNuki;   // [nReac][maxSpecInReac], row-major
  std::vector<int> reacType;      // per reaction: one of the RateType values below

  std::vector<ArrheniusParam> arrhenius;
  std::vector<int> reacPfal;      // Troe reaction indices
  std::vector<double> reacPpar;   // [nTroe][8]: k0_A*1e6, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc, N
  std::vector<CMAQ_H2O2Param> cmaq_h2o2;
  std::vector<JPLParam> jpl;
  std::vector<RJPLArrheniusParam> r_jpl_arrhenius;
  std::vector<AdjustReactionParam> adjust_reaction;
  std::vector<EmissionParam> emission;
  std::vector<ProdO1DParam> prod_O1D;
  int countPhotoRate = 0;

  enum RateType { ARRHENIUS = 0, TROE = 1, CMAQ_H2O2 = 2, JPL = 3, R_JPL_ARRHENIUS = 4, PHOTO_RATE = 5 };

  int nActive() const { return nSpec - nConstSpec; }
  int sidx(int r, int j) const { return reacSidx[r * maxSpecInReac + j]; }
  double nuki(int r, int j) const { return reacNuki[r * maxSpecInReac + j]; }
  int speciesIndex(const std::string& name) const;  // -1 if absent (first match, as std::map::insert keeps the first)

  // Parses an NCAR-format file; writes the kmod.echo lines to `echo` when given.
  static KineticModel fromYamlFile(const std::string& path, std::ostream* echo);
  static KineticModel fromYamlString(const std::string& text, std::ostream* echo);
};

// Scenario reader (src/core/TChem_AtmosphericChemistry.cpp:430-508): fills state[B][nSpec+3]
// with [0, p, T, x_0 .. x_{nSpec-1}] from environmental_conditions and initial_state.
// Units: "mol m-3" verbatim, "molecules cm-3" -> value/conv/1e6, "molecules m-3" -> value/conv,
// where conv = CONV_PPM * p / T.
void setScenarioConditions(const std::string& path, const KineticModel& km, std::vector<double>& state, int& nBatch);

// Photolysis-rate reader (src/core/TChem_AtmosphericChemistry.cpp:512-559): photo[nBatch][nPhoto]
// from photolysis_rates.r_0 .. r_{nPhoto-1}.value, nPhoto = the number of entries of that
// section (0 without it). Every list must hold nBatch values.
void setScenarioPhotolysisRates(const std::string& path, int nBatch, std::vector<double>& photo, int& nPhoto);

// External-forcing reader (src/core/TChem_AtmosphericChemistry.cpp:562-631): ext[nBatch][m],
// zero except the active species named by external_forcing entries (species_name, value list of
// nBatch values; a later entry for the same species overwrites). count = number of entries.
void setScenarioExternalForcing(const std::string& path, const KineticModel& km, int nBatch, std::vector<double>& ext,
                                int& count);

}  // namespace tchem_gb
