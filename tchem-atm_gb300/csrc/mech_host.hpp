// Mechanism object behind the opaque tchem_gb_mech handle (host part).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tchem_gb.h"
#include "kinetic_model.hpp"

namespace tchem_gb {

struct DeviceTables;  // device-resident packed tables (engine.cuh)

// Thread-local last-error message for tchem_gb_last_error().
void set_last_error(const std::string& msg);

}  // namespace tchem_gb

struct tchem_gb_mech {
  tchem_gb::KineticModel km;
  // Flattened copies backing tchem_gb_kmcd_view.
  std::vector<int32_t> arrhenius_reaction, cmaq_reaction, emission_species, reacPfal;
  std::vector<double> arrhenius_param, cmaq_param, emission_rate;
  tchem_gb_kmcd_view view{};
  // Device tables per CUDA device ordinal (built on first use on that device).
  std::vector<tchem_gb::DeviceTables*> device_tables;

  void build_view();
  ~tchem_gb_mech();
};
