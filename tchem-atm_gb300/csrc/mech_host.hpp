// Mechanism object behind the opaque tchem_gb_mech handle (host part).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tchem_gb.h"
#include "device_tables.hpp"
#include "kinetic_model.hpp"
#include <memory>
#include <mutex>

namespace tchem_gb {

// Thread-local last-error message for tchem_gb_last_error().
void set_last_error(const std::string& msg);

}  // namespace tchem_gb

struct tchem_gb_mech {
  tchem_gb::KineticModel km;
  // Flattened copies backing tchem_gb_kmcd_view.
  std::vector<int32_t> arrhenius_reaction, cmaq_reaction, emission_species, reacPfal;
  std::vector<double> arrhenius_param, cmaq_param, emission_rate;
  tchem_gb_kmcd_view view{};
  // Flattened copies backing tchem_gb_e3sm_view.
  std::vector<int32_t> jpl_reaction, rjpl_reaction, adjust_pair, o1d_index;
  std::vector<double> jpl_param, rjpl_param, o1d_param;
  tchem_gb_e3sm_view e3sm_view{};
  // Packed tables (built on first device use) and their device copies per CUDA device ordinal.
  std::unique_ptr<tchem_gb::HostTables> host_tables;
  std::vector<tchem_gb::DeviceTables*> device_tables;
  std::mutex mu;
  // Threads per sample used when a call leaves it to the library (opts.threads_per_sample == 0),
  // per tchem_gb_form; 0: the narrowest kernel shape. Set by tchem_gb_autotune.
  int tps_pref[3] = {0, 0, 0};

  void build_view();
  ~tchem_gb_mech();
};
