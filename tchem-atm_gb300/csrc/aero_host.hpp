// Aerosol model object behind the opaque tchem_gb_aero handle (host part), and its device tables.
#pragma once

#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/tchem_gb.h"
#include "aerosol_model.hpp"

namespace tchem_gb {

// The aerosol model's SIMPOL and species tables on one device (one allocation).
struct AeroDeviceTables {
  int device = -1;
  const int32_t* sim_idx = nullptr;  // [nSimpol][3], as tchem_gb_aero_view::simpol_index
  const double* sim_par = nullptr;   // [nSimpol][7], as tchem_gb_aero_view::simpol_param
  const double* density = nullptr;   // [nSpec]
  const double* mw = nullptr;        // [nSpec]
  void* allocation = nullptr;
};
void destroy_aero_device_tables(AeroDeviceTables* t);  // defined with the device code

}  // namespace tchem_gb

struct tchem_gb_aero {
  tchem_gb::AerosolModel am;
  // Flattened copies backing tchem_gb_aero_view.
  std::vector<int32_t> simpol_index;
  std::vector<double> simpol_param;
  tchem_gb_aero_view view{};
  // Device copies of the tables per CUDA device ordinal (uploaded on first device use; the
  // number of particles is a launch parameter, so set_number_of_particles keeps them valid).
  std::vector<tchem_gb::AeroDeviceTables*> device_tables;
  std::mutex mu;

  void build_view();
  ~tchem_gb_aero();
};
