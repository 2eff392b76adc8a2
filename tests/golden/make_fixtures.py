"""Regenerates the golden fixtures of this directory from a TChem-atm source tree.

Usage: python tests/golden/make_fixtures.py /path/to/TChem-atm

Everything copied is data the reference's own tests and examples use:
  * mechanism / scenario YAML files (src/examples/runs/atmospheric_chemistry/...),
  * the mechanism echo files the reference's gtests compare byte-for-byte
    (src/unit-tests/references/*/kmod.echo),
  * the CB05CL_AE5 TR-BDF2 golden (src/unit-tests/CB05CL_AE5/references/full_gas.hdf5), read
    without h5py at its raw data offset (3 x 87 little-endian doubles at byte 2048),
  * the reference's TR-BDF2 trajectory of the Emission case (Emissions.dat) and the CAMP
    analytic/solver result tables of the small test mechanisms (*_results.txt),
  * the E3SM goldens of the reference's gtests: the rate constant, rate-of-progress and
    net-production-rate files (src/unit-tests/references/{reaction_rates,rate_of_progress,
    net_production_rates}/*.dat, compared as text), the 80-column uci scenario they and the E3SM
    time advance read (photolysis rates and external forcing included), and that time advance's
    end states (src/unit-tests/references/atmospheric_chemistry_e3sm/uci_col/full_gas.dat),
  * the aerosol (SIMPOL.1 phase transfer) inputs and goldens: the Simpol and CB05CL_AE5_w_simpolSOA
    example files, the SIMPOL RHS golden (src/unit-tests/references/partmc_integration/simpol/),
    the TR-BDF2 goldens src/unit-tests/TinesODE/references/*.hdf5 (decoded at their raw data
    offset) and the CAMP SIMPOL trajectory,
  * the host-model driver interface test (src/unit-tests/TChem_Driver/): its solver settings file
    and its three reference outputs (gas species names, aerosol species properties, the state
    after one 30 s step).
Run settings of each case come from the reference's scripts and are recorded in manifest.json.
"""
from __future__ import annotations

import json
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
RUNS = "src/examples/runs/atmospheric_chemistry"


def main(ref: Path) -> None:
    mech_dir = HERE / "mechanisms"
    echo_dir = HERE / "echo"
    mech_dir.mkdir(exist_ok=True)
    echo_dir.mkdir(exist_ok=True)
    copies = {
        "cb05cl_ae5.yaml": f"{RUNS}/CB05CL_AE5/config_full_gas.yaml",
        "uci.yaml": f"{RUNS}/uci_e3sm_v3/uci.yaml",
        "uci_v2.yaml": f"{RUNS}/uci_e3sm_v3/uci_v2.yaml",
        "uci_v2_test3.yaml": f"{RUNS}/uci_col/uci_v2_test3.yaml",
        "arrhenius.yaml": f"{RUNS}/Arrhenius/config_arrhenius/config_arrhenius.yaml",
        "troe.yaml": f"{RUNS}/Troe/config_troe/config_troe.yaml",
        "photolysis.yaml": f"{RUNS}/Photolysis/config_photolysis.yaml",
        "cmaq_h2o2.yaml": f"{RUNS}/CMAQ_H2O2/config_cmaq_h2o2.yaml",
        "cmaq_oh_hno3.yaml": f"{RUNS}/CMAQ_OH_HNO3/config_oh_hno3.yaml",
        "emission.yaml": f"{RUNS}/Emission/config_emissions.yaml",
    }
    for dst, src in copies.items():
        shutil.copyfile(ref / src, mech_dir / dst)
    echoes = {
        "uci.echo": "src/unit-tests/references/reaction_rates/kmod.echo",
        "uci_v2.echo": "src/unit-tests/references/net_production_rates/kmod.echo",
        "uci_v2_test3.echo": "src/unit-tests/references/net_production_rates/uci_col/kmod.echo",
    }
    for dst, src in echoes.items():
        shutil.copyfile(ref / src, echo_dir / dst)

    raw = (ref / "src/unit-tests/CB05CL_AE5/references/full_gas.hdf5").read_bytes()
    golden = np.frombuffer(raw[2048:2048 + 261 * 8], dtype="<f8").reshape(3, 87)
    np.save(HERE / "cb05cl_ae5_full_gas.npy", golden)

    traj = np.genfromtxt(ref / f"{RUNS}/Emission/Emissions.dat", skip_header=1)
    np.save(HERE / "emission_trajectory.npy", traj)

    camp = {
        "arrhenius": ("Arrhenius/rxn_arrhenius_results.txt", 1e-6),
        "troe": ("Troe/troe_results.txt", 1e-8),
        "photolysis": ("Photolysis/photolysis_results.txt", 1e-6),
        "cmaq_h2o2": ("CMAQ_H2O2/CMAQ_H2O2_results.txt", 1e-6),
        "cmaq_oh_hno3": ("CMAQ_OH_HNO3/CMAQ_OH_HNO3_results.txt", 1e-6),
        "emission": ("Emission/emission_results.txt", 1e-6),
    }
    for name, (src, _) in camp.items():
        np.save(HERE / f"camp_{name}.npy", np.loadtxt(ref / RUNS / src))

    e3sm_dir = HERE / "e3sm"
    e3sm_dir.mkdir(exist_ok=True)
    e3sm_copies = {
        "uci_col_input_conditions.yaml": f"{RUNS}/uci_col/input_conditions_col.yaml",
        "reaction-rates.dat": "src/unit-tests/references/reaction_rates/reaction-rates.dat",
        "rate-of-progress.dat": "src/unit-tests/references/rate_of_progress/rate-of-progress.dat",
        "net-production-rates.dat": "src/unit-tests/references/net_production_rates/net-production-rates.dat",
        "uci_col_net_production_rates.dat":
            "src/unit-tests/references/net_production_rates/uci_col/net_production_rates.dat",
    }
    for dst, src in e3sm_copies.items():
        shutil.copyfile(ref / src, e3sm_dir / dst)
    full_gas = np.genfromtxt(ref / "src/unit-tests/references/atmospheric_chemistry_e3sm/uci_col/full_gas.dat",
                             skip_header=1)
    np.save(e3sm_dir / "uci_col_full_gas.npy", full_gas)

    aero_dir = HERE / "aerosol"
    aero_dir.mkdir(exist_ok=True)
    aero_copies = {
        "simpol_config_gas.yaml": f"{RUNS}/Simpol/config_gas.yaml",
        "simpol_phase_transfer.yaml": f"{RUNS}/Simpol/test_SIMPOL_phase_transfer.yaml",
        "simpol_scenario_particles.yaml": f"{RUNS}/Simpol/scenario_conditions_particle.yaml",
        "cb05_soa_config_full_gas.yaml": f"{RUNS}/CB05CL_AE5_w_simpolSOA/config_full_gas.yaml",
        "cb05_soa_mechanism_aero.yaml": f"{RUNS}/CB05CL_AE5_w_simpolSOA/mechanism_aero.yaml",
        "cb05_soa_scenario_particles.yaml": f"{RUNS}/CB05CL_AE5_w_simpolSOA/scenario_conditions_particle.yaml",
        "Simpol_RHS_HOST.txt": "src/unit-tests/references/partmc_integration/simpol/Simpol_RHS_HOST.txt",
    }
    for dst, src in aero_copies.items():
        shutil.copyfile(ref / src, aero_dir / dst)
    for name in ("full_gas", "batched_full_gas", "batched_cb_full_gas"):
        raw = (ref / f"src/unit-tests/TinesODE/references/{name}.hdf5").read_bytes()
        n = (len(raw) - 2048) // 8  # one dataset of little-endian doubles at byte 2048
        np.save(aero_dir / f"tines_{name}.npy", np.frombuffer(raw[2048:2048 + 8 * n], dtype="<f8"))
    np.save(aero_dir / "camp_simpol.npy",
            np.loadtxt(ref / RUNS / "Simpol" / "camp_out" / "SIMPOL_phase_transfer_results.txt"))

    driver_dir = HERE / "driver"
    driver_dir.mkdir(exist_ok=True)
    driver_copies = {
        "config_solver.yaml": "src/unit-tests/TChem_Driver/config_solver.yaml",
        "gas_species_names_ref.txt": "src/unit-tests/TChem_Driver/references/gas_species_names_ref.txt",
        "aero_species_props_ref.txt": "src/unit-tests/TChem_Driver/references/aero_species_props_ref.txt",
        "output_ref.txt": "src/unit-tests/TChem_Driver/references/output_ref.txt",
    }
    for dst, src in driver_copies.items():
        shutil.copyfile(ref / src, driver_dir / dst)

    manifest = {
        "cb05cl_ae5_full_gas": {
            "source": "src/unit-tests/CB05CL_AE5/references/full_gas.hdf5",
            "run": "src/unit-tests/CB05CL_AE5/CMakeLists.txt:22-34",
            "mechanism": "mechanisms/cb05cl_ae5.yaml",
            "settings": {"tend": 600, "dtmin": 1e-20, "dtmax": 10, "iters_per_interval": 10, "atol_newton": 1e-18,
                         "rtol_newton": 1e-8, "max_newton": 20, "intervals": 2, "rtol_time": 1e-4,
                         "atol_time": 1e-12},
            "criterion": "compare_tchem.py norm-relative L1/L2/Linf <= 1e-8 (src/unit-tests/scripts/compare_tchem.py)",
        },
        "emission_trajectory": {
            "source": f"{RUNS}/Emission/Emissions.dat",
            "mechanism": "mechanisms/emission.yaml",
            "settings": {"tend": 100, "dtmin": 1e-20, "dtmax": 0.1, "iters_per_interval": 10, "rtol_time": 1e-6,
                         "atol_newton": 1e-18, "rtol_newton": 1e-8, "max_newton": 20, "max_intervals": 200},
            "run": f"{RUNS}/Emission/runModel.sh",
        },
        "camp": {name: {"source": f"{RUNS}/{src}", "mechanism": f"mechanisms/{name}.yaml", "rtol_time": rt,
                        "settings": {"tend": 100, "dtmin": 1e-20, "dtmax": 0.1, "output_every": 1.0}}
                 for name, (src, rt) in camp.items()},
        "echo": {dst: src for dst, src in echoes.items()},
        "aerosol": {
            "files": {f"aerosol/{dst}": src for dst, src in aero_copies.items()},
            "Simpol_RHS_HOST.txt": {"run": "src/unit-tests/TChem_Test_Simpol_RHS.hpp:60-140",
                                    "inputs": {"T": 272.5, "p": 101253.3, "number_conc": 1.3e6, "ethanol": 0.1,
                                               "ethanol_aq": 1.0e-8, "H2O_aq": 1.4e-2},
                                    "criterion": "compareFilesValues <= 1e-12 on the written text"},
            "tines": {
                "source": "src/unit-tests/TinesODE/references/{full_gas,batched_full_gas,batched_cb_full_gas}.hdf5",
                "run": "src/unit-tests/TinesODE/CMakeLists.txt",
                "decode": "one dataset of doubles at byte 2048; rows (iter, t, dt, rho, p, T, species...), "
                          "all samples of an iteration in a row block",
                "settings": {"tend": 600, "dt_in": 1e-20, "dtmin": 1e-20, "dtmax": 10, "iters_per_interval": 10,
                             "max_intervals": 2, "atol_newton": 1e-18, "rtol_newton": 1e-8, "max_newton": 100,
                             "atol_time": 1e-12, "rtol_time": 1e-4, "jacobian_interval": 1},
                "cases": {"tines_full_gas.npy": {"gas": "simpol_config_gas.yaml", "aero": "simpol_phase_transfer.yaml",
                                                 "particles": "simpol_scenario_particles.yaml", "batch": 1},
                          "tines_batched_full_gas.npy": {"gas": "simpol_config_gas.yaml",
                                                         "aero": "simpol_phase_transfer.yaml",
                                                         "particles": "simpol_scenario_particles.yaml", "batch": 3},
                          "tines_batched_cb_full_gas.npy": {"gas": "cb05_soa_config_full_gas.yaml",
                                                            "aero": "cb05_soa_mechanism_aero.yaml",
                                                            "particles": "cb05_soa_scenario_particles.yaml",
                                                            "batch": 3}},
                "criterion": "compare_tchem.py norm-relative L1/L2/Linf <= 1e-8"},
            "camp_simpol.npy": {"source": f"{RUNS}/Simpol/camp_out/SIMPOL_phase_transfer_results.txt",
                                "columns": "time [s], then ethanol, ethanol_aq, H2O_aq as pairs of CAMP columns"},
        },
        "driver": {
            "files": {f"driver/{dst}": src for dst, src in driver_copies.items()},
            "run": "src/unit-tests/TChem_Driver/TChem_Driver.c, CMakeLists.txt (DriverInterface)",
            "gas": "aerosol/cb05_soa_config_full_gas.yaml", "aero": "aerosol/cb05_soa_mechanism_aero.yaml",
            "solver": "driver/config_solver.yaml", "batch": 1,
            "state": {"1": 81060.0, "2": 270.5, "36": 0.001, "50": 0.06, "51": 1e-06, "81": 1e8},
            "particles": {"first_species": 1e-08, "number_conc": 1e4},
            "del_t": 30.0,
            "outputs": {"gas_species_names_ref.txt": "one name per line",
                        "aero_species_props_ref.txt": "name density mw kappa, printf %s %f %f %f",
                        "output_ref.txt": "the state row after TChem_doTimestep, printf %e"},
            "criterion": "names and properties: identical lines; state: numpy isclose (rtol 1e-5, atol 1e-8) "
                         "(src/unit-tests/TChem_Driver/compare_files.py)"},
        "e3sm": {
            "files": {f"e3sm/{dst}": src for dst, src in e3sm_copies.items()},
            "reaction-rates.dat": {"run": "src/unit-tests/TChem_Test_ReactionRates.hpp:28-50",
                                   "mechanism": "mechanisms/uci.yaml", "sample": 0,
                                   "criterion": "byte-identical text (TChem::Test::compareFiles)"},
            "rate-of-progress.dat": {"run": "src/unit-tests/TChem_Test_RateofProgress.hpp:28-50",
                                     "mechanism": "mechanisms/uci_v2.yaml", "sample": 0,
                                     "criterion": "byte-identical text (TChem::Test::compareFiles)"},
            "net-production-rates.dat": {"run": "src/unit-tests/TChem_Test_NetProductionRates.hpp:28-51",
                                         "mechanism": "mechanisms/uci_v2.yaml", "sample": 0,
                                         "criterion": "byte-identical text (TChem::Test::compareFiles)"},
            "uci_col_net_production_rates.dat": {
                "run": "src/unit-tests/TChem_Test_NetProductionRates.hpp:54-79",
                "mechanism": "mechanisms/uci_v2_test3.yaml", "scenario": "e3sm/uci_col_input_conditions.yaml",
                "criterion": "byte-identical text (TChem::Test::compareFiles)"},
            "uci_col_full_gas.npy": {
                "source": "src/unit-tests/references/atmospheric_chemistry_e3sm/uci_col/full_gas.dat",
                "run": "src/unit-tests/TChem_Test_AtmosphericChemistryE3SM.hpp:56-93",
                "mechanism": "mechanisms/uci_v2_test3.yaml", "scenario": "e3sm/uci_col_input_conditions.yaml",
                "rows": "80 initial rows (iter -1) then 80 rows after one runDeviceBatch call (iter 0)",
                "settings": {"tbeg": 0, "tend": 1800, "dt_in": 1e-20, "dtmin": 1e-20, "dtmax": 3600,
                             "iters_per_interval": 100, "atol_newton": 1e-18, "rtol_newton": 1e-8,
                             "max_newton": 20, "atol_time": 1e-12, "rtol_time": 1e-6, "jacobian_interval": 1},
                "criterion": "TChem::Test::compareFilesValues: relative error at the largest absolute "
                             "difference <= 1e-8 (src/core/TChem_Util.hpp:1130-1180)"},
        },
    }
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    print(f"fixtures written to {HERE}")


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
