"""The host-model driver interface (include/tchem_gb_driver.h, libtchem_gb_driver.so: the
reference's TChem_Driver functions, src/core/TChem_Driver.hpp:106-132) on the CPU, with the inputs
of the reference's driver test (src/unit-tests/TChem_Driver: CB05CL_AE5 with SIMPOL SOA, its solver
settings file, one sample):

* the gas species names and the aerosol species properties, written as that test writes them,
  against its reference files (identical lines);
* the state and number-concentration accessors, a failed initialize, the solver settings reader
  (the reference's keys and defaults: the file's max_time_iterations is not a key the reference
  reads, so max_num_time_iterations keeps its default of 1000), and a C program compiled and
  linked against the header;
* the oracle's gas-aerosol TR-BDF2 from the test's state over its 30 s step against the
  reference's output under the test's criterion (numpy isclose), which pins the restatement for
  this row.
TChem_doTimestep itself runs the engine's kernel: tests/test_zzz_gpu_aerosol.py.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess

import numpy as np
import pytest

from helpers import GOLDEN, manifest
from oracle import AerosolOracle
from tchem_gb import KineticModel, _capi, time_advance_array
from tchem_gb.aerosol import AerosolModel
from tchem_gb.driver import DRIVER_LIB_PATH, Driver, lib

D = GOLDEN / "driver"
MAN = manifest()["driver"]


def files():
    return GOLDEN / MAN["gas"], GOLDEN / MAN["aero"], GOLDEN / MAN["solver"]


def initial_state(length: int, n_gas: int, n_particles: int):
    """The reference test's state and number concentrations (TChem_Driver.c)."""
    st = np.zeros(length)
    for k, v in MAN["state"].items():
        st[int(k)] = v
    for i in range(n_particles):
        st[3 + n_gas + 5 * i] = MAN["particles"]["first_species"]
    return st, np.full(n_particles, MAN["particles"]["number_conc"])


@pytest.fixture
def driver():
    d = Driver(*files(), MAN["batch"])
    yield d
    d.close()


def test_names_and_properties_match_reference_outputs(driver):
    names = driver.species_names()
    assert "".join(f"{n}\n" for n in names) == (D / "gas_species_names_ref.txt").read_text()
    props = "".join(f"{n} {rho:f} {mw:f} {kappa:f}\n" for n, rho, mw, kappa in driver.aerosol_species())
    assert props == (D / "aero_species_props_ref.txt").read_text()


def test_state_and_number_concentration_accessors(driver):
    L = lib()
    assert driver.length == 92 and driver.n_particles == 1
    assert L.TChem_getNumberOfSpecies() == 84 and L.TChem_getNumberOfAeroSpecies() == 5
    assert L.TChem_getStateVectorSize() == 92
    st, nc = initial_state(driver.length, 84, driver.n_particles)
    driver.set_state(st, 0)
    driver.set_number_concentration(nc, 0)
    np.testing.assert_array_equal(driver.state(0), st)
    np.testing.assert_array_equal(driver.all_states()[0], st)
    assert not driver.state(3).any()  # no such row: nothing copied
    idx = C.c_int(99)
    assert L.TChem_getAerosolSpeciesDensity(C.byref(idx)) == 0.0
    buf = C.create_string_buffer(4)
    idx = C.c_int(0)
    assert L.TChem_getSpeciesName(C.byref(idx), buf, 4) == len("ISOP-P1") and buf.value == b"ISO"


def test_solver_settings_reader():
    n = _capi.Numerics()
    _capi.check(_capi.lib().tchem_gb_numerics_read(str(files()[2]).encode(), C.byref(n)), "tchem_gb_numerics_read")
    assert (n.atol_time, n.rtol_time, n.dtmin, n.atol_newton, n.rtol_newton) == (1e-12, 1e-6, 1e-12, 1e-6, 1e-4)
    assert (n.max_newton_iterations, n.max_num_time_iterations, n.verbose) == (100, 1000, 1)
    assert (n.team_size, n.vector_size) == (-1, -1)


def test_failed_initialize_leaves_driver_uninitialized(tmp_path):
    gas, aero, _ = files()
    with pytest.raises(RuntimeError, match="initialize failed"):
        Driver(gas, aero, tmp_path / "missing.yaml", 1)
    assert lib().TChem_getLengthOfStateVector() == -1
    assert lib().TChem_getNumberConcentrationVectorSize() == -1


def test_c_program_links_against_the_driver_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = GOLDEN.parents[1] / "include"
    src = tmp_path / "host_model.c"
    src.write_text("""#include <stdio.h>
#include "tchem_gb_driver.h"
int main(int argc, char** argv) {
  char name[64];
  int i = 2;
  initialize(argv[1], argv[2], argv[3], 2);
  TChem_getAerosolSpeciesName(&i, name, sizeof(name));
  printf("%d %d %d %s %g\\n", TChem_getNumberOfSpecies(), TChem_getLengthOfStateVector(),
         TChem_getStateVectorSize(), name, TChem_getAerosolSpeciesMW(&i));
  finalize();
  printf("%d\\n", TChem_getLengthOfStateVector());
  return 0;
}
""")
    exe = tmp_path / "host_model"
    pkg = DRIVER_LIB_PATH.parent
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(inc), str(src), "-o", str(exe), "-L", str(pkg),
                        "-ltchem_gb_driver", f"-Wl,-rpath,{pkg}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), *map(str, files())], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-2:] == ["84 92 184 ISOP-P2_aero 0.09003", "-1"]


def test_oracle_reproduces_driver_output():
    gas_file, aero_file, solver_file = files()
    km = KineticModel.from_file(gas_file)
    am = AerosolModel.from_file(aero_file, km)
    n = _capi.Numerics()
    _capi.check(_capi.lib().tchem_gb_numerics_read(str(solver_file).encode(), C.byref(n)), "tchem_gb_numerics_read")
    st, nc = initial_state(am.state_dim, km.nSpec, am.nParticles)
    del_t = MAN["del_t"]
    # the time step TChem_doTimestep takes: [0, del_t] from dtmin, at most del_t per step
    tadv = time_advance_array(1, tend=del_t, dt=n.dtmin, dtmin=n.dtmin, dtmax=del_t,
                              max_num_newton_iterations=n.max_newton_iterations,
                              num_time_iterations_per_interval=n.max_num_time_iterations)
    tol_time = np.tile([n.atol_time, n.rtol_time], (am.n_ode, 1))
    out, t, _, status, _ = AerosolOracle(km, am).time_advance(tadv, st[None], nc[None], [n.atol_newton, n.rtol_newton],
                                                              tol_time)
    assert status[0] == 0 and t[0] == del_t
    ref = np.loadtxt(D / "output_ref.txt")
    assert np.all(np.isclose(out[0], ref))
    assert np.all(np.isclose(np.array([float(f"{v:e}") for v in out[0]]), ref))  # as the test writes it
