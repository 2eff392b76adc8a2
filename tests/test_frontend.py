"""Front end (CPU): YAML reader, kinetic model tables, mechanism echo, scenario reader, generator,
and the C ABI's exported symbols."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from helpers import GOLDEN, mech_path
from tchem_gb import KineticModel, set_scenario_conditions
from tchem_gb import _capi
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states, scenario_yaml

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("mech,echo", [("uci.yaml", "uci.echo"), ("uci_v2.yaml", "uci_v2.echo"),
                                       ("uci_v2_test3.yaml", "uci_v2_test3.echo")])
def test_echo_matches_reference_byte_for_byte(tmp_path, mech, echo):
    # The reference's gtests compare kmod.echo byte-exactly (TChem::Test::compareFiles).
    out = tmp_path / "kmod.echo"
    KineticModel.from_file(mech_path(mech), echo_path=out)
    assert out.read_bytes() == (GOLDEN / "echo" / echo).read_bytes()


def test_cb05cl_ae5_tables():
    km = KineticModel.from_file(mech_path("cb05cl_ae5.yaml"))
    assert (km.nSpec, km.nConstSpec, km.nReac) == (81, 7, 187)
    assert km.species_names[km.M_index] == "M"
    sidx, nuki = km.stoichiometry()
    v = km.view
    assert km.maxSpecInReac == 2 * 5 or km.maxSpecInReac % 2 == 0
    # R2: O + O2 + M -> O3 + M (3 reactants sorted by species index; constant species last)
    names = km.species_names
    r2 = [names[sidx[1, j]] for j in range(v.reacNreac[1])]
    assert sorted(r2) == ["M", "O", "O2"] and r2[-1] in ("M", "O2")
    assert all(nuki[1, j] == -1.0 for j in range(3))
    # convExponent = sum |nu_reac| - 1
    assert v.convExponent[1] == 2
    assert v.nArrhenius == 168 and v.nTroe == 16 and v.nCMAQ_H2O2 == 3


def test_scenario_reader_matches_golden_initial_state():
    km = KineticModel.from_file(mech_path("cb05cl_ae5.yaml"))
    state = set_scenario_conditions(mech_path("cb05cl_ae5.yaml"), km)
    golden = np.load(GOLDEN / "cb05cl_ae5_full_gas.npy")
    assert state.shape == (1, 84)
    np.testing.assert_array_equal(state[0], golden[0, 3:])


def test_scenario_units(tmp_path):
    # "molecules m-3" -> value/conv (src/core/TChem_AtmosphericChemistry.cpp:478-486)
    km = KineticModel.from_file(mech_path("arrhenius.yaml"))
    state = set_scenario_conditions(mech_path("arrhenius.yaml"), km)
    conv = 7.24296358205307e10 * state[:, 1] / state[:, 2]
    d = km.species_names.index("D")
    np.testing.assert_allclose(state[:, 3 + d], np.array([1.2, 17.0, 13.0, 9.0, 4.0]) / conv, rtol=1e-15)


def test_yaml_subset_features():
    text = """NCAR-version: v1.0   # comment
species:
- name: A
- description: a long
    description over two lines
  name: B
constant_species:
- {name: M}
reactions:
- reactants: &r1
    A: 1
  products: {B: 1.0}
  type: 'ARRHENIUS'
  coefficients:
    A: 2.0e-3
- reactants: *r1
  products: {}
  type: ARRHENIUS
  coefficients:
"""
    km = KineticModel.from_string(text)
    assert km.species_names == ["A", "B", "M"]
    assert km.nReac == 2
    v = km.view
    assert v.reacNprod[1] == 0 and v.reacNreac[1] == 1
    # Empty coefficients: A = 1, B = C = 0, D = 300, E = 0 (src/core/TChem_KineticModelData.cpp:396-447)
    assert list(v.arrhenius_param[5:10]) == [0.0, 1.0, 0.0, 0.0, 300.0]
    assert v.arrhenius_param[1] == 2.0e-3


@pytest.mark.parametrize("text,match", [
    ("NCAR-version: v1\nspecies:\n- name: A\nreactions: []\n", "M species"),
    ("NCAR-version: v1\nconstant_species:\n- name: M\nspecies:\n- name: A\nreactions:\n- reactants: {Z: 1}\n"
     "  products: {A: 1}\n  type: ARRHENIUS\n", "species does not exit Z"),
    ("NCAR-version: v1\nconstant_species:\n- name: M\nspecies:\n- name: A\nreactions:\n- reactants: {A: 1}\n"
     "  products: {A: 1}\n  type: NOPE\n", "reaction type does not exit"),
    ("species: []\n", "parser"),
])
def test_front_end_errors(text, match):
    with pytest.raises(_capi.TChemGBError, match=match):
        KineticModel.from_string(text)


def test_ea_and_time_unit_rules():
    text = """NCAR-version: v1
constant_species:
- name: M
species:
- name: A
reactions:
- reactants: {A: 1}
  products: {A: 1}
  type: ARRHENIUS
  time_unit: min
  coefficients: {A: 60.0, Ea: 1.3806504e-21}
- reactants: {A: 1, M: 1}
  products: {A: 1}
  type: TROE
  coefficients: {k0_A: 1.0e-30}
"""
    km = KineticModel.from_string(text)
    v = km.view
    E, A, B, Cc, D = v.arrhenius_param[0:5]
    assert A == 1.0 and Cc == pytest.approx(-100.0) and D == 300.0
    ppar = [v.reacPpar[i] for i in range(8)]
    assert ppar[0] == pytest.approx(1e-24) and ppar[6] == 0.6 and ppar[7] == 1.0 and ppar[3] == 1.0


def test_generator_is_seeded_and_shaped():
    spec = MechanismSpec()
    y1, y2 = mechanism_yaml(spec), mechanism_yaml(spec)
    assert y1 == y2
    km = KineticModel.from_string(y1)
    assert (km.n_active, km.nConstSpec, km.nReac) == (51, 1, 156)
    v = km.view
    assert v.nTroe == 16
    n_photo = y1.count("PHOTOLYSIS")
    assert n_photo == 47 and v.nArrhenius == 156 - 16
    sidx, nuki = km.stoichiometry()
    half = km.maxSpecInReac // 2
    for r in range(km.nReac):
        assert 1 <= v.reacNreac[r] <= 2 and 1 <= v.reacNprod[r] <= 4
        assert all(float(nuki[r, j]).is_integer() for j in range(v.reacNreac[r]))
        assert all(float(nuki[r, half + j]).is_integer() for j in range(v.reacNprod[r]))
    night = KineticModel.from_string(mechanism_yaml(spec, night=True))
    assert night.nReac == km.nReac


def test_generated_scenario_round_trip(tmp_path):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=8, n_reactions=20, seed=3)))
    st = sample_states(5, km.n_active, seed=11)
    path = tmp_path / "scenario.yaml"
    path.write_text(scenario_yaml(st, km.species_names[:km.n_active], km.n_active))
    back = set_scenario_conditions(path, km)
    np.testing.assert_array_equal(back[:, 1:3 + km.n_active], st[:, 1:3 + km.n_active])


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "tchem_gb.h").read_text()
    names = set(re.findall(r"^\s*(?:const\s+)?[a-zA-Z_][\w\s\*]*?\b(tchem_gb_\w+)\s*\(", header, flags=re.M))
    assert len(names) >= 15
    lib = C.CDLL(str(_capi.LIB_PATH))
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_cpp_shim_compiles_links_and_parses(tmp_path):
    """The C++ face in include/tchem_gb_atm.hpp builds against the library and parses a mechanism
    with the reference's names (host-only calls, no GPU)."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "shim.cpp"
    src.write_text(
        '#include "tchem_gb_atm.hpp"\n#include <cstdio>\n'
        "int main(int argc, char** argv) {\n"
        "  tchem_gb::KineticModel km(argv[1]);\n"
        "  tchem_gb_kmcd_view v = km.view();\n"
        '  std::printf("%d %d %d\\n", v.nSpec, v.nConstSpec, v.nReac);\n'
        "  if (argc > 4) {  // referenced, not run: the device entry points of the C++ face link\n"
        "    tchem_gb::AtmosphericChemistry::autotune(nullptr, km, 2, 0, nullptr, nullptr, nullptr, nullptr, nullptr,\n"
        "                                             nullptr, nullptr, nullptr);\n"
        "    tchem_gb::AtmosphericChemistry::adjointDeviceBatch(nullptr, nullptr, nullptr, nullptr, nullptr, km, 0,\n"
        "                                                       nullptr, nullptr, nullptr, 1, nullptr, nullptr, nullptr,\n"
        "                                                       nullptr);\n"
        "    tchem_gb::AtmosphericChemistryE3SM::runDeviceBatch(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,\n"
        "                                                       nullptr, 0, nullptr, nullptr, nullptr, nullptr, km, 0,\n"
        "                                                       nullptr);\n"
        "    tchem_gb::NetProductionRates::runDeviceBatch(nullptr, nullptr, nullptr, 0, nullptr, nullptr, km, 0);\n"
        "  }\n"
        "  if (argc > 3) {  // an aerosol model over this gas mechanism\n"
        "    tchem_gb::AerosolModel am(argv[3], km);\n"
        '    std::printf("aero %d %d\\n", am.view().nSpec, am.view().nSimpol);\n'
        "    if (argc > 4)  // referenced, not run: the gas-aerosol time advance of the C++ face links\n"
        "      tchem_gb::AerosolChemistry::runDeviceBatch(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,\n"
        "                                                 nullptr, nullptr, nullptr, km, am, 0, nullptr);\n"
        "  }\n"
        "  tchem_gb_e3sm_view e = km.e3sm_view();\n"
        '  std::printf("%d %d\\n", e.nJPL, e.nAdjust);\n'
        "  try { tchem_gb::KineticModel bad(\"/nonexistent.yaml\"); } catch (const std::logic_error&) { return 0; }\n"
        "  return 1;\n}\n")
    exe = tmp_path / "shim"
    libdir = Path(_capi.LIB_PATH).parent
    r = subprocess.run([cxx, "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{libdir}",
                        "-ltchem_gb", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), str(mech_path("uci_v2_test3.yaml"))], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    km = KineticModel.from_file(mech_path("uci_v2_test3.yaml"))
    assert km.e3sm_view.nJPL == 10 and km.e3sm_view.nAdjust == 83  # the echo's adjustment pairs
    aero_dir = mech_path("x").parent.parent / "aerosol"
    out_a = subprocess.run([str(exe), str(aero_dir / "simpol_config_gas.yaml"), "0", str(aero_dir / "simpol_phase_transfer.yaml")],
                           capture_output=True, text=True)
    assert out_a.returncode == 0, out_a.stderr
    assert "aero 2 1" in out_a.stdout
    assert out.stdout.split() == [str(km.nSpec), str(km.nConstSpec), str(km.nReac), str(km.e3sm_view.nJPL),
                                  str(km.e3sm_view.nAdjust)]
