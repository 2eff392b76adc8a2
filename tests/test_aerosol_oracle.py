"""Aerosol chemistry (SIMPOL.1 gas-particle phase transfer) on the CPU: the aerosol model parser
and particle scenario reader, and the oracle's restatement of the aerosol RHS and its TR-BDF2
advance, pinned to the reference's goldens:

* the SIMPOL RHS unit golden (src/unit-tests/references/partmc_integration/simpol/
  Simpol_RHS_HOST.txt): byte-identical text;
* the TR-BDF2 aerosol goldens src/unit-tests/TinesODE/references/{full_gas, batched_full_gas,
  batched_cb_full_gas}.hdf5 (the Simpol case and CB05CL_AE5 with SIMPOL SOA, 1 and 3 samples):
  compare_tchem <= 1e-8;
* the CAMP SIMPOL trajectory over 100 s (the Simpol example's camp_out): within the example's
  time tolerance (rtol 1e-3), converging towards it as the tolerance tightens.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GOLDEN, compare_tchem, format_reaction_rates, manifest
from oracle import AerosolOracle
from tchem_gb import KineticModel, time_advance_array
from tchem_gb._capi import TChemGBError
from tchem_gb.aerosol import AerosolModel

A = GOLDEN / "aerosol"


def simpol():
    km = KineticModel.from_file(A / "simpol_config_gas.yaml")
    return km, AerosolModel.from_file(A / "simpol_phase_transfer.yaml", km)


def test_simpol_model_tables():
    km, am = simpol()
    assert (km.n_active, km.nConstSpec) == (1, 1)
    assert am.species_names == ["ethanol_aq", "H2O_aq"] and am.nParticles == 1 and am.nSimpol == 1
    assert am.n_ode == 3 and am.state_dim == 3 + 2 + 2
    np.testing.assert_array_equal(np.ctypeslib.as_array(am.view.molecular_weights, (2,)), [0.04607, 0.01801])
    np.testing.assert_array_equal(np.ctypeslib.as_array(am.view.aerosol_density, (2,)), [1000.0, 1000.0])
    idx, par = am.simpol_table()
    np.testing.assert_array_equal(idx, [[1, 0, 1]])  # aerosol ODE index (1 active gas species before it)
    np.testing.assert_array_equal(par, [[-1970.0, 2.91, 0.00196, -0.496, 9.5e-06, 2.55, 0.04607]])
    am.set_number_of_particles(3)
    assert am.nParticles == 3 and am.n_ode == 7


def test_cb05_soa_model_tables():
    km = KineticModel.from_file(A / "cb05_soa_config_full_gas.yaml")
    am = AerosolModel.from_file(A / "cb05_soa_mechanism_aero.yaml", km)
    assert am.nSpec == 5 and am.nSimpol == 4 and am.nParticles == 1
    idx, par = am.simpol_table()
    assert np.all(idx[:, 0] >= km.n_active) and np.all(idx[:, 1] < km.n_active)
    assert am.state_dim == 95 - 3  # the golden rows: iter, t, dt, then the state


def test_aerosol_parser_errors():
    km, _ = simpol()
    base = """NCAR-version:
- name: ethanol
  type: CHEM_SPEC
  diffusion coeff [m2 s-1]: 9.5e-06
  molecular weight [kg mol-1]: 0.04607
- name: ethanol_aq
  phase: AEROSOL
  type: CHEM_SPEC
  density [kg m-3]: 1000.0
  molecular weight [kg mol-1]: 0.04607
  kappa: 0.0
- type: AERO_REP_SINGLE_PARTICLE
  maximum computational particles: 2
- type: MECHANISM
  reactions:
  - type: SIMPOL_PHASE_TRANSFER
    B: [-1970.0, 2.91, 0.00196, -0.496]
    gas-phase species: GAS_SPECIES
    aerosol-phase species: AEROSOL_SPECIES
"""
    am = AerosolModel.from_string(base.replace("GAS_SPECIES", "ethanol").replace("AEROSOL_SPECIES", "ethanol_aq"), km)
    assert am.nParticles == 2 and am.nSimpol == 1
    assert am.simpol_table()[0][0, 2] == 0 and am.simpol_table()[1][0, 5] == 999  # no N star: alpha = 0.1
    with pytest.raises(TChemGBError, match="species does not exit"):
        AerosolModel.from_string(base.replace("GAS_SPECIES", "ethanol").replace("AEROSOL_SPECIES", "nope"), km)
    with pytest.raises(TChemGBError, match="species does not exit"):
        AerosolModel.from_string(base.replace("GAS_SPECIES", "nope").replace("AEROSOL_SPECIES", "ethanol_aq"), km)
    with pytest.raises(TChemGBError, match="parser"):
        AerosolModel.from_string("reactions: []\n", km)


def test_particle_scenario_matches_golden_initial_row():
    km, am = simpol()
    state, nc = am.scenario(A / "simpol_config_gas.yaml", A / "simpol_scenario_particles.yaml")
    np.testing.assert_array_equal(nc, [[1.3e6]])
    golden = np.load(A / "tines_full_gas.npy").reshape(3, 10)
    np.testing.assert_allclose(state[0], golden[0, 3:], rtol=1e-10, atol=0)  # the golden holds 11 digits


def test_simpol_rhs_golden_byte_identical():
    km, am = simpol()
    inp = manifest()["aerosol"]["Simpol_RHS_HOST.txt"]["inputs"]
    nc = np.full(am.nParticles, inp["number_conc"])
    x = np.zeros(am.n_ode)
    x[0] = inp["ethanol"]
    for i in range(am.nParticles):
        x[1 + am.nSpec * i] = inp["ethanol_aq"] / nc[i]
        x[2 + am.nSpec * i] = inp["H2O_aq"] / nc[i]
    w = AerosolOracle(km, am).simpol_rhs(0, inp["T"], inp["p"], nc, x)
    assert format_reaction_rates(w, len(w)) == (A / "Simpol_RHS_HOST.txt").read_text()


def test_particles_are_independent_and_symmetric():
    """With equal particles, every particle block of the aerosol RHS is the same and the gas
    species sees their sum."""
    km, am = simpol()
    o1 = AerosolOracle(km, am)
    x1 = np.array([0.1, 7.7e-15, 1.08e-8])
    w1 = o1.rhs(272.5, 101253.3, [1.3e6], x1, [0.0])
    am.set_number_of_particles(3)
    o3 = AerosolOracle(km, am)
    x3 = np.concatenate([[0.1], np.tile(x1[1:], 3)])
    w3 = o3.rhs(272.5, 101253.3, [1.3e6] * 3, x3, [0.0])
    np.testing.assert_array_equal(w3[1:].reshape(3, 2), np.tile(w1[1:], (3, 1)))
    assert w3[0] == pytest.approx(3 * w1[0], rel=1e-14)


@pytest.mark.parametrize("name", ["tines_full_gas.npy", "tines_batched_full_gas.npy", "tines_batched_cb_full_gas.npy"])
def test_tines_aerosol_goldens(name):
    man = manifest()["aerosol"]["tines"]
    s, case = man["settings"], man["cases"][name]
    km = KineticModel.from_file(A / case["gas"])
    am = AerosolModel.from_file(A / case["aero"], km)
    st0, nc0 = am.scenario(A / case["gas"], A / case["particles"])
    B = case["batch"]  # cloned samples, as the reference's --use_cloned_samples
    state, nc = np.tile(st0[:1], (B, 1)), np.tile(nc0[:1], (B, 1))
    tadv = time_advance_array(B, tend=s["tend"], dt=s["dt_in"], dtmin=s["dtmin"], dtmax=s["dtmax"],
                              max_num_newton_iterations=s["max_newton"],
                              num_time_iterations_per_interval=s["iters_per_interval"],
                              jacobian_interval=s["jacobian_interval"])
    tol_time = np.tile([s["atol_time"], s["rtol_time"]], (am.n_ode, 1))
    o = AerosolOracle(km, am)
    t, dt = np.zeros(B), np.zeros(B)
    rows = [np.column_stack([np.full(B, -1.0), t, dt, state])]
    for it in range(s["max_intervals"]):  # the example's host loop (TChem_AerosolChemistry.cpp:376-410)
        state, t, dt, status, _ = o.time_advance(tadv, state, nc, [s["atol_newton"], s["rtol_newton"]], tol_time,
                                                 t_out=t)
        assert np.all(status == 0)
        rows.append(np.column_stack([np.full(B, float(it)), t, dt, state]))
        tadv["tbeg"], tadv["dt"] = t, dt
    rows = np.vstack(rows)
    golden = np.load(A / name).reshape(rows.shape)
    assert compare_tchem(rows, golden) <= 1e-8


@pytest.mark.parametrize("rtol,bound", [(1e-3, 2e-3), (1e-7, 1e-4)])
def test_camp_simpol_trajectory(rtol, bound):
    """The Simpol example's settings (runModel.sh: tol-time 1e-3, dtmax 10 s, Newton 1e-12 / 1e-8,
    20 iterations) against the CAMP trajectory every 10 s to 100 s; its second column of each
    species pair (single-precision output) is the one the restatement converges to."""
    km, am = simpol()
    state, nc = am.scenario(A / "simpol_config_gas.yaml", A / "simpol_scenario_particles.yaml")
    camp = np.load(A / "camp_simpol.npy")
    o = AerosolOracle(km, am)
    tol_time = np.tile([1e-12 if rtol >= 1e-3 else 1e-14, rtol], (am.n_ode, 1))
    t, dt = np.zeros(1), np.array([1e-20])
    out = [state[0]]
    for tk in camp[1:, 0]:
        tadv = time_advance_array(1, tbeg=t[0], tend=tk, dt=dt[0] if dt[0] > 0 else 1e-20, dtmin=1e-20, dtmax=10.0,
                                  max_num_newton_iterations=20, num_time_iterations_per_interval=1_000_000)
        state, t, dt, status, _ = o.time_advance(tadv, state, nc, [1e-12, 1e-8], tol_time, t_out=t)
        assert status[0] == 0 and t[0] == tk
        out.append(state[0])
    out = np.array(out)
    ours = out[:, [3, 5, 6]]  # ethanol, ethanol_aq, H2O_aq
    ref = camp[:, [2, 4, 6]]
    assert (np.abs(ours - ref) / np.abs(ref)).max() <= bound
