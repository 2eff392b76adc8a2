"""E3SM gas chemistry on the CPU: the scenario readers for photolysis rates and external forcing,
and the oracle's restatement of the E3SM rates and time advance pinned to the reference's goldens:

* rate constants, rates of progress and net production rates of the cloned uci samples
  (src/unit-tests/references/{reaction_rates,rate_of_progress,net_production_rates}/*.dat) and of
  the 80-column uci scenario with photolysis rates and external forcing
  (net_production_rates/uci_col/net_production_rates.dat): byte-identical text, the reference's
  own criterion (TChem::Test::compareFiles);
* the E3SM TR-BDF2 advance of the 80 columns over 1800 s
  (atmospheric_chemistry_e3sm/uci_col/full_gas.dat): per species within 10 units of the step
  tolerance (atol + rtol |x|). The reference's own file criterion (compareFilesValues <= 1e-8 on
  the written files) is not met: it measures 1.0e-6 (O3, 0.96 tolerance units), because the two
  integrators take different step sequences and Newton paths (the reference takes 78 doubling
  steps in 72 columns, this restatement's error control 78-86; with the reference's steps imposed
  the columns agree within 1.5 tolerance units); against a solution at rtol 1e-11 the golden is
  within 6.3 tolerance units and the restatement within 2.2. The measured value is bounded here so
  that a change shows.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import (GOLDEN, compare_files_values, format_2d_matrix, format_reaction_rates, manifest, mech_path,
                     printed, tolerance_units)
from oracle import E3smOracle
from oracle.binding import load as load_oracle
from tchem_gb import (KineticModel, set_scenario_conditions, set_scenario_external_forcing,
                      set_scenario_photolysis_rates, time_advance_array)

E3 = GOLDEN / "e3sm"
UCI_COL = E3 / "uci_col_input_conditions.yaml"


def uci_col():
    km = KineticModel.from_file(mech_path("uci_v2_test3.yaml"))
    state = set_scenario_conditions(UCI_COL, km)
    B = state.shape[0]
    return km, state, set_scenario_photolysis_rates(UCI_COL, B), set_scenario_external_forcing(UCI_COL, km, B)


def test_uci_col_scenario_inputs():
    km, state, photo, ext = uci_col()
    assert state.shape == (80, km.state_dim) and km.n_active == 53 and km.nReac == 106
    assert photo.shape == (80, 22) and ext.shape == (80, 53)
    # 11 forcing entries (NO, NO2, SO2, so4_a1, so4_a2, pom_a4, bc_a4, num_a1, num_a2, num_a4, SOAG0),
    # 8 of them nonzero in some column
    forced = [km.species_names[k] for k in np.nonzero(ext.any(axis=0))[0]]
    assert forced == ["NO2", "SO2", "SOAG0", "so4_a1", "pom_a4", "bc_a4", "num_a1", "num_a4"]
    assert np.all(photo >= 0.0) and photo[0, 0] == 0.007049313503079818
    # the golden's initial rows are this scenario, printed with 11 significant digits
    init = np.load(E3 / "uci_col_full_gas.npy")[:80, 3:]
    assert np.abs(init - state).max() <= 1e-10 * np.abs(state).max()
    assert (np.abs(init - state) <= 1e-10 * np.abs(state) + 1e-300).all()


def test_scenario_reader_edge_cases(tmp_path):
    km = KineticModel.from_file(mech_path("uci_v2_test3.yaml"))
    head = ("environmental_conditions:\n  pressure:\n    units: Pa\n    initial_value: [1.0, 2.0]\n"
            "  temperature:\n    units: K\n    initial_value: [250.0, 260.0]\ninitial_state: {}\n")
    p = tmp_path / "none.yaml"
    p.write_text(head)
    assert set_scenario_photolysis_rates(p, 2).shape == (2, 0)
    assert not set_scenario_external_forcing(p, km, 2).any()
    p.write_text(head + "photolysis_rates:\n  r_0:\n    value: [1.0, 2.0]\n  r_1:\n    value: [3.0, 4.0]\n"
                 "external_forcing:\n  e0:\n    species_name: NO\n    value: [5.0, 6.0]\n"
                 "  e1:\n    species_name: NO\n    value: [7.0, 8.0]\n")
    np.testing.assert_array_equal(set_scenario_photolysis_rates(p, 2), [[1.0, 3.0], [2.0, 4.0]])
    ext = set_scenario_external_forcing(p, km, 2)
    k = km.species_names.index("NO")
    np.testing.assert_array_equal(ext[:, k], [7.0, 8.0])  # a later entry for a species overwrites
    assert np.count_nonzero(ext) == 2
    p.write_text(head + "photolysis_rates:\n  r_0:\n    value: [1.0]\n")
    with pytest.raises(RuntimeError, match="photo reaction"):
        set_scenario_photolysis_rates(p, 2)
    p.write_text(head + "photolysis_rates:\n  r_1:\n    value: [1.0, 2.0]\n")
    with pytest.raises(RuntimeError, match="r_0"):
        set_scenario_photolysis_rates(p, 2)
    p.write_text(head + "external_forcing:\n  e0:\n    species_name: M\n    value: [1.0, 2.0]\n")
    with pytest.raises(RuntimeError, match="does not exits"):  # constant species take no forcing
        set_scenario_external_forcing(p, km, 2)


@pytest.mark.parametrize("mech,golden,kind", [("uci.yaml", "reaction-rates.dat", "kfor"),
                                              ("uci_v2.yaml", "rate-of-progress.dat", "rop"),
                                              ("uci_v2.yaml", "net-production-rates.dat", "omega")])
def test_cloned_sample_rates_byte_identical(mech, golden, kind):
    info = manifest()["e3sm"][golden]
    assert info["mechanism"] == f"mechanisms/{mech}"
    km = KineticModel.from_file(mech_path(mech))
    x0 = set_scenario_conditions(mech_path(mech), km)[0]
    o = E3smOracle(km)
    T, p, x = x0[2], x0[1], x0[3:]
    if kind == "kfor":
        v = o.kforward(T, p, x)
    elif kind == "rop":
        v = o.rate_of_progress(T, p, x)
    else:  # the reference's output has nSpec entries, the constant species' left 0
        v = np.zeros(km.nSpec)
        v[:km.n_active] = o.net_production_rates(T, p, x)
    assert format_reaction_rates(v, km.nReac) == (E3 / golden).read_text()


def test_uci_col_net_production_rates_byte_identical():
    km, state, photo, ext = uci_col()
    o = E3smOracle(km)
    W = np.zeros((state.shape[0], km.nSpec))
    for b in range(state.shape[0]):
        W[b, :km.n_active] = o.net_production_rates(state[b, 2], state[b, 1], state[b, 3:], photo[b], ext[b])
    assert format_2d_matrix(W) == (E3 / "uci_col_net_production_rates.dat").read_text()


def uci_col_tadv(B: int, s: dict):
    return time_advance_array(B, tbeg=s["tbeg"], tend=s["tend"], dt=s["dt_in"], dtmin=s["dtmin"], dtmax=s["dtmax"],
                              max_num_newton_iterations=s["max_newton"],
                              num_time_iterations_per_interval=s["iters_per_interval"],
                              jacobian_interval=s["jacobian_interval"])


def test_uci_col_time_advance_matches_reference():
    s = manifest()["e3sm"]["uci_col_full_gas.npy"]["settings"]
    km, state, photo, ext = uci_col()
    B, m = state.shape[0], km.n_active
    tol_time = np.tile([s["atol_time"], s["rtol_time"]], (m, 1))
    out, t, dt, status, stats = E3smOracle(km).time_advance(uci_col_tadv(B, s), state, photo, ext,
                                                            [s["atol_newton"], s["rtol_newton"]], tol_time)
    golden = np.load(E3 / "uci_col_full_gas.npy")[B:]
    assert np.all(status == 0) and np.all(t == 1800.0) and np.all(golden[:, 1] == 1800.0)
    # one runDeviceBatch call of at most 100 steps reaches t_end, as in the reference
    assert stats["n_steps"].max() <= s["iters_per_interval"]
    np.testing.assert_array_equal(out[:, :3], state[:, :3])  # rho, p, T copied through
    np.testing.assert_allclose(out[:, :3], golden[:, 3:6], rtol=1e-10)  # the golden's 11 digits
    np.testing.assert_array_equal(out[:, 3 + m:], state[:, 3 + m:])  # constant species unchanged
    # the reference's file criterion, both sides as written: 1.0e-6 (its 1e-8 is not met, see above)
    assert compare_files_values(printed(out[:, 3:]), golden[:, 6:]) <= 2e-6
    assert tolerance_units(out[:, 3:3 + m], golden[:, 6:6 + m], s["atol_time"], s["rtol_time"]).max() <= 10.0


def test_uci_col_reference_step_sequence_reproduces_every_column_to_1e8():
    """Where the reference's output pins its step sequence, its arithmetic is reproduced to the
    reference's own 1e-8 file criterion. The golden's dt_out (577.685 in columns 8-79, 388.791 in
    0-7) is 2 x the clipped last step of pure doubling from dt_in = 1e-20, in columns 0-7 with the
    step tried at 189 s halved once. Imposing those accepted steps and iterating Newton to
    convergence reproduces every column to about 1e-11. Two facts of the reference run follow. Its
    Newton stages are converged: the restatement's 2-norm test (tol_newton relative to ||y||) ends
    nearly every stage after one iteration on this state, because the aerosol number
    concentrations (up to 1.3e11) dominate ||y||, and that result is 1e-6 from the golden. And its
    step controller is not the restatement's (Hosea & Shampine's filtered estimate takes 79-86
    steps here): that controller is inside Tines, which is absent."""
    s = manifest()["e3sm"]["uci_col_full_gas.npy"]["settings"]
    km, state, photo, ext = uci_col()
    B, m = state.shape[0], km.n_active
    tol_time = np.tile([s["atol_time"], s["rtol_time"]], (m, 1))
    golden = np.load(E3 / "uci_col_full_gas.npy")[B:]
    o = E3smOracle(km)
    L = load_oracle()
    tn = [s["atol_newton"], s["rtol_newton"]]
    # the default test: one Newton iteration in nearly every stage on this state
    *_, stats = o.time_advance(uci_col_tadv(B, s), state, photo, ext, tn, tol_time)
    stages = 2 * (stats["n_steps"] + stats["n_rejected"])
    assert stats["n_newton_iter"].sum() <= 1.05 * stages.sum()
    assert np.mean(stats["n_newton_iter"] == stages) >= 0.8
    doubling = s["dt_in"] * 2.0 ** np.arange(78)               # columns 8-79
    halved = np.concatenate([doubling[:74], doubling[73:78]])  # columns 0-7: 189 s step halved
    for seq, cols, dt_out in ((doubling, slice(8, 80), 577.685), (halved, slice(0, 8), 388.791)):
        # the reference's dt_out: twice the last step, clipped to t_end
        assert abs(2.0 * (s["tend"] - seq[:-1].sum()) - dt_out) < 1e-3
        assert np.allclose(golden[cols, 2], dt_out, atol=1e-3)
        sel = np.arange(B)[cols]
        seq = np.ascontiguousarray(seq)
        assert L.oracle_set_newton_min_iterations(3) == 0
        assert L.oracle_set_step_sequence(len(seq), seq.ctypes.data) == 0
        try:
            out, t, dt, status, st = o.time_advance(uci_col_tadv(len(sel), s), state[sel], photo[sel], ext[sel], tn,
                                                    tol_time)
        finally:
            L.oracle_set_newton_min_iterations(1)
            L.oracle_set_step_sequence(0, None)
        assert np.all(status == 0) and np.all(t == 1800.0) and np.all(st["n_steps"] == len(seq))
        assert compare_files_values(printed(out[:, 3:]), golden[cols, 6:]) <= 1e-8
    assert L.oracle_set_newton_min_iterations(0) != 0
    bad = np.array([1.0, -1.0])
    assert L.oracle_set_step_sequence(2, bad.ctypes.data) != 0


def test_state_dependent_rate_constants_are_rejected():
    """M as an active species scales the JPL rate constants with the state, which the E3SM time
    advance (rate constants once per sample) does not support: the oracle refuses, as the engine."""
    text = """NCAR-version: v1.0
species:
- name: A
- name: M
constant_species: []
reactions:
- coefficients: {k0_A: 1.0e-30, k0_B: -3.0, kinf_A: 1.0e-11, kinf_B: 0.0}
  type: JPL
  reactants: {A: 1, M: 1}
  products: {M: 1}
"""
    km = KineticModel.from_string(text)
    assert km.M_index < km.n_active
    state = np.array([[0.0, 1e5, 280.0, 1.0, 2.5e19]])
    tadv = time_advance_array(1, tend=1.0)
    with pytest.raises(RuntimeError, match="returned 4"):
        E3smOracle(km).time_advance(tadv, state, None, None, [1e-18, 1e-8], np.tile([1e-12, 1e-6], (2, 1)))
