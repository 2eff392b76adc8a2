"""E3SM gas chemistry on the GPU, through the C ABI (tchem_gb_e3sm_*), against the reference's
goldens and the CPU oracle:

* rate constants, rates of progress and net production rates of 10 cloned uci samples (the
  reference's gtest setting) and of the 80-column uci scenario with photolysis rates and external
  forcing: the device output formatted as the reference writes it is byte-identical to the golden;
* the E3SM time advance of the 80 columns over 1800 s in the three forms: the plain form within
  1e-8 of the oracle per species; the FP32-LU form within 1e-6; the simplified form (its own
  Newton and step decisions) within 5 units of the step tolerance of the oracle; every form stays
  within 10 tolerance units of the reference's golden per species (the reference's file criterion,
  compareFilesValues <= 1e-8, is not met: 1.0e-6, the integrators' step sequences differ);
* no photolysis input and no sources (NULL arrays) match the oracle; samples already at t_end are
  skipped with their rows kept, in place (state_out = state) and through the host-array variant;
  a mechanism whose rate constants depend on an active species is refused.
"""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import (GOLDEN, compare_files_values, format_2d_matrix, format_reaction_rates, manifest,  # noqa: E402
                     mech_path, printed, rel_error, tolerance_units)
from oracle import E3smOracle  # noqa: E402
from tchem_gb import (KineticModel, set_scenario_conditions, set_scenario_external_forcing,  # noqa: E402
                      set_scenario_photolysis_rates, tadv_to_device, time_advance_array)
from tchem_gb._capi import TChemGBError  # noqa: E402
from tchem_gb.e3sm import AtmosphericChemistryE3SM, NetProductionRates, RateofProgress, ReactionRates  # noqa: E402

pytestmark = pytest.mark.gpu

E3 = GOLDEN / "e3sm"
UCI_COL = E3 / "uci_col_input_conditions.yaml"


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


@pytest.mark.parametrize("mech,golden,kind", [("uci.yaml", "reaction-rates.dat", "kfor"),
                                              ("uci_v2.yaml", "rate-of-progress.dat", "rop"),
                                              ("uci_v2.yaml", "net-production-rates.dat", "omega")])
def test_cloned_sample_rates_on_device_byte_identical(mech, golden, kind):
    km = KineticModel.from_file(mech_path(mech))
    state = dev(np.tile(set_scenario_conditions(mech_path(mech), km)[:1], (10, 1)))
    if kind == "kfor":
        out = torch.empty(10, km.nReac, dtype=torch.float64, device="cuda")
        ReactionRates.runDeviceBatch(state, out, km)
    elif kind == "rop":
        out = torch.empty(10, km.nReac, dtype=torch.float64, device="cuda")
        RateofProgress.runDeviceBatch(state, None, out, km)
    else:
        out = torch.empty(10, km.n_active, dtype=torch.float64, device="cuda")
        NetProductionRates.runDeviceBatch(state, None, None, out, km)
    torch.cuda.synchronize()
    v = out.cpu().numpy()
    assert np.all(v == v[:1])
    row = v[0] if kind != "omega" else np.concatenate([v[0], np.zeros(km.nSpec - km.n_active)])
    assert format_reaction_rates(row, km.nReac) == (E3 / golden).read_text()


def uci_col():
    km = KineticModel.from_file(mech_path("uci_v2_test3.yaml"))
    state = set_scenario_conditions(UCI_COL, km)
    B = state.shape[0]
    return km, state, set_scenario_photolysis_rates(UCI_COL, B), set_scenario_external_forcing(UCI_COL, km, B)


def test_uci_col_rates_on_device():
    km, state, photo, ext = uci_col()
    B, m = state.shape[0], km.n_active
    d_state, d_photo, d_ext = dev(state), dev(photo), dev(ext)
    omega = torch.empty(B, m, dtype=torch.float64, device="cuda")
    NetProductionRates.runDeviceBatch(d_state, d_photo, d_ext, omega, km)
    kfor = torch.empty(B, km.nReac, dtype=torch.float64, device="cuda")
    ReactionRates.runDeviceBatch(d_state, kfor, km, photo_rates=d_photo)
    rop = torch.empty_like(kfor)
    RateofProgress.runDeviceBatch(d_state, d_photo, rop, km)
    torch.cuda.synchronize()
    W = np.zeros((B, km.nSpec))
    W[:, :m] = omega.cpu().numpy()
    assert format_2d_matrix(W) == (E3 / "uci_col_net_production_rates.dat").read_text()
    o = E3smOracle(km)
    for b in (0, 17, 79):
        T, p, x = state[b, 2], state[b, 1], state[b, 3:]
        assert rel_error(kfor[b].cpu().numpy(), o.kforward(T, p, x, photo[b]), 1e-300).max() <= 1e-13
        assert rel_error(rop[b].cpu().numpy(), o.rate_of_progress(T, p, x, photo[b]), 1e-300).max() <= 1e-13


def advance(km, state, photo, ext, tadv, tol_time, tol_newton, form, tps=0):
    B = state.shape[0]
    d_state = dev(state)
    out = torch.empty_like(d_state)
    t = dev(tadv["tbeg"])
    dt = torch.zeros_like(t)
    status = AtmosphericChemistryE3SM.runDeviceBatch(
        dev(tol_newton), dev(tol_time), None, tadv_to_device(tadv), d_state, None if photo is None else dev(photo),
        None if ext is None else dev(ext), t, dt, out, km, form=form, threads_per_sample=tps)
    torch.cuda.synchronize()
    return out.cpu().numpy(), t.cpu().numpy(), status.cpu().numpy()


@pytest.fixture(scope="module")
def uci_col_run():
    s = manifest()["e3sm"]["uci_col_full_gas.npy"]["settings"]
    km, state, photo, ext = uci_col()
    B, m = state.shape[0], km.n_active
    tadv = time_advance_array(B, tbeg=s["tbeg"], tend=s["tend"], dt=s["dt_in"], dtmin=s["dtmin"], dtmax=s["dtmax"],
                              max_num_newton_iterations=s["max_newton"],
                              num_time_iterations_per_interval=s["iters_per_interval"],
                              jacobian_interval=s["jacobian_interval"])
    tol_time = np.tile([s["atol_time"], s["rtol_time"]], (m, 1))
    tol_newton = [s["atol_newton"], s["rtol_newton"]]
    o = E3smOracle(km)
    ref = o.time_advance(tadv, state, photo, ext, tol_newton, tol_time)
    ref_simpl = o.time_advance(tadv, state, photo, ext, tol_newton, tol_time, lu_fp32=1, simplified=True)
    golden = np.load(E3 / "uci_col_full_gas.npy")[B:]
    return km, state, photo, ext, tadv, tol_time, tol_newton, ref, ref_simpl, golden, s


@pytest.mark.parametrize("form,tps", [("plain", 0), ("mixed", 0), ("simplified", 32), ("simplified", 64)])
def test_uci_col_time_advance(uci_col_run, form, tps):
    km, state, photo, ext, tadv, tol_time, tol_newton, ref, ref_simpl, golden, s = uci_col_run
    m = km.n_active
    out, t, status = advance(km, state, photo, ext, tadv, tol_time, tol_newton, form, tps)
    assert np.all(status == 0) and np.all(t == s["tend"])
    y, y_ref = out[:, 3:3 + m], ref[0][:, 3:3 + m]
    if form == "plain":
        assert rel_error(y, y_ref, s["atol_time"]).max() <= 1e-8
    elif form == "mixed":
        assert rel_error(y, y_ref, s["atol_time"]).max() <= 1e-6
    else:
        assert tolerance_units(y, ref_simpl[0][:, 3:3 + m], s["atol_time"], s["rtol_time"]).max() <= 5.0
        assert tolerance_units(y, y_ref, s["atol_time"], s["rtol_time"]).max() <= 5.0
    np.testing.assert_array_equal(out[:, :3], state[:, :3])
    np.testing.assert_array_equal(out[:, 3 + m:], state[:, 3 + m:])
    if form in ("plain", "mixed"):  # they follow the oracle's steps: its 1.0e-6 (the simplified form's own
        # steps move the largest absolute difference to another species; its tolerance units below)
        assert compare_files_values(printed(out[:, 3:]), golden[:, 6:]) <= 2e-6
    assert tolerance_units(y, golden[:, 6:6 + m], s["atol_time"], s["rtol_time"]).max() <= 10.0


def test_no_photolysis_and_no_sources_match_oracle(uci_col_run):
    km, state, photo, ext, tadv, tol_time, tol_newton, *_ = uci_col_run
    m = km.n_active
    sel = slice(0, 16)
    tadv = tadv[sel].copy()
    tadv["tend"] = 60.0
    ref = E3smOracle(km).time_advance(tadv, state[sel], None, None, tol_newton, tol_time)
    out, t, status = advance(km, state[sel], None, None, tadv, tol_time, tol_newton, "plain")
    assert np.all(status == 0) and np.all(ref[3] == 0) and np.all(t == 60.0)
    assert rel_error(out[:, 3:3 + m], ref[0][:, 3:3 + m], tol_time[0, 0]).max() <= 1e-8


def test_state_dependent_rate_constants_are_refused():
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
    state = np.array([[0.0, 1e5, 280.0, 1.0, 2.5e19]])
    tadv = time_advance_array(1, tend=1.0)
    with pytest.raises(TChemGBError, match="active species"):
        advance(km, state, None, None, tadv, np.tile([1e-12, 1e-6], (2, 1)), [1e-18, 1e-8], "plain")


def test_skipped_samples_in_place_and_host_batch(uci_col_run):
    """Samples with t_out >= t_end are skipped and keep their rows; state_out may be state (the
    reference's E3SM driver advances in place); the host-array variant gives the same results."""
    km, state, photo, ext, tadv, tol_time, tol_newton, *_ = uci_col_run
    m = km.n_active
    sel = slice(0, 16)
    tadv = tadv[sel].copy()
    tadv["tend"] = 60.0
    t0 = np.zeros(16)
    t0[::2] = 60.0  # every other sample is already at t_end
    ref = E3smOracle(km).time_advance(tadv, state[sel], photo[sel], ext[sel], tol_newton, tol_time, t_out=t0)
    d_state = dev(state[sel])
    t = dev(t0)
    dt = torch.zeros_like(t)
    st = AtmosphericChemistryE3SM.runDeviceBatch(dev(tol_newton), dev(tol_time), None, tadv_to_device(tadv), d_state,
                                                 dev(photo[sel]), dev(ext[sel]), t, dt, d_state, km)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    out = d_state.cpu().numpy()
    assert np.all(st[::2] == 2) and np.all(st[1::2] == 0) and np.all(ref[3] == st)
    np.testing.assert_array_equal(out[::2], state[sel][::2])
    assert rel_error(out[1::2, 3:3 + m], ref[0][1::2, 3:3 + m], tol_time[0, 0]).max() <= 1e-8
    h_out, h_t, h_dt, h_st = AtmosphericChemistryE3SM.runHostBatch(tol_newton, tol_time, tadv, state[sel], photo[sel],
                                                                   ext[sel], t0, km)
    np.testing.assert_array_equal(h_st, st)
    np.testing.assert_array_equal(h_out, out)
    np.testing.assert_array_equal(h_t, t.cpu().numpy())


@pytest.mark.parametrize("chem,inputfile,extra,golden", [
    ("uci_v2.yaml", None, ["--batch_size=10", "--use_cloned_samples=true"], "net-production-rates.dat"),
    ("uci_v2_test3.yaml", "uci_col_input_conditions.yaml", [], "uci_col_net_production_rates.dat")])
def test_example_driver_writes_the_reference_output(tmp_path, chem, inputfile, extra, golden):
    """The example driver, run with the reference gtest's options, writes the golden file."""
    from tchem_gb.examples import net_production_rates as ex
    out = tmp_path / "npr.dat"
    args = [f"--chemfile={mech_path(chem)}", f"--outputfile={out}", f"--outputfile_times={tmp_path / 't.json'}",
            "--verbose=true", *extra]
    if inputfile:
        args.append(f"--inputfile={E3 / inputfile}")
    assert ex.main(args) == 0
    assert out.read_text() == (E3 / golden).read_text()
