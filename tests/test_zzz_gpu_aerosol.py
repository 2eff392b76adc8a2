"""The gas-aerosol (SIMPOL.1 phase transfer) right-hand side and TR-BDF2 advance on the GPU
(tchem_gb_aero_rhs, tchem_gb_aero_time_advance: TChem::AerosolChemistry::runDeviceBatch), against
the reference's goldens and the oracle:

* RHS: the SIMPOL unit golden (partmc_integration/simpol/Simpol_RHS_HOST.txt) written byte for byte
  as the reference writes it; the oracle's RHS at perturbed states of the Simpol model (1 and 3
  particles) and of CB05CL_AE5 with four SIMPOL SOA transfers: gas rows within 1e-12 of the
  largest gas rate (the box-model RHS bound), particle rows within 1e-9 relative;
* advance: the three TinesODE aerosol goldens under their criterion (compare_tchem <= 1e-8);
  16 perturbed samples per model over 100 s against the oracle (compare_tchem <= 1e-8 and the same
  step counts; two CPU builds with different rounding agree to 8e-12 there); the CAMP Simpol
  trajectory within the example's tolerance; in place with skipped samples; 100 particles
  (201 ODEs: the Newton matrix in global memory).

This file sorts after every other test file, so a run that stops at the first failure has run all
the others first."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import GOLDEN, compare_tchem, format_reaction_rates, manifest  # noqa: E402
from oracle import AerosolOracle  # noqa: E402
from tchem_gb import KineticModel, _capi, tadv_to_device, time_advance_array  # noqa: E402
from tchem_gb.aerosol import AerosolChemistry, AerosolModel, AerosolRHS  # noqa: E402

pytestmark = pytest.mark.gpu

A = GOLDEN / "aerosol"
SKIPPED = 2  # TCHEM_GB_SAMPLE_SKIPPED
TINES = manifest()["aerosol"]["tines"]


def models(case: str):
    if case == "simpol":
        km = KineticModel.from_file(A / "simpol_config_gas.yaml")
        return km, AerosolModel.from_file(A / "simpol_phase_transfer.yaml", km), "simpol_config_gas.yaml", \
            "simpol_scenario_particles.yaml"
    km = KineticModel.from_file(A / "cb05_soa_config_full_gas.yaml")
    return km, AerosolModel.from_file(A / "cb05_soa_mechanism_aero.yaml", km), "cb05_soa_config_full_gas.yaml", \
        "cb05_soa_scenario_particles.yaml"


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def gpu_rhs(km, am, state, nc):
    omega = torch.zeros(state.shape[0], am.n_ode, dtype=torch.float64, device="cuda")
    AerosolRHS.runDeviceBatch(dev(state), dev(nc), omega, km, am)
    torch.cuda.synchronize()
    return omega.cpu().numpy()


def oracle_rhs(km, am, row, nc):
    mg, n = km.n_active, km.nSpec
    x = np.concatenate([row[3:3 + mg], row[3 + n:]])
    return AerosolOracle(km, am).rhs(row[2], row[1], nc, x, row[3 + mg:3 + n])


def perturbed(km, am, gas_file, part_file, B, seed):
    """The scenario's first sample perturbed x0.5..1.5, with the SIMPOL gas species at 1e-4..1e-2
    and every particle's aerosol species at 1e-9..1e-7 (so that every transfer is active)."""
    st0, nc0 = am.scenario(A / gas_file, A / part_file)
    rng = np.random.default_rng(seed)
    state = np.tile(st0[:1], (B, 1))
    state[:, 3:] *= rng.uniform(0.5, 1.5, state[:, 3:].shape)
    for g in sorted(set(am.simpol_table()[0][:, 1])):
        state[:, 3 + g] = rng.uniform(1e-4, 1e-2, B)
    first = 3 + km.nSpec
    state[:, first:first + am.nSpec * am.nParticles] = rng.uniform(1e-9, 1e-7, (B, am.nSpec * am.nParticles))
    nc = np.tile(nc0[:1], (B, 1)) * rng.uniform(0.5, 1.5, (B, 1))
    return state, nc


def device_error() -> int:
    err = C.c_int32(0)
    _capi.check(_capi.lib().tchem_gb_device_error(None, None, C.byref(err)), "tchem_gb_device_error")
    return err.value


def test_rhs_reproduces_simpol_unit_golden():
    km, am, _, _ = models("simpol")
    inp = manifest()["aerosol"]["Simpol_RHS_HOST.txt"]["inputs"]
    row = np.zeros((1, am.state_dim))
    row[0, :3] = [1.0, inp["p"], inp["T"]]
    row[0, 3] = inp["ethanol"]
    nc = np.full((1, am.nParticles), inp["number_conc"])
    for i in range(am.nParticles):
        row[0, 3 + km.nSpec + am.nSpec * i] = inp["ethanol_aq"] / nc[0, i]
        row[0, 3 + km.nSpec + am.nSpec * i + 1] = inp["H2O_aq"] / nc[0, i]
    w = gpu_rhs(km, am, row, nc)[0]
    assert format_reaction_rates(w, len(w)) == (A / "Simpol_RHS_HOST.txt").read_text()


@pytest.mark.parametrize("case,particles", [("simpol", None), ("simpol", 3), ("cb05", None)])
def test_rhs_matches_oracle(case, particles):
    km, am, gf, pf = models(case)
    if particles:
        am.set_number_of_particles(particles)
    state, nc = perturbed(km, am, gf, pf, 8, 1)
    w = gpu_rhs(km, am, state, nc)
    mg = km.n_active
    for b in range(state.shape[0]):
        ref = oracle_rhs(km, am, state[b], nc[b])
        # gas rows: sums with cancellation, gathered in another order (the box-model RHS bound)
        assert np.abs(w[b, :mg] - ref[:mg]).max() <= 1e-12 * np.abs(ref[:mg]).max(), b
        # particle rows: condensation minus evaporation (cancels near equilibrium), per element
        aero = ref[mg:]
        scale = np.maximum(np.abs(aero), max(1e-9 * np.abs(aero).max(), 1e-300))
        assert (np.abs(w[b, mg:] - aero) / scale).max() <= 1e-9, b


def gpu_advance(km, am, tadv, state, nc, tol_newton, tol_time, t_out=None, in_place=False):
    B = state.shape[0]
    d_state = dev(state)
    out = d_state if in_place else d_state.clone()
    t = dev(tadv["tbeg"] if t_out is None else t_out)
    dt = torch.zeros_like(t)
    stats = torch.zeros(B * _capi.SAMPLE_STATS_DTYPE.itemsize // 4, dtype=torch.int32, device="cuda")
    status = AerosolChemistry.runDeviceBatch(dev(tol_newton), dev(tol_time), None,
                                             tadv_to_device(tadv, torch.device("cuda")), d_state, dev(nc), t, dt, out,
                                             km, am, stats=stats)
    torch.cuda.synchronize()
    st = np.frombuffer(stats.cpu().numpy().tobytes(), dtype=_capi.SAMPLE_STATS_DTYPE)
    return out.cpu().numpy(), t.cpu().numpy(), dt.cpu().numpy(), status.cpu().numpy(), st


@pytest.mark.parametrize("name", ["tines_full_gas.npy", "tines_batched_full_gas.npy", "tines_batched_cb_full_gas.npy"])
def test_tines_aerosol_goldens_on_the_engine(name):
    s, case = TINES["settings"], TINES["cases"][name]
    km = KineticModel.from_file(A / case["gas"])
    am = AerosolModel.from_file(A / case["aero"], km)
    st0, nc0 = am.scenario(A / case["gas"], A / case["particles"])
    B = case["batch"]
    state, nc = np.tile(st0[:1], (B, 1)), np.tile(nc0[:1], (B, 1))
    tadv = time_advance_array(B, tend=s["tend"], dt=s["dt_in"], dtmin=s["dtmin"], dtmax=s["dtmax"],
                              max_num_newton_iterations=s["max_newton"],
                              num_time_iterations_per_interval=s["iters_per_interval"],
                              jacobian_interval=s["jacobian_interval"])
    tol_time = np.tile([s["atol_time"], s["rtol_time"]], (am.n_ode, 1))
    t, dt = np.zeros(B), np.zeros(B)
    rows = [np.column_stack([np.full(B, -1.0), t, dt, state])]
    for it in range(s["max_intervals"]):
        state, t, dt, status, _ = gpu_advance(km, am, tadv, state, nc, [s["atol_newton"], s["rtol_newton"]], tol_time,
                                              t_out=t)
        assert np.all(status == 0)
        rows.append(np.column_stack([np.full(B, float(it)), t, dt, state]))
        tadv["tbeg"], tadv["dt"] = t, dt
    rows = np.vstack(rows)
    golden = np.load(A / name).reshape(rows.shape)
    assert compare_tchem(rows, golden) <= 1e-8
    assert device_error() == 0


@pytest.mark.parametrize("case", ["simpol", "cb05"])
def test_perturbed_batch_matches_oracle_over_100s(case):
    km, am, gf, pf = models(case)
    B = 16
    state, nc = perturbed(km, am, gf, pf, B, 2)
    tadv = time_advance_array(B, tend=100.0, dt=1e-6, dtmin=1e-20, dtmax=10.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=100000)
    tol_time = np.tile([1e-12, 1e-6], (am.n_ode, 1))
    out, t, dt, status, st = gpu_advance(km, am, tadv, state, nc, [1e-18, 1e-8], tol_time)
    ref, t_r, dt_r, status_r, st_r = AerosolOracle(km, am).time_advance(tadv, state, nc, [1e-18, 1e-8], tol_time)
    assert np.all(status == 0) and np.all(status_r == 0)
    np.testing.assert_array_equal(t, t_r)
    np.testing.assert_array_equal(st["n_steps"], st_r["n_steps"])
    assert compare_tchem(out[:, 3:], ref[:, 3:]) <= 1e-8
    np.testing.assert_array_equal(out[:, :3 + km.nSpec][:, [0, 1, 2]], state[:, :3])
    np.testing.assert_array_equal(out[:, 3 + km.n_active:3 + km.nSpec], state[:, 3 + km.n_active:3 + km.nSpec])


def test_camp_simpol_trajectory_on_the_engine():
    """The Simpol example's settings (tol-time 1e-3, dtmax 10 s, Newton 1e-12 / 1e-8, 20
    iterations) against the CAMP trajectory every 10 s to 100 s, as the oracle's test."""
    km, am, gf, pf = models("simpol")
    state, nc = am.scenario(A / gf, A / pf)
    camp = np.load(A / "camp_simpol.npy")
    tol_time = np.tile([1e-12, 1e-3], (am.n_ode, 1))
    t, dt = np.zeros(1), np.array([1e-20])
    out = [state[0]]
    for tk in camp[1:, 0]:
        tadv = time_advance_array(1, tbeg=t[0], tend=tk, dt=dt[0] if dt[0] > 0 else 1e-20, dtmin=1e-20, dtmax=10.0,
                                  max_num_newton_iterations=20, num_time_iterations_per_interval=1_000_000)
        state, t, dt, status, _ = gpu_advance(km, am, tadv, state, nc, [1e-12, 1e-8], tol_time, t_out=t)
        assert status[0] == 0 and t[0] == tk
        out.append(state[0])
    out = np.array(out)
    ours = out[:, [3, 5, 6]]  # ethanol, ethanol_aq, H2O_aq
    ref = camp[:, [2, 4, 6]]
    assert (np.abs(ours - ref) / np.abs(ref)).max() <= 2e-3


def test_in_place_with_skipped_samples_and_many_particles():
    km, am, gf, pf = models("simpol")
    am.set_number_of_particles(100)  # 201 ODEs: the Newton matrix does not fit in shared memory
    assert am.n_ode == 201
    B = 6
    state, nc = perturbed(km, am, gf, pf, B, 3)
    nc0 = am.scenario(A / gf, A / pf)[1][0, 0]
    nc = nc0 * np.random.default_rng(4).uniform(0.5, 1.5, (B, am.nParticles))
    tadv = time_advance_array(B, tend=5.0, dt=1e-6, dtmin=1e-20, dtmax=1.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=100000)
    t_in = np.zeros(B)
    t_in[[1, 4]] = 5.0  # already at t_end: skipped, rows unchanged
    tol_time = np.tile([1e-12, 1e-6], (am.n_ode, 1))
    out, t, dt, status, _ = gpu_advance(km, am, tadv, state, nc, [1e-18, 1e-8], tol_time, t_out=t_in, in_place=True)
    assert list(status[[1, 4]]) == [SKIPPED] * 2
    np.testing.assert_array_equal(out[[1, 4]], state[[1, 4]])
    live = [0, 2, 3, 5]
    assert np.all(status[live] == 0) and np.all(t[live] == 5.0)
    ref, t_r, _, status_r, _ = AerosolOracle(km, am).time_advance(tadv[live], state[live], nc[live], [1e-18, 1e-8],
                                                                  tol_time)
    assert np.all(status_r == 0)
    assert compare_tchem(out[live, 3:], ref[:, 3:]) <= 1e-8
    assert device_error() == 0


def test_driver_timestep_reproduces_reference_output():
    """The host-model driver interface end to end (libtchem_gb_driver.so: initialize,
    TChem_setStateVector, TChem_setNumberConcentrationVector, TChem_doTimestep(30 s)): the
    reference test's sample against its output under its criterion (numpy isclose) and, with two
    perturbed samples beside it, against the oracle's advance (every row written back)."""
    from test_driver import MAN, files, initial_state
    from tchem_gb.driver import Driver
    d = Driver(*files(), 3)
    try:
        km = KineticModel.from_file(files()[0])
        st, nc = initial_state(d.length, km.nSpec, d.n_particles)
        rng = np.random.default_rng(5)
        rows = np.stack([st, st * np.r_[1, 1, 1, rng.uniform(0.5, 1.5, d.length - 3)],
                         st * np.r_[1, 1, 1, rng.uniform(0.5, 1.5, d.length - 3)]])
        ncs = np.stack([nc, nc * 2.0, nc * 0.5])
        for i in range(3):
            d.set_state(rows[i], i)
            d.set_number_concentration(ncs[i], i)
        d.do_timestep(MAN["del_t"])
        out = d.all_states()
    finally:
        d.close()
    ref = np.loadtxt(GOLDEN / "driver" / "output_ref.txt")
    assert np.all(np.isclose(out[0], ref))
    am = AerosolModel.from_file(files()[1], km)
    n = _capi.Numerics()
    _capi.check(_capi.lib().tchem_gb_numerics_read(str(files()[2]).encode(), C.byref(n)), "tchem_gb_numerics_read")
    tadv = time_advance_array(3, tend=MAN["del_t"], dt=n.dtmin, dtmin=n.dtmin, dtmax=MAN["del_t"],
                              max_num_newton_iterations=n.max_newton_iterations,
                              num_time_iterations_per_interval=n.max_num_time_iterations)
    tol_time = np.tile([n.atol_time, n.rtol_time], (am.n_ode, 1))
    exp, _, _, status, _ = AerosolOracle(km, am).time_advance(tadv, rows, ncs, [n.atol_newton, n.rtol_newton], tol_time)
    assert np.all(status == 0)
    assert compare_tchem(out[:, 3:], exp[:, 3:]) <= 1e-8
    assert device_error() == 0


@pytest.mark.parametrize("name", ["tines_batched_full_gas.npy", "tines_batched_cb_full_gas.npy"])
def test_aerosol_example_on_the_engine(tmp_path, name):
    """The aerosol example driver (tchem_gb.examples.aerosol_chemistry) with the reference's
    TinesODE command line, through the engine's runHostBatch."""
    from test_examples import tines_args
    from tchem_gb.examples import aerosol_chemistry
    out = tmp_path / "full_gas.dat"
    assert aerosol_chemistry.main([*tines_args(name), f"--outputfile={out}",
                                   f"--outputfile_times={tmp_path / 't.json'}"]) == 0
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(A / name).reshape(rows.shape)
    assert compare_tchem(rows, golden) <= 1e-8
