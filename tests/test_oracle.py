"""Pins the CPU oracle against the reference's own golden data (CPU only).

* CB05CL_AE5 TR-BDF2 golden (src/unit-tests/CB05CL_AE5/references/full_gas.hdf5) with the
  reference's compare_tchem criterion at 1e-8;
* the reference's Emission trajectory (Emissions.dat): same step sequence, same states;
* CAMP analytic solutions of the small test mechanisms, to solver tolerance;
* the analytic Jacobian against central differences;
* the failure conventions of the reference's integrators.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GOLDEN, compare_tchem, host_time_loop, manifest, mech_path, rel_error
from oracle import Oracle
from tchem_gb import KineticModel, set_scenario_conditions, time_advance_array
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states


def _advance_oracle(o, tol_newton, tol_time):
    def adv(tadv, state, t):
        so, t_o, dt_o, st, _ = o.time_advance(tadv, state, tol_newton, tol_time, t_out=t)
        assert np.all((st == 0) | (st == 2))
        return so, t_o, dt_o
    return adv


def run_settings(km, state, s):
    m = km.n_active
    tadv = time_advance_array(state.shape[0], tbeg=0.0, tend=s["tend"], dt=s["dtmin"], dtmin=s["dtmin"],
                              dtmax=s["dtmax"], max_num_newton_iterations=s.get("max_newton", 20),
                              num_time_iterations_per_interval=s["iters_per_interval"])
    tol_time = np.tile([s.get("atol_time", 1e-12), s["rtol_time"]], (m, 1))
    tol_newton = [s.get("atol_newton", 1e-18), s.get("rtol_newton", 1e-8)]
    return tadv, tol_time, tol_newton


def test_oracle_reproduces_cb05cl_ae5_golden():
    man = manifest()["cb05cl_ae5_full_gas"]
    s = man["settings"]
    km = KineticModel.from_file(mech_path("cb05cl_ae5.yaml"))
    state = set_scenario_conditions(mech_path("cb05cl_ae5.yaml"), km)
    tadv, tol_time, tol_newton = run_settings(km, state, s)
    o = Oracle([km])
    rows, _ = host_time_loop(_advance_oracle(o, tol_newton, tol_time), state, tadv, s["tend"], s["intervals"],
                             s["dtmax"])
    golden = np.load(GOLDEN / "cb05cl_ae5_full_gas.npy")
    assert rows.shape == golden.shape
    assert compare_tchem(rows, golden) <= 1e-8


def test_oracle_reproduces_reference_emission_trajectory():
    s = manifest()["emission_trajectory"]["settings"]
    km = KineticModel.from_file(mech_path("emission.yaml"))
    state = set_scenario_conditions(mech_path("emission.yaml"), km)
    tadv, tol_time, tol_newton = run_settings(km, state, s)
    rows, _ = host_time_loop(_advance_oracle(Oracle([km]), tol_newton, tol_time), state, tadv, s["tend"],
                             s["max_intervals"], s["dtmax"])
    ref = np.load(GOLDEN / "emission_trajectory.npy")
    # The reference file predates the constant species M; compare iter, t, dt, rho, p, T, A, B.
    assert rows.shape[0] == ref.shape[0] == 108
    np.testing.assert_array_equal(rows[:, 0], ref[:, 0])
    # The file holds 11 significant digits.
    assert rel_error(rows[:, 1:8], ref[:, 1:8], 1e-300).max() < 1e-10
    assert rows[-1, 1] == 100.0 and rows[-1, 2] == 0.0  # lands on t_end, dt_out = 0


@pytest.mark.parametrize("case", ["arrhenius", "troe", "photolysis", "cmaq_h2o2", "cmaq_oh_hno3", "emission"])
def test_oracle_matches_camp_solutions(case):
    info = manifest()["camp"][case]
    km = KineticModel.from_file(GOLDEN / info["mechanism"])
    state = set_scenario_conditions(GOLDEN / info["mechanism"], km)[:1]
    camp = np.load(GOLDEN / f"camp_{case}.npy")
    m = km.n_active
    o = Oracle([km])
    tadv = time_advance_array(1, dt=1e-20, dtmin=1e-20, dtmax=0.1, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=100000)
    tol_time = np.tile([1e-12, info["rtol_time"]], (m, 1))
    out = [state[0, 3:3 + m].copy()]
    t = np.zeros(1)
    for k in range(1, camp.shape[0]):
        tadv["tbeg"], tadv["tend"] = t, camp[k, 0]
        state, t, dt, st, _ = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, t_out=t)
        assert st[0] == 0 and t[0] == camp[k, 0]
        tadv["dt"] = np.where(dt > 0, dt, 1e-20)
        out.append(state[0, 3:3 + m].copy())
    out = np.array(out)
    ncol = (camp.shape[1] - 1) // 2
    for c in range(min(ncol, m)):
        solver, analytic = camp[:, 1 + 2 * c], camp[:, 2 + 2 * c]
        # The photolysis table's analytic columns for B and C are off by a factor 2 from CAMP's own
        # solver column; compare with the solver there.
        target = solver if case == "photolysis" and c > 0 else analytic
        scale = np.max(np.abs(target))
        assert np.max(np.abs(out[:, c] - target)) / scale < 2e-5, (case, km.species_names[c])


def _fd_jacobian(o, T, p, x, m, h=1e-3):
    # Mass-action rates are polynomials of degree <= 2 in each concentration, so central
    # differences have no truncation error and a large step keeps cancellation small.
    J = np.zeros((m, m))
    for j in range(m):
        dx = h * max(abs(x[j]), 1e-4)
        xp, xm = x.copy(), x.copy()
        xp[j] += dx
        xm[j] -= dx
        J[:, j] = (o.reaction_rates(T, p, xp) - o.reaction_rates(T, p, xm)) / (2 * dx)
    return J


@pytest.mark.parametrize("which", ["cb05cl_ae5", "generated"])
def test_analytic_jacobian_matches_central_differences(which):
    if which == "cb05cl_ae5":
        km = KineticModel.from_file(mech_path("cb05cl_ae5.yaml"))
        state = set_scenario_conditions(mech_path("cb05cl_ae5.yaml"), km)[0]
        state = state.copy()
        state[3:3 + km.n_active] += 1e-3  # make every species nonzero
    else:
        km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
        state = sample_states(1, km.n_active, seed=5)[0]
    o = Oracle([km])
    m = km.n_active
    T, p, x = state[2], state[1], state[3:3 + km.nSpec]
    J = o.jacobian(T, p, x)
    Jfd = _fd_jacobian(o, T, p, x.copy(), m)[:m]
    scale = np.maximum(np.abs(J).max(axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(J - Jfd) / scale) < 1e-5


def _generated_batch(B, seed=7):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=3600.0, dt=1e-10, dtmin=1e-10, dtmax=3600.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    tol_time = np.tile([1e-12, 1e-6], (km.n_active, 1))
    return km, state, tadv, tol_time


def test_fp32_lu_mode_tracks_fp64():
    km, state, tadv, tol_time = _generated_batch(8)
    o = Oracle([km])
    a = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time)
    b = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, lu_fp32=True)
    m = km.n_active
    assert np.all(a[3] == 0) and np.all(b[3] == 0)
    assert np.all(a[1] == 3600.0) and np.all(b[1] == 3600.0)
    err = rel_error(b[0][:, 3:3 + m], a[0][:, 3:3 + m], 1e-10)
    assert err.max() < 1e-5
    # one FP64-residual refinement sweep per Newton solve (the engine's mixed form) follows the
    # FP64 Newton iterates
    c = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, lu_fp32=2)
    assert rel_error(c[0][:, 3:3 + m], a[0][:, 3:3 + m], 1e-12).max() < 1e-7
    np.testing.assert_array_equal(c[4]["n_steps"], a[4]["n_steps"])


@pytest.mark.parametrize("lu_fp32", [0, 1])
def test_simplified_newton_mode_tracks_fp64(lu_fp32):
    """Carried factors, componentwise Newton test and the filter at I - c J(y_{n+1}): end states
    within 1e-6 of the full-Newton FP64 run, with the same step sequence and about a quarter of
    the factorizations."""
    km, state, tadv, tol_time = _generated_batch(16, seed=21)
    o = Oracle([km])
    a = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time)
    b = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, lu_fp32=lu_fp32, simplified=True)
    m = km.n_active
    assert np.all(b[3] == 0) and np.all(b[1] == 3600.0)
    assert rel_error(b[0][:, 3:3 + m], a[0][:, 3:3 + m], 1e-12).max() <= 1e-6
    assert abs(b[4]["n_steps"].mean() / a[4]["n_steps"].mean() - 1.0) < 0.01
    assert b[4]["n_lu"].sum() < 0.35 * a[4]["n_lu"].sum()
    # every accepted step formed the filter factors once
    assert np.all(b[4]["n_lu"] >= b[4]["n_steps"])


def test_failure_conventions():
    km, state, tadv, tol_time = _generated_batch(3)
    o = Oracle([km])
    # Unreachable Newton tolerance (negative): 4 halvings, then state 0, t_out = t_end, dt_out = -1.
    so, t, dt, st, stats = o.time_advance(tadv, state, [-1.0, 0.0], tol_time)
    assert np.all(st == 1) and np.all(t == 3600.0) and np.all(dt == -1.0)
    assert np.all(so[:, 3:3 + km.n_active] == 0.0)
    assert np.all(stats["n_newton_fail"] == 4) and np.all(stats["n_steps"] == 0)
    # dt_in < 0: status 3, outputs untouched.
    tadv2 = tadv.copy()
    tadv2["dt"] = -1.0
    so, t, dt, st, _ = o.time_advance(tadv2, state, [1e-18, 1e-8], tol_time, t_out=np.full(3, 0.0))
    assert np.all(st == 3) and np.all(t == 0.0)
    np.testing.assert_array_equal(so, state)
    # Samples already at t_end are skipped.
    so, t, dt, st, _ = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, t_out=np.full(3, 3600.0))
    assert np.all(st == 2)
    np.testing.assert_array_equal(so, state)


def test_step_budget_resumes_like_the_host_loop():
    km, state, tadv, tol_time = _generated_batch(2)
    o = Oracle([km])
    full = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time)
    t2 = tadv.copy()
    t2["num_time_iterations_per_interval"] = 50
    st, t = state.copy(), np.zeros(2)
    for _ in range(10000):
        st, t, dt, status, _ = o.time_advance(t2, st, [1e-18, 1e-8], tol_time, t_out=t)
        t2["tbeg"], t2["dt"] = t, dt
        if np.all(t >= 3600.0):
            break
    # Splitting the run into 50-step calls reproduces the single call exactly.
    np.testing.assert_array_equal(st, full[0])


def test_adjoint_restatement_dot_product_and_finite_differences():
    """The oracle's discrete adjoint against its forward sensitivities (dot-product test) and
    central differences of the recorded-step replay."""
    from oracle import binding as ob
    km, state, tadv, tol_time = _generated_batch(2, seed=13)
    tadv["tend"] = tadv["dtmax"] = 300.0
    o = Oracle([km])
    m, R = km.n_active, km.nReac
    out, t, dt, st, tape = ob.record(o, tadv, state, [1e-18, 1e-8], tol_time, 2048)
    assert np.all(st == 0) and np.all(t == 300.0)
    assert np.allclose(tape.dt.sum(axis=1), 300.0, rtol=1e-12, atol=0)
    y = out[:, 3:3 + m]
    np.testing.assert_allclose(ob.replay(o, tadv, state, [1e-18, 1e-8], tape), y, rtol=0, atol=0)
    tg = [2, 11, 30]
    lam = np.zeros((2, m))
    lam[:, tg] = 2 * np.log(y[:, tg]) / y[:, tg]
    gx, gk = ob.adjoint(o, tadv, state, [1e-18, 1e-8], tape, lam)
    rng = np.random.default_rng(2)
    dx0, dth = rng.normal(size=(2, m)) * state[:, 3:3 + m], rng.normal(size=(2, R))
    dy = ob.tangent(o, tadv, state, [1e-18, 1e-8], tape, dx0, dth)
    lhs, rhs = (lam * dy).sum(axis=1), (gx * dx0).sum(axis=1) + (gk * dth).sum(axis=1)
    assert (np.abs(lhs - rhs) / np.abs(lhs)).max() < 1e-10
    h = 1e-6
    for r in (4, 90):
        ks = np.ones(R)
        ks[r] = np.exp(h)
        lp = (np.log(ob.replay(o, tadv, state, [1e-18, 1e-8], tape, ks)[:, tg]) ** 2).sum(axis=1)
        ks[r] = np.exp(-h)
        lm = (np.log(ob.replay(o, tadv, state, [1e-18, 1e-8], tape, ks)[:, tg]) ** 2).sum(axis=1)
        assert np.abs((lp - lm) / (2 * h) - gk[:, r]).max() <= 1e-5 * np.abs(gk[:, r]).max() + 1e-12
