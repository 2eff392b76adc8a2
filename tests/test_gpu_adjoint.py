"""Discrete adjoint of the plain FP64 form on the GPU (tchem_gb_time_advance_record /
tchem_gb_adjoint) against the oracle's dense restatement on the same recorded step sequence,
against the oracle's forward sensitivities (dot-product test) and against central finite
differences (h = 1e-6) of the recorded-step replay; plus the torch.autograd face."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import rel_error  # noqa: E402
from oracle import Oracle  # noqa: E402
from oracle import binding as ob  # noqa: E402
from tchem_gb import AtmosphericChemistry, KineticModel, tadv_to_device, time_advance_array  # noqa: E402
from tchem_gb import adjoint as adj  # noqa: E402
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states  # noqa: E402

pytestmark = pytest.mark.gpu

TN = [1e-18, 1e-8]
CAP = 4096


@pytest.fixture(scope="module")
def km():
    return KineticModel.from_string(mechanism_yaml(MechanismSpec()))


def case(km, B, horizon=1800.0, seed=11):
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=horizon, dt=1e-10, dtmin=1e-10, dtmax=horizon, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    tol_time = np.tile([1e-12, 1e-6], (km.n_active, 1))
    return state, tadv, tol_time


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def gpu_record(km, state, tadv, tol_time, cap=CAP, k_scale=None):
    B = state.shape[0]
    d_state = dev(state)
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device="cuda")
    dt = torch.zeros_like(t)
    stats = torch.zeros(B, 8, dtype=torch.int32, device="cuda")
    tape = adj.new_tape(B, km.n_active, cap)
    st = adj.record(km, dev(TN), dev(tol_time), tadv_to_device(tadv), d_state, t, dt, out, tape,
                    k_scale=None if k_scale is None else dev(k_scale), stats=stats)
    torch.cuda.synchronize()
    return out.cpu().numpy(), st.cpu().numpy(), stats.cpu().numpy(), tape, t.cpu().numpy()


def loss_and_seed(y, tg, ref):
    L = (np.log(y[:, tg] / ref) ** 2).sum(axis=1)
    lam = np.zeros_like(y)
    lam[:, tg] = 2 * np.log(y[:, tg] / ref) / y[:, tg]
    return L, lam


def host_tape(tape):
    return ob.Tape(tape.dt.cpu().numpy(), tape.nsteps.cpu().numpy())


def test_record_is_the_plain_run_and_checkpoints_the_trajectory(km):
    state, tadv, tol_time = case(km, 32, horizon=600.0)
    out, st, stats, tape, t = gpu_record(km, state, tadv, tol_time)
    m = km.n_active
    assert np.all(st == 0) and np.all(t == 600.0)
    # the same kernel path as tchem_gb_time_advance: identical end states and step counts
    d_state = dev(state)
    ref_out = torch.empty_like(d_state)
    tt = torch.zeros(32, dtype=torch.float64, device="cuda")
    dd = torch.zeros_like(tt)
    ref_stats = torch.zeros(32, 8, dtype=torch.int32, device="cuda")
    AtmosphericChemistry.runDeviceBatch(dev(TN), dev(tol_time), None, tadv_to_device(tadv), d_state, tt, dd, ref_out,
                                        km, stats=ref_stats)
    np.testing.assert_array_equal(out, ref_out.cpu().numpy())
    ns = tape.nsteps.cpu().numpy()
    np.testing.assert_array_equal(ns, ref_stats.cpu().numpy()[:, 0])
    dts = tape.dt.cpu().numpy()
    for b in range(32):
        assert abs(dts[b, :ns[b]].sum() - 600.0) < 1e-9 * 600.0
        assert np.all(dts[b, ns[b]:] == 0.0)
    np.testing.assert_array_equal(tape.ckpt.cpu().numpy()[:, 0, :], state[:, 3:3 + m])
    # the oracle's recorded run of the same inputs takes the same number of steps on most samples
    ref = ob.record(Oracle([km]), tadv, state, TN, tol_time, CAP)
    assert np.mean(ref[4].nsteps == ns) >= 0.9


def test_tape_full_is_reported(km):
    state, tadv, tol_time = case(km, 4, horizon=600.0)
    _, st, _, tape, t = gpu_record(km, state, tadv, tol_time, cap=8)
    assert np.all(st == 7) and np.all(t == 600.0)


@pytest.fixture(scope="module")
def adj_case(km):
    B = 64
    state, tadv, tol_time = case(km, B)
    out, st, _, tape, _ = gpu_record(km, state, tadv, tol_time)
    assert np.all(st == 0)
    m = km.n_active
    y = out[:, 3:3 + m]
    rng = np.random.default_rng(5)
    tg = rng.choice(m, 5, replace=False)
    ref = y[:, tg] * np.exp(rng.normal(0.0, 0.1, size=(B, 5)))
    _, lam = loss_and_seed(y, tg, ref)
    gx, gk, ast = adj.adjoint(km, dev(TN), tadv_to_device(tadv), dev(state), tape, dev(lam))
    torch.cuda.synchronize()
    assert int((ast != 0).sum()) == 0
    return dict(state=state, tadv=tadv, tol_time=tol_time, tape=tape, y=y, tg=tg, ref=ref, lam=lam,
                gx=gx.cpu().numpy(), gk=gk.cpu().numpy())


def test_adjoint_matches_oracle_on_the_same_steps(km, adj_case):
    """The oracle replays the GPU's step sequence with its own Newton solves; the two sets of
    linearisation points agree to the Newton tolerance (rtol 1e-8), so the gradients agree to
    about 1e-7 relative on a few samples and to rounding on the rest."""
    c = adj_case
    gx, gk = ob.adjoint(Oracle([km]), c["tadv"], c["state"], TN, host_tape(c["tape"]), c["lam"])
    sx = np.abs(gx).max(axis=1, keepdims=True) + 1e-300
    sk = np.abs(gk).max(axis=1, keepdims=True) + 1e-300
    ex, ek = np.abs(c["gx"] - gx) / sx, np.abs(c["gk"] - gk) / sk
    assert ex.max() <= 1e-6 and ek.max() <= 1e-6
    assert np.median(ex.max(axis=1)) <= 1e-10 and np.median(ek.max(axis=1)) <= 1e-10


def test_adjoint_dot_product_with_forward_sensitivities(km, adj_case):
    c = adj_case
    B, m, R = c["state"].shape[0], km.n_active, km.nReac
    rng = np.random.default_rng(9)
    dx0 = rng.normal(size=(B, m)) * c["state"][:, 3:3 + m]
    dth = rng.normal(size=(B, R))
    dy = ob.tangent(Oracle([km]), c["tadv"], c["state"], TN, host_tape(c["tape"]), dx0, dth)
    lhs = (c["lam"] * dy).sum(axis=1)
    rhs = (c["gx"] * dx0).sum(axis=1) + (c["gk"] * dth).sum(axis=1)
    e = np.abs(lhs - rhs) / np.maximum(np.abs(lhs), 1e-300)
    assert e.max() <= 1e-6 and np.median(e) <= 1e-10  # linearisation points agree to the Newton tolerance


def test_adjoint_central_finite_differences(km, adj_case):
    """Central differences (h = 1e-6) of the loss through the recorded steps, 64 samples."""
    c = adj_case
    o = Oracle([km])
    R = km.nReac
    h = 1e-6
    tape = host_tape(c["tape"])

    def L(k_scale=None, state=None):
        y = ob.replay(o, c["tadv"], c["state"] if state is None else state, TN, tape, k_scale)
        return loss_and_seed(y, c["tg"], c["ref"])[0]

    for r in (3, 17, 40, 101, 150):
        ks = np.ones(R)
        ks[r] = np.exp(h)
        lp = L(k_scale=ks)
        ks[r] = np.exp(-h)
        fd = (lp - L(k_scale=ks)) / (2 * h)
        g = c["gk"][:, r]
        assert np.abs(fd - g).max() <= 1e-5 * np.abs(g).max() + 1e-12, r
    for k in (0, 7, 30):
        sp, sm = c["state"].copy(), c["state"].copy()
        sp[:, 3 + k] *= np.exp(h)
        sm[:, 3 + k] *= np.exp(-h)
        fd = (L(state=sp) - L(state=sm)) / (2 * h)
        g = c["gx"][:, k] * c["state"][:, 3 + k]
        assert np.abs(fd - g).max() <= 1e-5 * np.abs(g).max() + 1e-12, k


def test_autograd_function(km):
    B = 8
    state, tadv, tol_time = case(km, B, horizon=300.0, seed=21)
    m, R = km.n_active, km.nReac
    log_x0 = dev(np.log(state[:, 3:3 + m])).requires_grad_(True)
    log_k = torch.zeros(R, dtype=torch.float64, device="cuda", requires_grad=True)
    args = (km, dev(state), tadv_to_device(tadv), dev(TN), dev(tol_time), CAP)
    y = adj.BoxModelSolve.apply(log_x0, log_k, *args)
    tg = [1, 4, 9]
    L = (torch.log(y[:, tg]) ** 2).sum()
    L.backward()
    assert log_x0.grad.shape == (B, m) and log_k.grad.shape == (R,)
    # against central differences of the (adaptive) forward in two rate parameters
    h = 1e-6
    for r in (5, 60):
        with torch.no_grad():
            e = torch.zeros(R, dtype=torch.float64, device="cuda")
            e[r] = h
            lp = (torch.log(adj.BoxModelSolve.apply(log_x0, log_k + e, *args)[:, tg]) ** 2).sum()
            lm = (torch.log(adj.BoxModelSolve.apply(log_x0, log_k - e, *args)[:, tg]) ** 2).sum()
        fd = float((lp - lm) / (2 * h))
        g = float(log_k.grad[r])
        assert abs(fd - g) <= 1e-3 * max(abs(g), 1e-6), (r, fd, g)
