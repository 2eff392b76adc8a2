"""GPU checks of the tensor-core code: the building blocks (tchem_gb_tc_tile_update_tf32,
tchem_gb_tc_lu_factor_tf32) and the large-mechanism time advance built on the same tcgen05 pieces.

* one 128 x 64 tile update against the FP64 product (TF32 operands: relative error ~1e-3);
* four 300 x 300 Newton-like matrices factored in place against the oracle's restatement in the
  same order (oracle.lu_factor_blocked, TF32 operands): equal pivots, factors within the TF32
  bound, P A = L U to the TF32 level; and the device error word clear;
* the time advance of the 300-species / 1000-reaction and a 160-species mechanism in the
  tensor-core form against the FP64 oracle, and its host loop against one call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lu_factor_blocked  # noqa: E402
from tchem_gb import _capi  # noqa: E402
from tchem_gb.tensor_core import lu_factor_tf32, tile_update_tf32  # noqa: E402

pytestmark = pytest.mark.gpu


def device_error() -> int:
    err = C.c_int32(0)
    _capi.check(_capi.lib().tchem_gb_device_error(None, None, C.byref(err)), "tchem_gb_device_error")
    return err.value


def test_tile_update_against_fp64_product():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((1, 128, 32)).astype(np.float32)
    b = rng.standard_normal((1, 32, 64)).astype(np.float32)
    d = rng.standard_normal((1, 128, 64)).astype(np.float32)
    ref = d.astype(np.float64) - a.astype(np.float64) @ b.astype(np.float64)
    D = torch.from_numpy(d).cuda()
    tile_update_tf32(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), D)
    torch.cuda.synchronize()
    assert device_error() == 0
    out = D.cpu().numpy().astype(np.float64)
    assert np.abs(out - ref).max() / np.abs(ref).max() <= 1e-2


def test_lu_against_blocked_restatement():
    rng = np.random.default_rng(3)
    n, lda, B = 300, 304, 4
    mats = [(np.eye(n) - 0.05 * rng.standard_normal((n, n))).astype(np.float32) for _ in range(B)]
    A = np.zeros((B, n, lda), np.float32)
    for b in range(B):
        A[b, :, :n] = mats[b]
    dA = torch.from_numpy(A).cuda()
    piv, info = lu_factor_tf32(dA)
    torch.cuda.synchronize()
    assert device_error() == 0
    assert np.all(info.cpu().numpy() == 0)
    lu = dA.cpu().numpy()[:, :, :n]
    pv = piv.cpu().numpy()
    for b in range(B):
        ref_lu, ref_piv = lu_factor_blocked(mats[b], keep=10)
        np.testing.assert_array_equal(pv[b], ref_piv)
        assert np.abs(lu[b] - ref_lu).max() <= 1e-3 * np.abs(ref_lu).max()
        L = np.tril(lu[b].astype(np.float64), -1) + np.eye(n)
        U = np.triu(lu[b].astype(np.float64))
        pa = mats[b].astype(np.float64).copy()
        for k in range(n):
            pa[[k, pv[b, k]]] = pa[[pv[b, k], k]]
        assert np.abs(pa - L @ U).max() / np.abs(mats[b]).max() <= 5e-4


# --- the tensor-core time advance (mechanisms of 129 to 320 active species) ------------------------

def _large_case(n_species, n_reactions, B, horizon, seed):
    from tchem_gb import KineticModel, time_advance_array
    from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=n_species, n_reactions=n_reactions,
                                                               seed=20251205)))
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=horizon, dt=1e-10, dtmin=1e-10, dtmax=horizon, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=10_000_000)
    tol_time = np.tile([1e-12, 1e-6], (km.n_active, 1))
    return km, state, tadv, tol_time


def _advance(km, tadv, state, tol_time, form, stats=True):
    from tchem_gb import AtmosphericChemistry, tadv_to_device
    B = state.shape[0]
    d_state = torch.as_tensor(state).cuda()
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device="cuda")
    dt = torch.zeros_like(t)
    st = torch.full((B,), -7, dtype=torch.int32, device="cuda")
    s = torch.zeros(B, 8, dtype=torch.int32, device="cuda") if stats else None
    AtmosphericChemistry.runDeviceBatch(torch.tensor([1e-18, 1e-8], dtype=torch.float64, device="cuda"),
                                        torch.as_tensor(tol_time).cuda(), None, tadv_to_device(tadv), d_state, t, dt,
                                        out, km, status=st, stats=s, form=form)
    torch.cuda.synchronize()
    assert device_error() == 0
    return out.cpu().numpy(), t.cpu().numpy(), dt.cpu().numpy(), st.cpu().numpy(), (s.cpu().numpy() if stats else None)


@pytest.mark.parametrize("n_species,n_reactions,B,horizon", [(300, 1000, 6, 10.0), (160, 480, 16, 60.0)])
def test_tensor_core_time_advance_matches_fp64_oracle(n_species, n_reactions, B, horizon):
    """The large-mechanism form (full Newton; FP32 Newton matrix factored by the blocked LU whose
    trailing updates run as TF32 tcgen05 MMAs; FP64 residual refinement of every Newton solve)
    against the FP64 oracle: every species within 1e-6 relative (floored at atol_time), the same
    step counts within a few percent."""
    from oracle import Oracle
    km, state, tadv, tol_time = _large_case(n_species, n_reactions, B, horizon, seed=71)
    m = km.n_active
    ref = Oracle([km]).time_advance(tadv, state, [1e-18, 1e-8], tol_time)
    out, t, dt, st, stats = _advance(km, tadv, state, tol_time, "mixed")
    assert np.all(st == 0) and np.all(ref[3] == 0)
    assert np.all(t == horizon)
    err = np.abs(out[:, 3:3 + m] - ref[0][:, 3:3 + m]) / np.maximum(np.abs(ref[0][:, 3:3 + m]), 1e-12)
    assert err.max() <= 1e-6, err.max()
    np.testing.assert_array_equal(out[:, :3], state[:, :3])
    np.testing.assert_array_equal(out[:, 3 + m:], state[:, 3 + m:])
    assert np.all(stats[:, 4] > 0) and np.all(stats[:, 4] == stats[:, 7])  # one factorization per Jacobian
    assert abs(stats[:, 0].mean() / ref[4]["n_steps"].mean() - 1.0) < 0.03


def test_tensor_core_time_advance_host_loop_reproduces_one_call():
    """The reference's host loop over the tensor-core form (calls of at most 25 steps with the
    carry-over of t and dt) gives exactly the one-call trajectory: the form carries nothing across
    steps but t, dt and the state."""
    from tchem_gb import AtmosphericChemistry, tadv_to_device
    km, state, tadv, tol_time = _large_case(160, 480, 8, 5.0, seed=72)
    one, t1, *_ = _advance(km, tadv, state, tol_time, "mixed", stats=False)
    d_tadv = tadv_to_device(tadv)
    d_state = torch.as_tensor(state).cuda()
    d_t = torch.zeros(8, dtype=torch.float64, device="cuda")
    d_dt = torch.zeros_like(d_t)
    AtmosphericChemistry.carry_over(d_tadv, d_t, torch.as_tensor(tadv["dt"]).cuda(), 25)
    for _ in range(400):
        AtmosphericChemistry.runDeviceBatch(torch.tensor([1e-18, 1e-8], dtype=torch.float64, device="cuda"),
                                            torch.as_tensor(tol_time).cuda(), None, d_tadv, d_state, d_t, d_dt,
                                            d_state, km, form="mixed")
        AtmosphericChemistry.carry_over(d_tadv, d_t, d_dt, 25)
        if bool((d_t >= 5.0).all()):
            break
    np.testing.assert_array_equal(d_state.cpu().numpy(), one)
    np.testing.assert_array_equal(d_t.cpu().numpy(), t1)
