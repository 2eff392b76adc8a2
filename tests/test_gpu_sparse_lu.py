"""The sparse-LU shape of the full-Newton FP32 form (one warp per sample, static-order sparse LU of
I - c J, one FP64 refinement sweep per solve) against the FP64 oracle on the GPU: the 51-species
benchmark mechanism over the full 3600 s horizon and a 120-species mechanism (four rows per lane),
plus the oracle's emulation of the same factorization."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_error
from oracle import Oracle
from oracle.binding import load as load_oracle
from tchem_gb import AtmosphericChemistry, KineticModel, _capi, time_advance_array, tadv_to_device
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ATOL_TIME = 1e-12
TN = [1e-18, 1e-8]


def _dev(a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


def case(km, B, seed, horizon):
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=horizon, dt=1e-10, dtmin=1e-10, dtmax=horizon, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    tol_time = np.tile([ATOL_TIME, 1e-6], (km.n_active, 1))
    return state, tadv, tol_time


def sparse_advance(km, state, tadv, tol_time):
    B = state.shape[0]
    d_state = _dev(state)
    d_out = d_state.clone()
    d_t = torch.zeros(B, dtype=torch.float64, device="cuda")
    d_dt = torch.zeros_like(d_t)
    d_st = torch.full((B,), -7, dtype=torch.int32, device="cuda")
    d_stats = torch.zeros(B, 8, dtype=torch.int32, device="cuda")
    AtmosphericChemistry.runDeviceBatch(_dev(TN, torch.float64), _dev(tol_time, torch.float64), None,
                                        tadv_to_device(tadv), d_state, d_t, d_dt, d_out, km, status=d_st,
                                        stats=d_stats, form="mixed", threads_per_sample=32)
    torch.cuda.synchronize()
    assert AtmosphericChemistry.device_error() == 0
    return d_out.cpu().numpy(), d_t.cpu().numpy(), d_st.cpu().numpy(), d_stats.cpu().numpy()


def order_of(km):
    info = np.zeros(12, dtype=np.int32)
    assert _capi.lib().tchem_gb_mech_sparse_lu(km.handle, info.ctypes.data, None, 0) == 0
    prog = np.zeros(int(info[3]), dtype=np.int32)
    _capi.lib().tchem_gb_mech_sparse_lu(km.handle, info.ctypes.data, prog.ctypes.data, len(prog))
    pos = prog[info[5]:info[5] + info[0]]
    return np.ascontiguousarray(np.argsort(pos).astype(np.int32))


@pytest.mark.parametrize("m,R,seed,B,horizon", [(51, 156, 20251203, 256, 3600.0), (120, 330, 4242, 16, 600.0)])
def test_sparse_shape_matches_fp64_oracle(m, R, seed, B, horizon):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=m, n_reactions=R, seed=seed)))
    state, tadv, tol_time = case(km, B, 11, horizon)
    ref = Oracle([km]).time_advance(tadv, state, TN, tol_time)
    out, t, st, stats = sparse_advance(km, state, tadv, tol_time)
    assert np.all(st == 0) and np.all(t == horizon)
    err = rel_error(out[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL_TIME)
    assert err.max() <= 1e-7, (err.max(), int(err.argmax()))
    # full Newton: one factorization per Newton iteration, the oracle's work counts
    np.testing.assert_array_equal(stats[:, 4], stats[:, 3])
    assert abs(stats[:, 0].mean() / ref[4]["n_steps"].mean() - 1.0) < 0.01
    assert abs(stats[:, 3].mean() / ref[4]["n_newton_iter"].mean() - 1.0) < 0.01


def test_sparse_shape_follows_the_oracle_emulation():
    """Against the oracle's FP32 factorization in the same static order without pivoting (one
    refinement sweep): the same arithmetic up to FMA contraction and summation order."""
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    state, tadv, tol_time = case(km, 64, 12, 600.0)
    L = load_oracle()
    order = order_of(km)
    assert L.oracle_set_lu_static_order(len(order), order.ctypes.data) == 0
    try:
        ref = Oracle([km]).time_advance(tadv, state, TN, tol_time, lu_fp32=2)
    finally:
        L.oracle_set_lu_static_order(0, None)
    out, t, st, stats = sparse_advance(km, state, tadv, tol_time)
    assert np.all(st == 0)
    m = km.n_active
    err = rel_error(out[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL_TIME)
    assert err.max() <= 1e-7, (err.max(), int(err.argmax()))
    assert np.mean(stats[:, 0] == ref[4]["n_steps"]) >= 0.95
