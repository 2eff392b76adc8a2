"""tchem_gb_time_advance_noalloc: the time advance for callers that may not allocate device memory
(a host model whose device memory all comes from its own pool, or a loop that cannot afford the
device synchronisation of cudaMalloc / cudaFree). It keeps its scratch in a fixed array inside the
library. Checked through the C ABI against tchem_gb_time_advance on the same inputs, on two calls
in a row (one mechanism, and two mechanism structures whose per-group sample lists live in the
fixed scratch), with the device's free memory unchanged across each call; plus its rejections
(tables not yet on the device; more scratch than it holds) and an unsupported mechanism, which
both entry points refuse with the same code.

This file sorts last so that a run stopping at the first failure has run every other test first;
it also passes alone in a fresh process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tchem_gb import KineticModel, tadv_to_device, time_advance_array  # noqa: E402
from tchem_gb import _capi  # noqa: E402
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states  # noqa: E402

pytestmark = pytest.mark.gpu

vp = C.c_void_p


def _lib():
    L = _capi.lib()
    f = L.tchem_gb_time_advance_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                  C.POINTER(_capi.AdvanceOpts), vp]
    return L


def _p(t):
    return vp(0) if t is None else vp(t.data_ptr())


def _handles(mechs):
    return (vp * len(mechs))(*[m.handle.value for m in mechs])


def _inputs(km, B, seed):
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=600.0, dt=1e-10, dtmin=1e-10, dtmax=600.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    tol_time = np.tile([1e-12, 1e-6], (km.n_active, 1))
    return (torch.as_tensor(state).cuda(), tadv_to_device(tadv),
            torch.tensor([1e-18, 1e-8], dtype=torch.float64, device="cuda"), torch.as_tensor(tol_time).cuda())


def _run(L, fn, km, d_state, d_tadv, d_tn, d_tt, form, mos=None):
    mechs = km if isinstance(km, list) else [km]
    B = d_state.shape[0]
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device="cuda")
    dt = torch.zeros_like(t)
    st = torch.full((B,), -1, dtype=torch.int32, device="cuda")
    o = _capi.AdvanceOpts()
    o.form = form
    stream = vp(torch.cuda.current_stream().cuda_stream)
    args = [_handles(mechs), len(mechs), _p(mos), B, _p(d_tn), _p(d_tt), None, _p(d_tadv), _p(d_state), _p(t), _p(dt),
            _p(out), _p(st), None]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    if fn == "noalloc":
        rc = L.tchem_gb_time_advance_noalloc(*args, C.byref(o), stream)
    else:
        rc = L.tchem_gb_time_advance(*args, None, C.c_size_t(0), C.byref(o), stream)
    torch.cuda.synchronize()
    if fn == "noalloc":  # nothing allocated: the device's free memory is unchanged across the call
        assert torch.cuda.mem_get_info()[0] == free0
    return rc, out.cpu().numpy(), t.cpu().numpy(), dt.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("form", [2, 0])  # simplified-Newton mixed form, plain FP64
def test_noalloc_matches_time_advance_on_two_calls_in_a_row(form):
    L = _lib()
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    d_state, d_tadv, d_tn, d_tt = _inputs(km, 48, seed=77)
    # before set-up the mechanism has no tables on the device: rejected, nothing launched
    rc, *_ = _run(L, "noalloc", km, d_state, d_tadv, d_tn, d_tt, form)
    assert rc == 1 and b"set-up" in L.tchem_gb_last_error()
    # set-up (allocation allowed here): put the tables on the device
    o = _capi.AdvanceOpts()
    o.form = form
    assert L.tchem_gb_workspace_bytes(_handles([km]), 1, 48, C.byref(o)) > 0
    m = km.n_active
    for call in range(2):
        # the regular entry point first: its first launch also loads the kernel's code (CUDA loads
        # modules lazily), which is set-up work, not the no-alloc call's
        rc2, ref, t2, dt2, st2 = _run(L, "regular", km, d_state, d_tadv, d_tn, d_tt, form)
        assert rc2 == 0
        rc, out, t, dt, st = _run(L, "noalloc", km, d_state, d_tadv, d_tn, d_tt, form)
        assert rc == 0, L.tchem_gb_last_error()
        np.testing.assert_array_equal(st, st2)
        assert np.all(st == 0) and np.all(t == 600.0)
        # the same kernel on the same inputs: identical results
        np.testing.assert_array_equal(out[:, 3:3 + m], ref[:, 3:3 + m])
        np.testing.assert_array_equal(t, t2)
        np.testing.assert_array_equal(dt, dt2)


def test_noalloc_two_mechanism_structures_on_two_calls_in_a_row():
    """Samples of two mechanism structures: the per-group sample lists and counts live in the fixed
    scratch and are cleared by each call, so stale counts of the first call would show in the
    second."""
    L = _lib()
    big = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    small = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=20, n_reactions=60, seed=99)))
    mechs = [big, small]
    B = 1000
    rng = np.random.default_rng(3)
    mos = rng.integers(0, 2, B).astype(np.int32)
    state = np.zeros((B, big.state_dim))
    s_big = sample_states(B, big.n_active, seed=31)
    s_small = sample_states(B, small.n_active, seed=32)
    state[:, :s_big.shape[1]] = s_big
    state[mos == 1, :s_small.shape[1]] = s_small[mos == 1]
    state[mos == 1, s_small.shape[1]:] = 0.0
    tadv = time_advance_array(B, tend=300.0, dt=1e-10, dtmin=1e-10, dtmax=300.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    d_state, d_tadv = torch.as_tensor(state).cuda(), tadv_to_device(tadv)
    d_tn = torch.tensor([1e-18, 1e-8], dtype=torch.float64, device="cuda")
    d_tt = torch.as_tensor(np.tile([1e-12, 1e-6], (big.n_active, 1))).cuda()
    d_mos = torch.as_tensor(mos).cuda()
    o = _capi.AdvanceOpts()
    o.form = 2
    need = L.tchem_gb_workspace_bytes(_handles(mechs), 2, B, C.byref(o))  # set-up: tables on the device
    assert 0 < need <= (1 << 20)
    for call in range(2):
        rc2, ref, t2, dt2, st2 = _run(L, "regular", mechs, d_state, d_tadv, d_tn, d_tt, 2, mos=d_mos)
        assert rc2 == 0
        rc, out, t, dt, st = _run(L, "noalloc", mechs, d_state, d_tadv, d_tn, d_tt, 2, mos=d_mos)
        assert rc == 0, L.tchem_gb_last_error()
        assert np.all(st == 0) and np.all(t == 300.0), call
        np.testing.assert_array_equal(st, st2)
        np.testing.assert_array_equal(out, ref)
        np.testing.assert_array_equal(dt, dt2)


def test_noalloc_refuses_an_unsupported_mechanism_like_time_advance():
    """A mechanism outside the box-model path (JPL rate types): both entry points return
    TCHEM_GB_ERR_UNSUPPORTED."""
    from pathlib import Path
    L = _lib()
    km = KineticModel.from_file(Path(__file__).resolve().parent / "golden" / "mechanisms" / "uci.yaml")
    d_state, d_tadv, d_tn, d_tt = _inputs(km, 4, seed=5)
    o = _capi.AdvanceOpts()
    o.form = 0
    assert L.tchem_gb_workspace_bytes(_handles([km]), 1, 4, C.byref(o)) == 0  # refused, tables uploaded
    rc_regular, *_ = _run(L, "regular", km, d_state, d_tadv, d_tn, d_tt, 0)
    rc_noalloc, *_ = _run(L, "noalloc", km, d_state, d_tadv, d_tn, d_tt, 0)
    assert rc_regular == 4 and rc_noalloc == 4


def test_noalloc_rejects_more_scratch_than_it_holds():
    L = _lib()
    day = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    small = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=20, n_reactions=60, seed=99)))
    mechs = [day, small]
    B = 200_000  # two structure groups: 4 bytes per sample and group of sample lists > 1 MiB
    o = _capi.AdvanceOpts()
    o.form = 2
    need = L.tchem_gb_workspace_bytes(_handles(mechs), 2, B, C.byref(o))
    assert need > (1 << 20)
    # full-size, valid inputs (a short horizon), so that nothing could read out of bounds even if
    # the call went ahead
    state = np.zeros((B, day.state_dim))
    state[:, :3 + day.nSpec] = sample_states(B, day.n_active, seed=5)
    tadv = time_advance_array(B, tend=1e-6, dt=1e-10, dtmin=1e-10, dtmax=1e-6, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    d_state = torch.as_tensor(state).cuda()
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device="cuda")
    dt = torch.zeros_like(t)
    st = torch.full((B,), -1, dtype=torch.int32, device="cuda")
    mos = torch.zeros(B, dtype=torch.int32, device="cuda")
    d_tn = torch.tensor([1e-18, 1e-8], dtype=torch.float64, device="cuda")
    d_tt = torch.as_tensor(np.tile([1e-12, 1e-6], (day.n_active, 1))).cuda()
    d_tadv = tadv_to_device(tadv)
    rc = L.tchem_gb_time_advance_noalloc(_handles(mechs), 2, _p(mos), B, _p(d_tn), _p(d_tt), None,
                                         _p(d_tadv), _p(d_state), _p(t), _p(dt), _p(out), _p(st), None,
                                         C.byref(o), vp(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rc == 1
    assert b"bytes of scratch" in L.tchem_gb_last_error()
    assert int((st != -1).sum()) == 0  # nothing ran
