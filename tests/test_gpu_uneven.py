"""Uneven batches on the GPU: the simplified form's multi-warp sample shapes (64 and 128 threads
per sample), a 120-species / 330-reaction mechanism, the autotuner and a CUDA-graph replay of a
mixed batch (51- and 120-species mechanisms, day and night variants, three horizons), each
against the CPU oracle."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import rel_error  # noqa: E402
from oracle import Oracle  # noqa: E402
from tchem_gb import AtmosphericChemistry, KineticModel, tadv_to_device, time_advance_array  # noqa: E402
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states  # noqa: E402

pytestmark = pytest.mark.gpu

ATOL = 1e-12
TN = [1e-18, 1e-8]
SPEC_120 = MechanismSpec(n_species=120, n_reactions=330, seed=20251204)


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def run(km, state, tadv, tol_time, form, tps=0, mos=None):
    B = state.shape[0]
    d_state = dev(state)
    out = torch.empty_like(d_state)
    t = dev(tadv["tbeg"])
    dt = torch.zeros_like(t)
    st = AtmosphericChemistry.runDeviceBatch(dev(TN), dev(tol_time), None, tadv_to_device(tadv), d_state, t, dt, out,
                                             km, form=form, threads_per_sample=tps,
                                             mech_of_sample=None if mos is None else dev(mos, torch.int32))
    torch.cuda.synchronize()
    return out.cpu().numpy(), st.cpu().numpy(), t.cpu().numpy()


def case(km, B, horizon, seed):
    state = sample_states(B, km.n_active, seed=seed)
    tadv = time_advance_array(B, tend=horizon, dt=1e-10, dtmin=1e-10, dtmax=horizon, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    return state, tadv, np.tile([ATOL, 1e-6], (km.n_active, 1))


@pytest.mark.parametrize("tps", [64, 128])
def test_multi_warp_shapes_match_oracle_and_one_warp(tps):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    state, tadv, tol_time = case(km, 40, 1800.0, seed=41)
    m = km.n_active
    ref = Oracle([km]).time_advance(tadv, state, TN, tol_time)
    out, st, t = run(km, state, tadv, tol_time, "simplified", tps)
    one, st1, _ = run(km, state, tadv, tol_time, "simplified", 32)
    assert np.all(st == 0) and np.all(t == 1800.0)
    assert rel_error(out[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL).max() <= 1e-6
    # same algorithm, different thread mapping: same decisions, end states to rounding
    assert rel_error(out[:, 3:3 + m], one[:, 3:3 + m], ATOL).max() <= 1e-9


def test_120_species_mechanism_plain_and_simplified():
    km = KineticModel.from_string(mechanism_yaml(SPEC_120))
    assert km.n_active == 120
    state, tadv, tol_time = case(km, 16, 600.0, seed=43)
    m = km.n_active
    ref = Oracle([km]).time_advance(tadv, state, TN, tol_time)
    assert np.all(ref[3] == 0)
    plain, st_p, _ = run(km, state, tadv, tol_time, "plain")
    simp, st_s, t = run(km, state, tadv, tol_time, "simplified")
    assert np.all(st_p == 0) and np.all(st_s == 0) and np.all(t == 600.0)
    assert rel_error(plain[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL).max() <= 1e-8
    assert rel_error(simp[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL).max() <= 1e-6
    # the 51-or-fewer-species shapes do not fit: only 128 threads per sample is offered
    with pytest.raises(Exception):
        run(km, state[:2], tadv[:2], tol_time, "simplified", 32)


def uneven_batch(B, seed=3):
    """75 % on the 51-species mechanism, 25 % on the 120-species one; half night (photolysis off);
    horizons drawn from {600, 1800, 3600} s."""
    mechs = [KineticModel.from_string(mechanism_yaml(MechanismSpec())),
             KineticModel.from_string(mechanism_yaml(MechanismSpec(), night=True)),
             KineticModel.from_string(mechanism_yaml(SPEC_120)),
             KineticModel.from_string(mechanism_yaml(SPEC_120, night=True))]
    rng = np.random.default_rng(seed)
    big = rng.random(B) < 0.25
    night = rng.random(B) < 0.5
    mos = (2 * big + night).astype(np.int32)
    dim = mechs[2].state_dim
    state = np.zeros((B, dim))
    s51 = sample_states(B, mechs[0].n_active, seed=seed + 1)
    s120 = sample_states(B, mechs[2].n_active, seed=seed + 2)
    for b in range(B):
        if big[b]:
            state[b] = s120[b]
        else:
            state[b, :s51.shape[1]] = s51[b]
    horizon = rng.choice([600.0, 1800.0, 3600.0], size=B)
    tadv = time_advance_array(B, tend=3600.0, dt=1e-10, dtmin=1e-10, dtmax=3600.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=1_000_000)
    tadv["tend"] = horizon
    tadv["dtmax"] = horizon
    tol_time = np.tile([ATOL, 1e-6], (mechs[2].n_active, 1))
    return mechs, state, tadv, tol_time, mos


def test_autotune_and_graph_replay_of_an_uneven_batch():
    mechs, state, tadv, tol_time, mos = uneven_batch(192)
    # autotune each structure on a probe of its own samples
    chosen = {}
    for k in (0, 2):
        sel = np.nonzero(mos == k)[0][:32]
        km = mechs[k]
        n = km.state_dim
        tps, times = AtmosphericChemistry.autotune(km, dev(TN), dev(tol_time[:km.n_active]),
                                                   tadv_to_device(tadv[sel]), dev(state[sel][:, :n]),
                                                   form="simplified")
        assert tps in times and times[tps] == min(times.values())
        chosen[k] = tps
        AtmosphericChemistry.set_threads_per_sample(mechs[k + 1], tps)  # the night variant shares the structure
    assert chosen[2] == 128
    B = state.shape[0]
    d_state, d_tt, d_tn = dev(state), dev(tol_time), dev(TN)
    d_tadv, d_mos = tadv_to_device(tadv), dev(mos, torch.int32)
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device="cuda")
    dt = torch.zeros_like(t)
    g, status = AtmosphericChemistry.capture(d_tn, d_tt, d_tadv, d_state, t, dt, out, mechs, mech_of_sample=d_mos,
                                             form="simplified")
    results = []
    for _ in range(2):
        out.fill_(0.0)
        g.replay()
        torch.cuda.synchronize()
        results.append((out.cpu().numpy().copy(), status.cpu().numpy().copy(), t.cpu().numpy().copy()))
    eager, st_e, _ = run(mechs, state, tadv, tol_time, "simplified", mos=mos)
    for o, st, tt in results:
        assert np.all(st == 0)
        np.testing.assert_array_equal(tt, tadv["tend"])
        np.testing.assert_array_equal(o, eager)
    # against the oracle on a subsample of each mechanism
    pick = np.concatenate([np.nonzero(mos == k)[0][:4] for k in range(4)])
    ref = Oracle(mechs).time_advance(tadv[pick], state[pick], TN, tol_time, mech_of_sample=mos[pick])
    for i, b in enumerate(pick):
        m = mechs[mos[b]].n_active
        assert rel_error(eager[b, 3:3 + m], ref[0][i, 3:3 + m], ATOL).max() <= 1e-6, b


def test_300_species_mechanism_plain_form():
    """The plain FP64 form takes any mechanism size (its Newton matrix moves to global memory when
    shared memory cannot hold it): a seeded 300-species / 1000-reaction mechanism, 2 samples over
    the first millisecond (one warp per sample on a global-memory matrix is slow at this size)."""
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=300, n_reactions=1000, seed=20251206)))
    state, tadv, tol_time = case(km, 2, 1e-3, seed=47)
    m = km.n_active
    ref = Oracle([km]).time_advance(tadv, state, TN, tol_time)
    out, st, t = run(km, state, tadv, tol_time, "plain")
    assert np.all(st == 0) and np.all(t == 1e-3) and np.all(ref[3] == 0)
    assert rel_error(out[:, 3:3 + m], ref[0][:, 3:3 + m], ATOL).max() <= 1e-8
