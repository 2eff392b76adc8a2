"""Numerics of a tensor-core factorization on the CPU (the design study for large mechanisms):
the oracle's FP32 factorizations computed as 32-column panels with the trailing update on TF32 or
BF16 operands and FP32 accumulation, inside the mixed forms' FP64 Newton residual and refinement.
On a seeded 120-species / 330-reaction mechanism the end states stay within 1e-7 (TF32) and 1e-6
(BF16) of the FP64 form with the same step counts; measured on the 300-species / 1000-reaction
mechanism over 10 s: TF32 2.2e-9 (simplified, +4.5 % Newton iterations) and 2.6e-10 (full Newton
with refinement), BF16 1.2e-9 (+9 %) and 3.1e-7."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_error
from oracle import Oracle, load
from tchem_gb import KineticModel, time_advance_array
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states


def test_round_mantissa_and_setting():
    L = load()
    assert L.oracle_set_lu_tile_bits(24) != 0 and L.oracle_set_lu_tile_bits(-1) != 0
    assert L.oracle_set_lu_tile_bits(0) == 0


@pytest.mark.parametrize("bits,simplified,bound", [(10, True, 1e-7), (7, True, 1e-6), (10, False, 1e-7),
                                                   (7, False, 1e-6)])
def test_tile_precision_against_fp64(bits, simplified, bound):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=120, n_reactions=330, seed=20251204)))
    m = km.n_active
    B = 4
    state = sample_states(B, m, seed=47)
    tadv = time_advance_array(B, tend=10.0, dt=1e-10, dtmin=1e-10, dtmax=10.0, max_num_newton_iterations=20,
                              num_time_iterations_per_interval=10**7)
    tol_time = np.tile([1e-12, 1e-6], (m, 1))
    o = Oracle([km])
    ref = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time)
    L = load()
    assert L.oracle_set_lu_tile_bits(bits) == 0
    try:
        r = o.time_advance(tadv, state, [1e-18, 1e-8], tol_time, lu_fp32=1 if simplified else 2, simplified=simplified)
    finally:
        L.oracle_set_lu_tile_bits(0)
    assert np.all(r[3] == 0)
    assert rel_error(r[0][:, 3:3 + m], ref[0][:, 3:3 + m], 1e-12).max() <= bound
    np.testing.assert_array_equal(r[4]["n_steps"], ref[4]["n_steps"])


@pytest.mark.parametrize("keep,bound", [(23, 2e-6), (10, 5e-4)])  # measured 3.4e-7, 7.7e-5
def test_blocked_lu_restatement_factors_the_matrix(keep, bound):
    """The oracle's factorization in the tensor-core LU's order (the reference a GPU run of
    tchem_gb_tc_lu_factor_tf32 is compared with): P A = L U to FP32 (keep = 23) or TF32-operand
    (keep = 10) accuracy on a 300 x 300 Newton-like matrix I - c J, with the pivots LAPACK's
    partial pivoting gives on the same matrix."""
    from oracle import lu_factor_blocked
    rng = np.random.default_rng(3)
    n = 300
    a = (np.eye(n) - 0.05 * rng.standard_normal((n, n))).astype(np.float32)
    lu, piv = lu_factor_blocked(a, keep)
    L = np.tril(lu.astype(np.float64), -1) + np.eye(n)
    U = np.triu(lu.astype(np.float64))
    pa = a.astype(np.float64).copy()
    for k in range(n):
        pa[[k, piv[k]]] = pa[[piv[k], k]]
    assert np.abs(pa - L @ U).max() / np.abs(a).max() <= bound
    import scipy.linalg
    _, piv_ref = scipy.linalg.lu_factor(a.astype(np.float64))
    assert np.mean(piv == piv_ref) > 0.95
