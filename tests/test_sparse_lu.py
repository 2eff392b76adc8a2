"""The static-order sparse LU of the full-Newton FP32 form's one-warp shape (csrc/sparse_lu.cpp,
Solver::factor_sp / solve_sp in csrc/kernels_mixed_impl.cuh), checked on the CPU.

The program the library builds per mechanism (tchem_gb_mech_sparse_lu) is run here with the
kernel's loops restated in numpy: assembly of I - c J into the filled pattern's entries, per
elimination step the pivot's reciprocal, the scaled column of L and the step's trailing updates,
then the column-oriented substitutions. In FP64 the result must equal numpy.linalg.solve to
rounding, which pins the ordering, the fill, the entry numbering and every index list before any
GPU run. The oracle's static-order FP32 factorization (oracle_set_lu_static_order) then shows that
this factorization, with one FP64 refinement sweep per solve, keeps the time advance within 1e-7 of
the FP64 oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import Oracle
from oracle.binding import load as load_oracle
from tchem_gb import KineticModel, _capi
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states

ERR_UNSUPPORTED = 4


def program(km):
    L = _capi.lib()
    info = np.zeros(12, dtype=np.int32)
    assert L.tchem_gb_mech_sparse_lu(km.handle, info.ctypes.data, None, 0) == 0
    prog = np.zeros(int(info[3]), dtype=np.int32)
    assert L.tchem_gb_mech_sparse_lu(km.handle, info.ctypes.data, prog.ctypes.data, len(prog)) == 0
    m, nnz, n_ops = (int(v) for v in info[:3])
    o = [int(v) for v in info[4:]]
    P = {"m": m, "nnz": nnz, "n_ops": n_ops,
         "diag": prog[o[0]:o[0] + m], "pos": prog[o[1]:o[1] + m],
         "lc_ptr": prog[o[2]:o[2] + m + 1], "uc_ptr": prog[o[4]:o[4] + m + 1], "up_ptr": prog[o[6]:o[6] + m + 1]}
    P["lc"] = prog[o[3]:o[3] + P["lc_ptr"][-1]]
    P["uc"] = prog[o[5]:o[5] + P["uc_ptr"][-1]]
    P["up"] = prog[o[7]:o[7] + 2 * n_ops].reshape(-1, 2)
    return P


def pattern_entries(P):
    """(position row, position col) of every entry, recovered from the lists."""
    m, nnz = P["m"], P["nnz"]
    rc = np.full((nnz, 2), -1)
    for k in range(m):
        rc[P["diag"][k]] = (k, k)
        for v in P["lc"][P["lc_ptr"][k]:P["lc_ptr"][k + 1]]:
            rc[v & 0xffff] = (v >> 16, k)
        for v in P["uc"][P["uc_ptr"][k]:P["uc_ptr"][k + 1]]:
            rc[v & 0xffff] = (v >> 16, k)
    return rc


def assemble(P, A, dtype):
    """The filled pattern's entries of A (species order) in position order."""
    rc = pattern_entries(P)
    order = np.argsort(P["pos"])
    return A[order[rc[:, 0]], order[rc[:, 1]]].astype(dtype)


def factor(P, a):
    dinv = np.zeros(P["m"], dtype=a.dtype)
    for k in range(P["m"]):
        piv = a[P["diag"][k]]
        assert piv != 0 and np.isfinite(piv)
        dinv[k] = a.dtype.type(1) / piv
        for v in P["lc"][P["lc_ptr"][k]:P["lc_ptr"][k + 1]]:
            a[v & 0xffff] *= dinv[k]
        for x, u in P["up"][P["up_ptr"][k]:P["up_ptr"][k + 1]]:
            a[x & 0xffff] -= a[(x >> 16) & 0xffff] * a[u]
    return dinv


def solve(P, a, dinv, g):
    m = P["m"]
    w = np.zeros(m, dtype=a.dtype)
    w[P["pos"]] = g
    for k in range(m):
        for v in P["lc"][P["lc_ptr"][k]:P["lc_ptr"][k + 1]]:
            w[v >> 16] -= a[v & 0xffff] * w[k]
    for k in range(m - 1, -1, -1):
        xk = w[k] * dinv[k]
        for v in P["uc"][P["uc_ptr"][k]:P["uc_ptr"][k + 1]]:
            w[v >> 16] -= a[v & 0xffff] * xk
        w[k] = xk
    return w[P["pos"]]


def newton_matrix(km, seed: int, c: float):
    o = Oracle([km])
    st = sample_states(1, km.n_active, seed=seed)[0]
    m = km.n_active
    J = o.jacobian(st[2], st[1], st[3:])[:m, :m]
    return np.eye(m) - c * J, J


@pytest.fixture(scope="module")
def mechs():
    return {51: KineticModel.from_string(mechanism_yaml(MechanismSpec())),
            120: KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=120, n_reactions=330, seed=4242)))}


@pytest.mark.parametrize("m", [51, 120])
def test_program_is_consistent(mechs, m):
    km = mechs[m]
    P = program(km)
    assert P["m"] == m
    assert sorted(P["pos"]) == list(range(m))
    rc = pattern_entries(P)
    assert (rc >= 0).all(), "every entry is a diagonal, L or U entry"
    # entries are numbered row-major in position order
    assert np.all(np.diff(rc[:, 0] * m + rc[:, 1]) > 0)
    # the Jacobian's nonzeros lie in the pattern, and every update's target too
    _, J = newton_matrix(km, 3, 1.0)
    order = np.argsort(P["pos"])
    inpat = np.zeros((m, m), bool)
    inpat[rc[:, 0], rc[:, 1]] = True
    Jp = J[np.ix_(order, order)]
    assert not np.any((Jp != 0) & ~inpat)
    for k in range(m):
        for x, u in P["up"][P["up_ptr"][k]:P["up_ptr"][k + 1]]:
            i, j = rc[x & 0xffff]
            assert rc[(x >> 16) & 0xffff].tolist() == [i, k] and rc[u].tolist() == [k, j] and i > k and j > k
    assert P["nnz"] < m * m


@pytest.mark.parametrize("m", [51, 120])
@pytest.mark.parametrize("c", [1e-6, 1.0, 300.0])
def test_fp64_program_solves_the_newton_system(mechs, m, c):
    km = mechs[m]
    P = program(km)
    A, _ = newton_matrix(km, 5, c)
    a = assemble(P, A, np.float64)
    dinv = factor(P, a)
    rng = np.random.default_rng(m)
    g = rng.standard_normal(m)
    x = solve(P, a, dinv, g)
    ref = np.linalg.solve(A, g)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()


def test_fp32_program_with_one_refinement_sweep(mechs):
    km = mechs[51]
    P = program(km)
    A, _ = newton_matrix(km, 9, 50.0)
    a = assemble(P, A, np.float32)
    dinv = factor(P, a)
    g = np.random.default_rng(1).standard_normal(51)
    x = solve(P, a, dinv, g.astype(np.float32)).astype(np.float64)
    r = g - A @ x
    x = x + solve(P, a, dinv, r.astype(np.float32)).astype(np.float64)
    ref = np.linalg.solve(A, g)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()


def test_larger_mechanisms_have_no_program():
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=160, n_reactions=480, seed=3)))
    info = np.zeros(12, dtype=np.int32)
    assert _capi.lib().tchem_gb_mech_sparse_lu(km.handle, info.ctypes.data, None, 0) == ERR_UNSUPPORTED


def test_oracle_static_order_time_advance_within_1e7_of_fp64(mechs):
    """The oracle's FP32 factorization in the program's order without pivoting, one refinement
    sweep per solve (the kernel's numerics), over 600 s of 24 samples."""
    import bench
    km = mechs[51]
    P = program(km)
    order = np.ascontiguousarray(np.argsort(P["pos"]).astype(np.int32))
    _, state, tadv, tol_time = bench.workload(24, 0)
    tadv["tend"], tadv["dtmax"] = 600.0, 600.0
    o = Oracle([km])
    ref = o.time_advance(tadv, state, bench.TOL_NEWTON, tol_time)
    L = load_oracle()
    assert L.oracle_set_lu_static_order(51, order.ctypes.data) == 0
    try:
        got = o.time_advance(tadv, state, bench.TOL_NEWTON, tol_time, lu_fp32=2)
    finally:
        L.oracle_set_lu_static_order(0, None)
    m = km.n_active
    err = bench.rel_err(got[0][:, 3:3 + m], ref[0][:, 3:3 + m])
    assert (got[3] == 0).all()
    assert err.max() <= 1e-7
    bad = np.array([0, 0, 5], dtype=np.int32)
    assert L.oracle_set_lu_static_order(3, bad.ctypes.data) != 0


TINY = """NCAR-version: v1.0
constant_species:
- name: M
species:
- name: A
- name: B
- name: C
reactions:{reactions}
"""

R_AB = """
- type: ARRHENIUS
  reactants:
    A: 1
  products:
    B: 1
  coefficients:
    A: 0.5"""
R_CYCLE = """
- type: ARRHENIUS
  reactants:
    A: 1
    B: 1
  products:
    C: 2
  coefficients:
    A: 1.0e-3
- type: ARRHENIUS
  reactants:
    C: 1
  products:
    A: 1
  coefficients:
    A: 2.0"""


@pytest.mark.parametrize("reactions,nnz", [(" []", 3), (R_AB, 4), (R_CYCLE, None)])
def test_small_mechanisms(reactions, nnz):
    """Edge cases of the program builder: a mechanism without reactions (the identity), one
    first-order reaction, and a cycle; each solved exactly in FP64."""
    km = KineticModel.from_string(TINY.format(reactions=reactions))
    P = program(km)
    assert P["m"] == 3
    if nnz is not None:
        assert P["nnz"] == nnz
    A, _ = newton_matrix(km, 2, 10.0)
    a = assemble(P, A, np.float64)
    dinv = factor(P, a)
    g = np.array([1.0, -2.0, 0.5])
    np.testing.assert_allclose(solve(P, a, dinv, g), np.linalg.solve(A, g), rtol=1e-12, atol=1e-15)
