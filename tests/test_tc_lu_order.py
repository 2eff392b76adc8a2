"""The elimination order of the tensor-core form's LU (csrc/kernels_tc_advance.cu), restated in
numpy and checked against numpy.linalg.solve on the CPU: 32-column panels factored with implicit
partial pivoting (the pivot row leaves the active set, no row moves; the largest |a| among active
rows, ties to the lowest panel row), the new logical order = the panel's pivots in step order, then
the remaining rows by increasing panel row; U12 = L11^-1 A12 through that order; the trailing update
A22 -= L21 U12 in logical rows mapped to physical rows through the permutation; and the blocked
substitutions in the kernel's order (warp 0 applies the previous block to the next block's rows and
solves that block, the others update the remaining rows). This pins the index logic the kernel's
first GPU runs relied on, for sizes with full and ragged last panels."""
from __future__ import annotations

import numpy as np
import pytest


def factor(A0: np.ndarray, PW: int = 32):
    m = A0.shape[0]
    A = A0.copy()
    perm = np.arange(m)
    for k0 in range(0, m, PW):
        kb, np_ = min(PW, m - k0), m - k0
        p1 = k0 + kb
        prow = [perm[k0 + r] for r in range(np_)]
        a = np.zeros((np_, PW))
        for r in range(np_):
            a[r, :kb] = A[prow[r], k0:k0 + kb]
        act = np.ones(np_, bool)
        pn = np.zeros((PW, PW))
        pphys = [0] * kb
        for c in range(kb):
            cand = np.nonzero(act)[0]
            bi = cand[int(np.argmax(np.abs(a[cand, c])))]  # first maximum = lowest panel row
            pn[c] = a[bi]
            act[bi] = False
            pphys[c] = prow[bi]
            for r in cand:
                if r != bi:
                    l = a[r, c] / pn[c, c]
                    a[r, c] = l
                    a[r, c + 1:] -= l * pn[c, c + 1:]
        for r in range(np_):
            A[prow[r], k0:k0 + kb] = a[r, :kb]
        trail = [r for r in range(np_) if act[r]]
        perm = perm.copy()
        perm[k0:p1] = pphys
        perm[p1:] = [prow[r] for r in trail]
        W = m - p1
        if W <= 0:
            break
        U = np.array([A[perm[k0 + i], p1:] for i in range(kb)])
        for i in range(1, kb):
            U[i] -= pn[i, :i] @ U[:i]
        for i in range(kb):
            A[perm[k0 + i], p1:] = U[i]
        L21 = np.array([a[r, :kb] for r in trail])
        update = L21 @ U
        for q in range(W):
            A[perm[p1 + q], p1:] -= update[q]
    return A, perm


def solve(A: np.ndarray, perm: np.ndarray, b: np.ndarray, PW: int = 32) -> np.ndarray:
    m = A.shape[0]
    L = lambda i, j: A[perm[i], j]  # noqa: E731
    w = b[perm].copy()
    nb = (m + PW - 1) // PW

    def diag_lower(k0):
        kb = min(PW, m - k0)
        for c in range(kb):
            for r in range(k0 + c + 1, k0 + kb):
                w[r] -= L(r, k0 + c) * w[k0 + c]

    def diag_upper(k0):
        kb = min(PW, m - k0)
        for c in range(kb - 1, -1, -1):
            w[k0 + c] /= L(k0 + c, k0 + c)
            for r in range(k0, k0 + c):
                w[r] -= L(r, k0 + c) * w[k0 + c]

    diag_lower(0)
    for blk in range(nb - 1):
        k0 = blk * PW
        nxt = k0 + PW
        for r in range(nxt, min(nxt + PW, m)):
            w[r] -= sum(L(r, k0 + c) * w[k0 + c] for c in range(PW))
        diag_lower(nxt)
        for i in range(nxt + PW, m):
            w[i] -= sum(L(i, k0 + c) * w[k0 + c] for c in range(PW))
    diag_upper((nb - 1) * PW)
    for blk in range(nb - 1, 0, -1):
        k0, kb = blk * PW, min(PW, m - blk * PW)
        prev = k0 - PW
        for r in range(prev, prev + PW):
            w[r] -= sum(L(r, k0 + c) * w[k0 + c] for c in range(kb))
        diag_upper(prev)
        for i in range(prev):
            w[i] -= sum(L(i, k0 + c) * w[k0 + c] for c in range(kb))
    return w


@pytest.mark.parametrize("m", [51, 64, 130, 257, 300, 320])
def test_tensor_core_lu_order_solves_newton_like_systems(m):
    rng = np.random.default_rng(m)
    c = 10.0 ** rng.uniform(-3, 1)
    J = rng.standard_normal((m, m)) * (rng.random((m, m)) < 0.1)
    A0 = np.eye(m) - c * J  # a Newton matrix I - c J with a sparse random Jacobian
    A, perm = factor(A0)
    assert sorted(perm.tolist()) == list(range(m))  # a permutation of the rows
    b = rng.standard_normal(m)
    x = solve(A, perm, b)
    ref = np.linalg.solve(A0, b)
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()
