"""First GPU checks of the tensor-core building blocks (tchem_gb_tc_tile_update_tf32,
tchem_gb_tc_lu_factor_tf32). Kept out of the default collection (the file name does not start with
test_) until their first run on a GB300, which is made by hand on these small cases:

  python -m pytest tests/gpu_pending_tc.py -x -q

* one 128 x 64 tile update against the FP64 product (TF32 operands: relative error ~1e-3);
* four 300 x 300 Newton-like matrices factored in place against the oracle's restatement in the
  same order (oracle.lu_factor_blocked, TF32 operands): equal pivots, factors within the TF32
  bound, P A = L U to the TF32 level; and the device error word clear.
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
