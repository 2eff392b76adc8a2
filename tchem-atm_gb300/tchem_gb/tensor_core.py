"""Python face of the tensor-core building blocks of the large-mechanism factorization
(tchem_gb_tc_tile_update_tf32, tchem_gb_tc_lu_factor_tf32 in include/tchem_gb.h): thin wrappers
over contiguous float32 CUDA tensors. The kernels are tcgen05 (5th-generation tensor core) code
for sm_103a with TF32 operands, FP32 accumulation in TMEM and bounded waits that report through
tchem_gb_device_error.
"""
from __future__ import annotations

from . import _capi
from .atmospheric_chemistry import _ptr, _stream_ptr, _torch


def _check(*ts):
    torch = _torch()
    for t in ts:
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise ValueError("expected contiguous float32 CUDA tensors")


def tile_update_tf32(A, B, D, stream=None):
    """D[t] -= A[t] @ B[t] in place for tiles A [T, 128, 32], B [T, 32, N], D [T, 128, N]
    (N a multiple of 16 in [16, 256])."""
    _check(A, B, D)
    T, N = int(D.shape[0]), int(D.shape[2])
    if tuple(A.shape) != (T, 128, 32) or tuple(B.shape) != (T, 32, N) or int(D.shape[1]) != 128:
        raise ValueError("tile shapes: A [T,128,32], B [T,32,N], D [T,128,N]")
    rc = _capi.lib().tchem_gb_tc_tile_update_tf32(T, N, _ptr(A), _ptr(B), _ptr(D), _stream_ptr(stream))
    _capi.check(rc, "tchem_gb_tc_tile_update_tf32")
    return D


def lu_factor_tf32(A, stream=None):
    """In-place blocked LU with partial pivoting of A [nbatch, m, lda] (float32, row-major, the
    first m columns used). Returns (piv [nbatch, m] int32, info [nbatch] int32)."""
    torch = _torch()
    _check(A)
    nb, m, lda = (int(x) for x in A.shape)
    piv = torch.zeros(nb, m, dtype=torch.int32, device=A.device)
    info = torch.zeros(nb, dtype=torch.int32, device=A.device)
    rc = _capi.lib().tchem_gb_tc_lu_factor_tf32(nb, m, lda, _ptr(A), _ptr(piv), _ptr(info), _stream_ptr(stream))
    _capi.check(rc, "tchem_gb_tc_lu_factor_tf32")
    return piv, info
