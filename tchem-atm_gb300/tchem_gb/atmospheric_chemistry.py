"""Python face of the batched box-model time advance, mirroring TChem::AtmosphericChemistry.

Reference interface (src/core/TChem_AtmosphericChemistry.hpp:47-157):
  getWorkSpaceSize(kmcd)
  runDeviceBatch(policy, tol_newton, tol_time, fac, tadv, state, t_out, dt_out, state_out, kmcd)
  runDeviceBatch(policy, ..., kmcds)            # one mechanism per sample
Here the arrays are torch CUDA tensors (device memory and streams only; the computation is the
engine's CUDA kernels behind the C ABI). There is no CPU fallback: without the compiled library
and a CUDA device the calls raise.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _capi
from .mechanism import KineticModel

FORMS = {"plain": 0, "fp64": 0, "mixed": 1, "simplified": 2, "mixed_simplified": 2}


AdvanceOpts = _capi.AdvanceOpts


def _torch():
    import torch  # imported lazily: the front end does not need it
    return torch


def time_advance_array(n: int, tbeg=0.0, tend=1.0, dt=1e-8, dtmin=1e-8, dtmax=1e-1, max_num_newton_iterations=100,
                       num_time_iterations_per_interval=10, jacobian_interval=1) -> np.ndarray:
    """Host array of TimeAdvance structs (src/core/TChem_Util.hpp:469-477) with the given fields."""
    a = np.zeros(n, dtype=_capi.TIME_ADVANCE_DTYPE)
    a["tbeg"], a["tend"], a["dt"], a["dtmin"], a["dtmax"] = tbeg, tend, dt, dtmin, dtmax
    a["max_num_newton_iterations"] = max_num_newton_iterations
    a["num_time_iterations_per_interval"] = num_time_iterations_per_interval
    a["jacobian_interval"] = jacobian_interval
    return a


def tadv_to_device(tadv: np.ndarray, device="cuda"):
    """TimeAdvance array -> uint8 CUDA tensor [n, 56] holding the packed structs."""
    torch = _torch()
    raw = np.ascontiguousarray(tadv).view(np.uint8).reshape(len(tadv), _capi.TIME_ADVANCE_DTYPE.itemsize)
    return torch.from_numpy(raw.copy()).to(device)


def _mechs(kmcd) -> list[KineticModel]:
    if isinstance(kmcd, KineticModel):
        return [kmcd]
    return list(kmcd)


def _handles(mechs: Sequence[KineticModel]):
    arr = (C.c_void_p * len(mechs))(*[m.handle.value for m in mechs])
    return arr


def _ptr(t) -> C.c_void_p:
    if t is None:
        return C.c_void_p(0)
    return C.c_void_p(t.data_ptr())


def _stream_ptr(stream) -> C.c_void_p:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _opts(form: str | int, threads_per_sample: int = 0) -> AdvanceOpts:
    o = AdvanceOpts()
    o.form = FORMS[form] if isinstance(form, str) else int(form)
    o.threads_per_sample = int(threads_per_sample)
    return o


class AtmosphericChemistry:
    """Batched TR-BDF2 box-model advance (TChem::AtmosphericChemistry)."""

    @staticmethod
    def getWorkSpaceSize(kmcd, nbatch: int = 1, form: str | int = "plain") -> int:
        mechs = _mechs(kmcd)
        o = _opts(form)
        n = _capi.lib().tchem_gb_workspace_bytes(_handles(mechs), len(mechs), int(nbatch), C.byref(o))
        if n == 0:
            _capi.check(1, "tchem_gb_workspace_bytes")
        return int(n)

    @staticmethod
    def runDeviceBatch(tol_newton, tol_time, fac, tadv, state, t_out, dt_out, state_out, kmcd, *,
                       mech_of_sample=None, status=None, stats=None, form: str | int = "plain",
                       threads_per_sample: int = 0, workspace=None, stream=None):
        """Advances every sample whose t_out < tadv.tend; returns the status tensor.

        tol_newton [2], tol_time [m][2], tadv (uint8 [B,56] from tadv_to_device), state
        [B][nSpec+3], t_out [B] (read and written), dt_out [B], state_out (may be state): float64
        CUDA tensors. kmcd is a KineticModel or a sequence of them with mech_of_sample [B] int32.
        """
        torch = _torch()
        mechs = _mechs(kmcd)
        B = int(state.shape[0])
        for t in (tol_newton, tol_time, state, t_out, dt_out, state_out):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("runDeviceBatch expects contiguous float64 CUDA tensors")
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=state.device)
        o = _opts(form, threads_per_sample)
        L = _capi.lib()
        ws_ptr, ws_bytes = C.c_void_p(0), 0
        if workspace is not None:
            ws_ptr, ws_bytes = _ptr(workspace), workspace.numel() * workspace.element_size()
        rc = L.tchem_gb_time_advance(
            _handles(mechs), len(mechs), _ptr(mech_of_sample), B, _ptr(tol_newton), _ptr(tol_time), _ptr(fac),
            _ptr(tadv), _ptr(state), _ptr(t_out), _ptr(dt_out), _ptr(state_out), _ptr(status), _ptr(stats),
            ws_ptr, ws_bytes, C.byref(o), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_time_advance")
        return status

    @staticmethod
    def runHostBatch(tol_newton, tol_time, tadv: np.ndarray, state: np.ndarray, t_out: np.ndarray, kmcd, *,
                     mech_of_sample=None, form: str | int = "plain", threads_per_sample: int = 0,
                     with_stats: bool = False, stream=None):
        """Host-array variant: copies in, advances on the GPU, copies out (synchronous).

        Returns (state_out, t_out, dt_out, status, stats-or-None) as numpy arrays.
        """
        mechs = _mechs(kmcd)
        B = state.shape[0]
        state = np.ascontiguousarray(state, dtype=np.float64)
        state_out = state.copy()
        t_o = np.ascontiguousarray(t_out, dtype=np.float64).copy()
        dt_o = np.zeros(B)
        status = np.zeros(B, dtype=np.int32)
        stats = np.zeros(B, dtype=_capi.SAMPLE_STATS_DTYPE) if with_stats else None
        tn = np.ascontiguousarray(tol_newton, dtype=np.float64)
        tt = np.ascontiguousarray(tol_time, dtype=np.float64)
        tadv = np.ascontiguousarray(tadv)
        mos = None if mech_of_sample is None else np.ascontiguousarray(mech_of_sample, dtype=np.int32)
        o = _opts(form, threads_per_sample)
        p = lambda a: C.c_void_p(0) if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
        rc = _capi.lib().tchem_gb_time_advance_hostbuf(
            _handles(mechs), len(mechs), p(mos), B, p(tn), p(tt), p(tadv), p(state), p(t_o), p(dt_o), p(state_out),
            p(status), p(stats), C.byref(o), _stream_ptr(stream) if stream is not None else C.c_void_p(0))
        _capi.check(rc, "tchem_gb_time_advance_hostbuf")
        return state_out, t_o, dt_o, status, stats

    @staticmethod
    def autotune(kmcd: KineticModel, tol_newton, tol_time, tadv, state, *, form: str | int = "simplified",
                 stream=None):
        """Times the form's kernel shapes (32/64/128 threads per sample) on the probe batch (device
        arrays as for runDeviceBatch; the probe starts at t = 0), keeps the fastest as the mechanism's
        default and returns (threads_per_sample, {shape: ms})."""
        torch = _torch()
        B = int(state.shape[0])
        out = torch.empty_like(state)
        t = torch.zeros(B, dtype=torch.float64, device=state.device)
        dt = torch.zeros_like(t)
        st = torch.empty(B, dtype=torch.int32, device=state.device)
        chosen = C.c_int(0)
        ms = (C.c_float * 3)()
        o = _opts(form)
        rc = _capi.lib().tchem_gb_autotune(kmcd.handle, o.form, B, _ptr(tol_newton), _ptr(tol_time), _ptr(tadv),
                                           _ptr(state), _ptr(t), _ptr(dt), _ptr(out), _ptr(st), None, 0,
                                           _stream_ptr(stream), C.byref(chosen), ms)
        _capi.check(rc, "tchem_gb_autotune")
        return chosen.value, {32 * (1 << i): ms[i] for i in range(3) if ms[i] >= 0}

    @staticmethod
    def set_threads_per_sample(kmcd: KineticModel, threads_per_sample: int, form: str | int = "simplified"):
        o = _opts(form)
        _capi.check(_capi.lib().tchem_gb_mech_set_threads_per_sample(kmcd.handle, o.form, int(threads_per_sample)),
                    "tchem_gb_mech_set_threads_per_sample")

    @staticmethod
    def capture(tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, kmcd, *, mech_of_sample=None,
                status=None, form: str | int = "simplified", threads_per_sample: int = 0):
        """Captures one whole-batch advance -- t_out reset to tadv.tbeg's start (0), the per-sample
        mechanism bucketing and one persistent kernel per mechanism structure -- into a CUDA graph and
        returns it; graph.replay() re-runs the batch from its initial state with one launch. The
        workspace is allocated here, before capture, and kept with the graph."""
        torch = _torch()
        mechs = _mechs(kmcd)
        B = int(state.shape[0])
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=state.device)
        o = _opts(form, threads_per_sample)
        n = _capi.lib().tchem_gb_workspace_bytes(_handles(mechs), len(mechs), B, C.byref(o))
        if n == 0:
            _capi.check(1, "tchem_gb_workspace_bytes")
        ws = torch.zeros(int(n), dtype=torch.uint8, device=state.device)  # error word starts clear
        side = torch.cuda.Stream(device=state.device)
        side.wait_stream(torch.cuda.current_stream(state.device))
        # one eager call with every sample already past its end (all skipped: no integration work):
        # mechanism tables on the device, kernel attributes and side streams set up before capture
        with torch.cuda.stream(side):
            t_out.fill_(float("inf"))
            AtmosphericChemistry.runDeviceBatch(tol_newton, tol_time, None, tadv, state, t_out, dt_out, state_out,
                                                kmcd, mech_of_sample=mech_of_sample, status=status, form=form,
                                                threads_per_sample=threads_per_sample, workspace=ws, stream=side)
        torch.cuda.current_stream(state.device).wait_stream(side)
        torch.cuda.synchronize(state.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            t_out.zero_()
            AtmosphericChemistry.runDeviceBatch(tol_newton, tol_time, None, tadv, state, t_out, dt_out, state_out,
                                                kmcd, mech_of_sample=mech_of_sample, status=status, form=form,
                                                threads_per_sample=threads_per_sample, workspace=ws)
        g._tchem_workspace = ws  # keep the workspace alive with the graph
        return g, status

    @staticmethod
    def carry_over(tadv, t_out, dt_out, iters_per_interval: int = 0, t_sum=None, stream=None):
        """The host loop's carry-over between two runDeviceBatch calls
        (src/examples/TChem_AtmosphericChemistry.cpp:340-350): tadv.tbeg = t_out, tadv.dt = dt_out
        per sample, the next call's step budget when iters_per_interval > 0, and the sum of t_out
        into t_sum (a float64 CUDA tensor of one element) when given. One kernel on the stream."""
        rc = _capi.lib().tchem_gb_time_advance_carry_over(_ptr(tadv), _ptr(t_out), _ptr(dt_out), int(t_out.shape[0]),
                                                          int(iters_per_interval), _ptr(t_sum), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_time_advance_carry_over")

    @staticmethod
    def device_error(workspace=None, stream=None) -> int:
        err = C.c_int32(0)
        _capi.check(_capi.lib().tchem_gb_device_error(_ptr(workspace), _stream_ptr(stream), C.byref(err)),
                    "tchem_gb_device_error")
        return err.value


def _unit(fn_name: str, kmcd, state, out, mech_of_sample=None, stream=None):
    mechs = _mechs(kmcd)
    rc = getattr(_capi.lib(), fn_name)(_handles(mechs), len(mechs), _ptr(mech_of_sample), int(state.shape[0]),
                                      _ptr(state), _ptr(out), _stream_ptr(stream))
    _capi.check(rc, fn_name)
    return out


def kforward(kmcd, state, out=None, **kw):
    """Rate constants kfor[B][nReac] (KForwardAerosol)."""
    torch = _torch()
    km = _mechs(kmcd)[0]
    out = out if out is not None else torch.empty(state.shape[0], km.nReac, dtype=torch.float64, device=state.device)
    return _unit("tchem_gb_kforward", kmcd, state, out, **kw)


def reaction_rates(kmcd, state, out=None, **kw):
    """Net production rates omega[B][m] of the active species (ReactionRatesAerosol)."""
    torch = _torch()
    km = _mechs(kmcd)[0]
    out = out if out is not None else torch.empty(state.shape[0], km.n_active, dtype=torch.float64,
                                                  device=state.device)
    return _unit("tchem_gb_reaction_rates", kmcd, state, out, **kw)


def jacobian(kmcd, state, out=None, **kw):
    """Analytic Jacobian d omega / d x [B][m][m]."""
    torch = _torch()
    km = _mechs(kmcd)[0]
    out = out if out is not None else torch.empty(state.shape[0], km.n_active, km.n_active, dtype=torch.float64,
                                                  device=state.device)
    return _unit("tchem_gb_jacobian", kmcd, state, out, **kw)


def kernel_launches() -> int:
    """Kernels the engine library has launched in this process (tchem_gb_kernel_launches)."""
    return int(_capi.lib().tchem_gb_kernel_launches())
