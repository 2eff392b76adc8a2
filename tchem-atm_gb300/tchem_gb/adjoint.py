"""Discrete adjoint of the batched TR-BDF2 box model (plain FP64 form) and its autograd face.

  record(...)   forward run that also records the accepted step sizes and a checkpoint of the
                state every 32 steps (tchem_gb_time_advance_record)
  adjoint(...)  dL/dy0 and dL/dtheta for a cotangent dL/dy_end (tchem_gb_adjoint), where
                exp(theta_r) multiplies reaction r's rate constant (theta_r = d ln A_r)
  BoxModelSolve torch.autograd.Function: (log_x0 [B][m], log_k [R]) -> y_end [B][m]

The reference's TR-BDF2 has no adjoint; this extends runDeviceBatch
(src/core/TChem_AtmosphericChemistry.hpp:83-105). The step sequence of the recorded run is
held fixed in the backward pass (step-size control is not differentiated).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _capi
from .mechanism import KineticModel

SEGMENT = 32  # steps between checkpoints


def _torch():
    import torch
    return torch


def _p(t) -> C.c_void_p:
    return C.c_void_p(0) if t is None else C.c_void_p(t.data_ptr())


def _stream(stream):
    torch = _torch()
    return C.c_void_p((stream if stream is not None else torch.cuda.current_stream()).cuda_stream)


@dataclass
class Tape:
    """Trajectory record of a forward run (device tensors)."""
    dt: "object"       # [B][cap] float64
    ckpt: "object"     # [B][cap // 32 + 1][m] float64
    nsteps: "object"   # [B] int32
    cap: int


def new_tape(B: int, m: int, cap: int, device="cuda") -> Tape:
    torch = _torch()
    return Tape(torch.zeros(B, cap, dtype=torch.float64, device=device),
                torch.zeros(B, cap // SEGMENT + 1, m, dtype=torch.float64, device=device),
                torch.zeros(B, dtype=torch.int32, device=device), cap)


def record(km: KineticModel, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, tape: Tape, *,
           k_scale=None, status=None, stats=None, stream=None):
    """Plain FP64 time advance that also fills `tape`; returns the status tensor."""
    torch = _torch()
    B = int(state.shape[0])
    if status is None:
        status = torch.empty(B, dtype=torch.int32, device=state.device)
    rc = _capi.lib().tchem_gb_time_advance_record(
        km.handle, B, _p(tol_newton), _p(tol_time), _p(k_scale), _p(tadv), _p(state), _p(t_out), _p(dt_out),
        _p(state_out), _p(status), _p(stats), _p(tape.dt), _p(tape.ckpt), _p(tape.nsteps), tape.cap,
        _stream(stream))
    _capi.check(rc, "tchem_gb_time_advance_record")
    return status


def adjoint(km: KineticModel, tol_newton, tadv, state, tape: Tape, lam, *, k_scale=None, status=None,
            stream=None):
    """(dL/dy0 [B][m], dL/dtheta [B][R], status) for lam = dL/dy_end [B][m] of a recorded run."""
    torch = _torch()
    B = int(state.shape[0])
    m, R = km.n_active, km.nReac
    gx = torch.empty(B, m, dtype=torch.float64, device=state.device)
    gk = torch.empty(B, R, dtype=torch.float64, device=state.device)
    if status is None:
        status = torch.empty(B, dtype=torch.int32, device=state.device)
    rc = _capi.lib().tchem_gb_adjoint(km.handle, B, _p(tol_newton), _p(k_scale), _p(tadv), _p(state), _p(tape.dt),
                                      _p(tape.ckpt), _p(tape.nsteps), tape.cap, _p(lam.contiguous()), _p(gx), _p(gk),
                                      _p(status), None, 0, _stream(stream))
    _capi.check(rc, "tchem_gb_adjoint")
    return gx, gk, status


class BoxModelSolve:
    """Differentiable end state of the box-model batch.

    y_end = BoxModelSolve.apply(log_x0, log_k, km, state, tadv, tol_newton, tol_time, cap)
      log_x0 [B][m]: log of the initial active-species concentrations (replaces state's)
      log_k [R]:     log multipliers of the rate constants (0 = the mechanism as parsed)
    Gradients flow to log_x0 and log_k through the discrete adjoint; the other arguments are
    constants. Samples whose forward run fails raise in the backward pass.
    """

    @staticmethod
    def _fn():
        torch = _torch()

        class _F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, log_x0, log_k, km, state, tadv, tol_newton, tol_time, cap):
                m = km.n_active
                st = state.clone()
                st[:, 3:3 + m] = torch.exp(log_x0)
                k_scale = torch.exp(log_k).contiguous()
                B = st.shape[0]
                out = torch.empty_like(st)
                t = torch.zeros(B, dtype=torch.float64, device=st.device)
                dt = torch.zeros_like(t)
                tape = new_tape(B, m, cap, st.device)
                status = record(km, tol_newton, tol_time, tadv, st, t, dt, out, tape, k_scale=k_scale)
                if int((status != 0).sum()):
                    raise RuntimeError("BoxModelSolve: forward run failed for some samples")
                ctx.km, ctx.tape = km, tape
                ctx.save_for_backward(st, k_scale, tadv, tol_newton)
                return out[:, 3:3 + m].clone()

            @staticmethod
            def backward(ctx, grad_y):
                st, k_scale, tadv, tol_newton = ctx.saved_tensors
                m = ctx.km.n_active
                gx, gk, status = adjoint(ctx.km, tol_newton, tadv, st, ctx.tape,
                                         grad_y.to(torch.float64).contiguous(), k_scale=k_scale)
                if int((status != 0).sum()):
                    raise RuntimeError("BoxModelSolve: adjoint failed for some samples")
                return gx * st[:, 3:3 + m], gk.sum(dim=0), None, None, None, None, None, None

        return _F

    @classmethod
    def apply(cls, *args):
        if not hasattr(cls, "_F"):
            cls._F = cls._fn()
        return cls._F.apply(*args)
