"""Python face of the E3SM gas chemistry: per-sample photolysis rates and external sources.

Reference interfaces mirrored (names and argument order):
  TChem::AtmosphericChemistryE3SM::getWorkSpaceSize(kmcd)
  TChem::AtmosphericChemistryE3SM::runDeviceBatch(policy, tol_newton, tol_time, fac, tadv, state,
      photo_rates, external_sources, t_out, dt_out, state_out, kmcd)
                                          src/core/TChem_AtmosphericChemistryE3SM.hpp:47-104
  TChem::ReactionRates::runDeviceBatch(policy, state, kfwd, kmcd)
                                          src/core/TChem_ReactionRates.hpp:59-72
  TChem::RateofProgress::runDeviceBatch(policy, state, photo_rates, rate_of_progress, kmcd)
                                          src/core/TChem_RateofProgress.hpp:60-75
  TChem::NetProductionRates::runDeviceBatch(policy, state, photo_rates, external_sources,
      net_production_rates, kmcd)         src/core/TChem_NetProductionRates.hpp:61-78
The arrays are contiguous float64 torch CUDA tensors; photo_rates [B, n_photo] and
external_sources [B, m] may be None (no photolysis input, zero sources). The computation is the
engine's CUDA kernels behind the C ABI (tchem_gb_e3sm_*); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .atmospheric_chemistry import _opts, _ptr, _stream_ptr, _torch
from .mechanism import KineticModel


def _check_tensors(*ts):
    torch = _torch()
    for t in ts:
        if t is not None and not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise ValueError("expected contiguous float64 CUDA tensors")


def _n_photo(photo_rates) -> int:
    return 0 if photo_rates is None else int(photo_rates.shape[1])


class AtmosphericChemistryE3SM:
    """Batched TR-BDF2 advance of the E3SM gas chemistry (TChem::AtmosphericChemistryE3SM)."""

    @staticmethod
    def getWorkSpaceSize(kmcd: KineticModel, nbatch: int = 1, form: str | int = "plain") -> int:
        o = _opts(form)
        n = _capi.lib().tchem_gb_e3sm_workspace_bytes(kmcd.handle, int(nbatch), C.byref(o))
        if n == 0:
            _capi.check(1, "tchem_gb_e3sm_workspace_bytes")
        return int(n)

    @staticmethod
    def runDeviceBatch(tol_newton, tol_time, fac, tadv, state, photo_rates, external_sources, t_out, dt_out,
                       state_out, kmcd: KineticModel, *, status=None, stats=None, form: str | int = "plain",
                       threads_per_sample: int = 0, workspace=None, stream=None):
        """Advances every sample whose t_out < tadv.tend; returns the status tensor. Arguments as
        AtmosphericChemistry.runDeviceBatch plus photo_rates and external_sources."""
        torch = _torch()
        _check_tensors(tol_newton, tol_time, state, photo_rates, external_sources, t_out, dt_out, state_out)
        B = int(state.shape[0])
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=state.device)
        o = _opts(form, threads_per_sample)
        ws_ptr, ws_bytes = C.c_void_p(0), 0
        if workspace is not None:
            ws_ptr, ws_bytes = _ptr(workspace), workspace.numel() * workspace.element_size()
        rc = _capi.lib().tchem_gb_e3sm_time_advance(
            kmcd.handle, B, _ptr(tol_newton), _ptr(tol_time), _ptr(fac), _ptr(tadv), _ptr(state), _ptr(photo_rates),
            _n_photo(photo_rates), _ptr(external_sources), _ptr(t_out), _ptr(dt_out), _ptr(state_out), _ptr(status),
            _ptr(stats), ws_ptr, ws_bytes, C.byref(o), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_e3sm_time_advance")
        return status

    @staticmethod
    def runHostBatch(tol_newton, tol_time, tadv: np.ndarray, state: np.ndarray, photo_rates, external_sources,
                     t_out: np.ndarray, kmcd: KineticModel, *, form: str | int = "plain", threads_per_sample: int = 0):
        """Host-array variant (runHostBatch): copies in, advances on the GPU, copies out
        (synchronous). Returns (state_out, t_out, dt_out, status) as numpy arrays."""
        torch = _torch()
        from .atmospheric_chemistry import tadv_to_device
        dev = torch.device("cuda", torch.cuda.current_device())

        def d(a):
            return None if a is None or np.size(a) == 0 else torch.as_tensor(
                np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        d_state = d(state)
        out = d_state.clone()  # rows the advance does not write (skipped samples) come back unchanged
        t = d(t_out)
        dt = torch.zeros_like(t)
        status = AtmosphericChemistryE3SM.runDeviceBatch(d(tol_newton), d(tol_time), None, tadv_to_device(tadv, dev),
                                                         d_state, d(photo_rates), d(external_sources), t, dt, out,
                                                         kmcd, form=form, threads_per_sample=threads_per_sample)
        torch.cuda.synchronize(dev)
        return out.cpu().numpy(), t.cpu().numpy(), dt.cpu().numpy(), status.cpu().numpy()


class ReactionRates:
    """Rate constants kfwd[B, nReac] in the E3SM forms (TChem::ReactionRates)."""

    @staticmethod
    def runDeviceBatch(state, kfwd, kmcd: KineticModel, *, photo_rates=None, stream=None):
        _check_tensors(state, kfwd, photo_rates)
        rc = _capi.lib().tchem_gb_e3sm_reaction_rates(kmcd.handle, int(state.shape[0]), _ptr(state), _ptr(photo_rates),
                                                      _n_photo(photo_rates), _ptr(kfwd), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_e3sm_reaction_rates")
        return kfwd


class RateofProgress:
    """Rates of progress q[B, nReac] (TChem::RateofProgress)."""

    @staticmethod
    def runDeviceBatch(state, photo_rates, rate_of_progress, kmcd: KineticModel, *, stream=None):
        _check_tensors(state, photo_rates, rate_of_progress)
        rc = _capi.lib().tchem_gb_e3sm_rate_of_progress(kmcd.handle, int(state.shape[0]), _ptr(state),
                                                        _ptr(photo_rates), _n_photo(photo_rates),
                                                        _ptr(rate_of_progress), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_e3sm_rate_of_progress")
        return rate_of_progress


class NetProductionRates:
    """Net production rates omega[B, m] of the active species (TChem::NetProductionRates; the
    reference's output has nSpec columns of which the active ones are written)."""

    @staticmethod
    def runDeviceBatch(state, photo_rates, external_sources, net_production_rates, kmcd: KineticModel, *,
                       stream=None):
        _check_tensors(state, photo_rates, external_sources, net_production_rates)
        rc = _capi.lib().tchem_gb_e3sm_net_production_rates(kmcd.handle, int(state.shape[0]), _ptr(state),
                                                            _ptr(photo_rates), _n_photo(photo_rates),
                                                            _ptr(external_sources), _ptr(net_production_rates),
                                                            _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_e3sm_net_production_rates")
        return net_production_rates
