"""ctypes binding of liboracle.so (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB_PATH, build

_libs: dict = {}


def load(native: bool = False) -> C.CDLL:
    """The oracle library: the accuracy reference, or (native) the host-tuned build timed as the
    CPU baseline."""
    if native not in _libs:
        path = build(native=native)  # rebuilt when missing or older than its sources
        L = C.CDLL(str(path))
        vp = C.c_void_p
        L.oracle_set_lu_tile_bits.restype = C.c_int
        L.oracle_set_lu_tile_bits.argtypes = [C.c_int]
        L.oracle_set_newton_min_iterations.restype = C.c_int
        L.oracle_set_newton_min_iterations.argtypes = [C.c_int]
        L.oracle_set_step_sequence.restype = C.c_int
        L.oracle_set_step_sequence.argtypes = [C.c_int, C.c_void_p]
        L.oracle_set_lu_static_order.restype = C.c_int
        L.oracle_set_lu_static_order.argtypes = [C.c_int, C.c_void_p]
        L.oracle_lu_factor_blocked.restype = C.c_int
        L.oracle_lu_factor_blocked.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.oracle_kforward.restype = C.c_int
        L.oracle_kforward.argtypes = [vp, C.c_double, C.c_double, vp]
        L.oracle_reaction_rates.restype = C.c_int
        L.oracle_reaction_rates.argtypes = [vp, C.c_double, C.c_double, vp, vp]
        L.oracle_jacobian.restype = C.c_int
        L.oracle_jacobian.argtypes = [vp, C.c_double, C.c_double, vp, vp]
        L.oracle_time_advance.restype = C.c_int
        L.oracle_time_advance.argtypes = [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                          C.c_int, C.c_int, C.c_int]
        i = C.c_int
        L.oracle_time_advance_record.restype = i
        L.oracle_time_advance_record.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i]
        L.oracle_replay.restype = i
        L.oracle_replay.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, i, vp, i]
        L.oracle_adjoint.restype = i
        L.oracle_adjoint.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, i, vp, vp, vp, i]
        L.oracle_tangent.restype = i
        L.oracle_tangent.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, i, vp, vp, vp, i]
        d = C.c_double
        for name in ("oracle_e3sm_kforward", "oracle_e3sm_rate_of_progress"):
            getattr(L, name).restype = i
            getattr(L, name).argtypes = [vp, vp, d, d, vp, vp, i, vp]
        L.oracle_e3sm_net_production_rates.restype = i
        L.oracle_e3sm_net_production_rates.argtypes = [vp, vp, d, d, vp, vp, i, vp, vp]
        L.oracle_e3sm_time_advance.restype = i
        L.oracle_e3sm_time_advance.argtypes = [vp, vp, i, vp, vp, vp, vp, vp, i, vp, vp, vp, vp, vp, vp, i, i, i]
        L.oracle_simpol_rhs.restype = i
        L.oracle_simpol_rhs.argtypes = [vp, i, d, d, vp, vp, vp]
        L.oracle_aerosol_rhs.restype = i
        L.oracle_aerosol_rhs.argtypes = [vp, vp, d, d, vp, vp, vp, vp]
        L.oracle_aerosol_time_advance.restype = i
        L.oracle_aerosol_time_advance.argtypes = [vp, vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i]
        _libs[native] = L
    return _libs[native]


def _p(a: np.ndarray | None) -> C.c_void_p:
    return C.c_void_p(0) if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """FP64 CPU restatement of the box-model path for one or more kinetic models.

    ``models`` are objects with a ``view`` attribute (a KmcdView ctypes struct) that stay alive
    for the lifetime of this object.
    """

    def __init__(self, models, native: bool = False):
        self.models = list(models)
        self.lib = load(native)
        self._views = [m.view for m in self.models]
        self._ptrs = (C.c_void_p * len(self._views))(*[C.cast(C.pointer(v), C.c_void_p) for v in self._views])

    def _vp(self, k: int = 0) -> C.c_void_p:
        return C.cast(C.pointer(self._views[k]), C.c_void_p)

    def kforward(self, T: float, p: float, k: int = 0) -> np.ndarray:
        out = np.zeros(self.models[k].nReac)
        assert self.lib.oracle_kforward(self._vp(k), T, p, _p(out)) == 0
        return out

    def reaction_rates(self, T: float, p: float, x: np.ndarray, k: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.models[k].nSpec - self.models[k].nConstSpec)
        assert self.lib.oracle_reaction_rates(self._vp(k), T, p, _p(x), _p(out)) == 0
        return out

    def jacobian(self, T: float, p: float, x: np.ndarray, k: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        m = self.models[k].nSpec - self.models[k].nConstSpec
        out = np.zeros((m, m))
        assert self.lib.oracle_jacobian(self._vp(k), T, p, _p(x), _p(out)) == 0
        return out

    def time_advance(self, tadv: np.ndarray, state: np.ndarray, tol_newton, tol_time: np.ndarray,
                     t_out: np.ndarray | None = None, mech_of_sample: np.ndarray | None = None,
                     lu_fp32: int = 0, nthreads: int = 0, simplified: bool = False):
        """Returns (state_out, t_out, dt_out, status, stats).

        lu_fp32: 0 FP64 LU; k >= 1 FP32 LU with k - 1 refinement sweeps of every Newton linear solve
        (k = 2 is the engine's mixed form).
        simplified: the simplified-Newton form (factors carried across iterations and steps).
        """
        B = state.shape[0]
        state = np.ascontiguousarray(state, dtype=np.float64)
        state_out = state.copy()
        t_out = np.array(tadv["tbeg"], dtype=np.float64) if t_out is None else np.array(t_out, dtype=np.float64)
        dt_out = np.zeros(B)
        status = np.zeros(B, dtype=np.int32)
        from tchem_gb._capi import SAMPLE_STATS_DTYPE  # struct layout shared with the engine
        stats = np.zeros(B, dtype=SAMPLE_STATS_DTYPE)
        tn = np.ascontiguousarray(tol_newton, dtype=np.float64)
        tt = np.ascontiguousarray(tol_time, dtype=np.float64)
        mos = None if mech_of_sample is None else np.ascontiguousarray(mech_of_sample, dtype=np.int32)
        tadv = np.ascontiguousarray(tadv)
        rc = self.lib.oracle_time_advance(self._ptrs, len(self._views), _p(mos), B, _p(tn), _p(tt), _p(tadv),
                                          _p(state), _p(t_out), _p(dt_out), _p(state_out), _p(status), _p(stats),
                                          int(lu_fp32), int(bool(simplified)), int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle_time_advance returned {rc}")
        return state_out, t_out, dt_out, status, stats


class E3smOracle:
    """FP64 CPU restatement of the E3SM gas-chemistry rates and time advance for one kinetic model
    (an object with ``view`` and ``e3sm_view`` attributes that outlives this one)."""

    def __init__(self, model, native: bool = False):
        self.model = model
        self.lib = load(native)
        self._km = C.cast(C.pointer(model.view), C.c_void_p)
        self._e3 = C.cast(C.pointer(model.e3sm_view), C.c_void_p)
        self.m = model.nSpec - model.nConstSpec

    def _rates(self, fn, T, p, x, photo, n_out):
        x = _a(x)
        ph = None if photo is None or len(photo) == 0 else _a(photo)
        out = np.zeros(n_out)
        rc = fn(self._km, self._e3, float(T), float(p), _p(x), _p(ph), 0 if ph is None else ph.size, _p(out))
        assert rc == 0, rc
        return out

    def kforward(self, T, p, x, photo=None) -> np.ndarray:
        return self._rates(self.lib.oracle_e3sm_kforward, T, p, x, photo, self.model.nReac)

    def rate_of_progress(self, T, p, x, photo=None) -> np.ndarray:
        return self._rates(self.lib.oracle_e3sm_rate_of_progress, T, p, x, photo, self.model.nReac)

    def net_production_rates(self, T, p, x, photo=None, ext=None) -> np.ndarray:
        x = _a(x)
        ph = None if photo is None or len(photo) == 0 else _a(photo)
        out = np.zeros(self.m)
        rc = self.lib.oracle_e3sm_net_production_rates(self._km, self._e3, float(T), float(p), _p(x), _p(ph),
                                                       0 if ph is None else ph.size,
                                                       _p(None if ext is None else _a(ext)), _p(out))
        assert rc == 0, rc
        return out

    def time_advance(self, tadv, state, photo, ext, tol_newton, tol_time, t_out=None, lu_fp32: int = 0,
                     simplified: bool = False, nthreads: int = 0):
        """Returns (state_out, t_out, dt_out, status, stats); photo [B, n_photo] or None, ext [B, m] or None."""
        B = state.shape[0]
        state = _a(state)
        state_out = state.copy()
        t_out = np.array(tadv["tbeg"], dtype=np.float64) if t_out is None else np.array(t_out, dtype=np.float64)
        dt_out = np.zeros(B)
        status = np.zeros(B, dtype=np.int32)
        from tchem_gb._capi import SAMPLE_STATS_DTYPE
        stats = np.zeros(B, dtype=SAMPLE_STATS_DTYPE)
        ph = None if photo is None or np.size(photo) == 0 else _a(photo)
        n_photo = 0 if ph is None else ph.shape[1]
        rc = self.lib.oracle_e3sm_time_advance(self._km, self._e3, B, _p(_a(tol_newton)), _p(_a(tol_time)),
                                               _p(np.ascontiguousarray(tadv)), _p(state), _p(ph), n_photo,
                                               _p(None if ext is None else _a(ext)), _p(t_out), _p(dt_out),
                                               _p(state_out), _p(status), _p(stats), int(lu_fp32),
                                               int(bool(simplified)), int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle_e3sm_time_advance returned {rc}")
        return state_out, t_out, dt_out, status, stats


class AerosolOracle:
    """FP64 CPU restatement of the aerosol chemistry (gas RHS + SIMPOL.1 phase transfer) and its
    TR-BDF2 advance, for a gas KineticModel and an AerosolModel (both outlive this object)."""

    def __init__(self, gas, aero, native: bool = False):
        self.gas, self.aero = gas, aero
        self.lib = load(native)
        self._km = C.cast(C.pointer(gas.view), C.c_void_p)
        self._av = C.cast(C.pointer(aero.view), C.c_void_p)

    def simpol_rhs(self, i_simpol: int, T, p, number_conc, x) -> np.ndarray:
        x = _a(x)
        out = np.zeros_like(x)
        assert self.lib.oracle_simpol_rhs(self._av, int(i_simpol), float(T), float(p), _p(_a(number_conc)), _p(x),
                                          _p(out)) == 0
        return out

    def rhs(self, T, p, number_conc, x, xconst) -> np.ndarray:
        x = _a(x)
        out = np.zeros_like(x)
        xc = _a(xconst) if np.size(xconst) else None
        assert self.lib.oracle_aerosol_rhs(self._km, self._av, float(T), float(p), _p(_a(number_conc)), _p(x), _p(xc),
                                           _p(out)) == 0
        return out

    def time_advance(self, tadv, state, number_conc, tol_newton, tol_time, t_out=None, nthreads: int = 0):
        """Returns (state_out, t_out, dt_out, status, stats) for state rows [rho, p, T, gas, particles]."""
        B = state.shape[0]
        state = _a(state)
        state_out = state.copy()
        t_out = np.array(tadv["tbeg"], dtype=np.float64) if t_out is None else np.array(t_out, dtype=np.float64)
        dt_out = np.zeros(B)
        status = np.zeros(B, dtype=np.int32)
        from tchem_gb._capi import SAMPLE_STATS_DTYPE
        stats = np.zeros(B, dtype=SAMPLE_STATS_DTYPE)
        rc = self.lib.oracle_aerosol_time_advance(self._km, self._av, B, _p(_a(tol_newton)), _p(_a(tol_time)),
                                                  _p(np.ascontiguousarray(tadv)), _p(state), _p(_a(number_conc)),
                                                  _p(t_out), _p(dt_out), _p(state_out), _p(status), _p(stats),
                                                  int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle_aerosol_time_advance returned {rc}")
        return state_out, t_out, dt_out, status, stats


class Tape:
    """Recorded accepted step sizes of a forward run (for replay, adjoint and tangent)."""

    def __init__(self, dt: np.ndarray, nsteps: np.ndarray):
        self.dt, self.nsteps = dt, nsteps

    @property
    def cap(self) -> int:
        return self.dt.shape[1]


def _a(x, dtype=np.float64):
    return np.ascontiguousarray(x, dtype=dtype)


def record(o: "Oracle", tadv, state, tol_newton, tol_time, cap: int, k_scale=None, nthreads: int = 0):
    """FP64 forward run recording the step sequence: (state_out, t_out, dt_out, status, Tape)."""
    B = state.shape[0]
    state = _a(state)
    out = state.copy()
    t_out, dt_out = np.zeros(B), np.zeros(B)
    status = np.zeros(B, dtype=np.int32)
    dt = np.zeros((B, cap))
    ns = np.zeros(B, dtype=np.int32)
    rc = o.lib.oracle_time_advance_record(o._vp(0), B, _p(_a(tol_newton)), _p(_a(tol_time)),
                                          _p(None if k_scale is None else _a(k_scale)), _p(np.ascontiguousarray(tadv)),
                                          _p(state), _p(t_out), _p(dt_out), _p(out), _p(status), _p(dt), _p(ns), cap,
                                          nthreads)
    assert rc == 0, rc
    return out, t_out, dt_out, status, Tape(dt, ns)


def replay(o: "Oracle", tadv, state, tol_newton, tape: Tape, k_scale=None, nthreads: int = 0) -> np.ndarray:
    """End states [B][m] of the recorded steps re-run from state (fixed step sequence)."""
    B = state.shape[0]
    m = o.models[0].nSpec - o.models[0].nConstSpec
    y = np.zeros((B, m))
    rc = o.lib.oracle_replay(o._vp(0), B, _p(_a(tol_newton)), _p(None if k_scale is None else _a(k_scale)),
                             _p(np.ascontiguousarray(tadv)), _p(_a(state)), _p(tape.dt), _p(tape.nsteps), tape.cap,
                             _p(y), nthreads)
    assert rc == 0, rc
    return y


def adjoint(o: "Oracle", tadv, state, tol_newton, tape: Tape, lam, k_scale=None, nthreads: int = 0):
    """(dL/dy0 [B][m], dL/dtheta [B][R]) for the cotangent lam = dL/dy_end [B][m]."""
    B = state.shape[0]
    km = o.models[0]
    m, R = km.nSpec - km.nConstSpec, km.nReac
    gx, gk = np.zeros((B, m)), np.zeros((B, R))
    rc = o.lib.oracle_adjoint(o._vp(0), B, _p(_a(tol_newton)), _p(None if k_scale is None else _a(k_scale)),
                              _p(np.ascontiguousarray(tadv)), _p(_a(state)), _p(tape.dt), _p(tape.nsteps), tape.cap,
                              _p(_a(lam)), _p(gx), _p(gk), nthreads)
    assert rc == 0, rc
    return gx, gk


def tangent(o: "Oracle", tadv, state, tol_newton, tape: Tape, dx0, dtheta, k_scale=None, nthreads: int = 0):
    """Forward sensitivities dy_end [B][m] along (dx0 [B][m], dtheta [B][R])."""
    B = state.shape[0]
    m = o.models[0].nSpec - o.models[0].nConstSpec
    dy = np.zeros((B, m))
    rc = o.lib.oracle_tangent(o._vp(0), B, _p(_a(tol_newton)), _p(None if k_scale is None else _a(k_scale)),
                              _p(np.ascontiguousarray(tadv)), _p(_a(state)), _p(tape.dt), _p(tape.nsteps), tape.cap,
                              _p(_a(dx0)), _p(_a(dtheta)), _p(dy), nthreads)
    assert rc == 0, rc
    return dy


def library_path() -> Path:
    return LIB_PATH


def lu_factor_blocked(a: np.ndarray, keep: int = 10) -> tuple[np.ndarray, np.ndarray]:
    """(lu, piv) of the FP32 matrix a as the tensor-core LU computes it (TF32 tiles for keep = 10)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    n = a.shape[0]
    lu = np.zeros_like(a)
    piv = np.zeros(n, dtype=np.int32)
    rc = load().oracle_lu_factor_blocked(n, a.ctypes.data, int(keep), lu.ctypes.data, piv.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle_lu_factor_blocked returned {rc}")
    return lu, piv
