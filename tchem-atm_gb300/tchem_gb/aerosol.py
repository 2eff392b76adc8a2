"""Gas-aerosol chemistry: the aerosol model handle and the batched SIMPOL.1 time advance.

Reference interfaces mirrored (names and argument order):
  TChem::AerosolModelData (src/core/TChem_AerosolModelData.hpp:30-80): the aerosol species with
      their molecular weights, densities and kappa, the number of computational particles, the
      SIMPOL_PHASE_TRANSFER entries, setNumberofParticles and scenarioConditionParticles;
  TChem::AerosolChemistry::getWorkSpaceSize(kmcd, amcd), runDeviceBatch(policy, tol_newton,
      tol_time, fac, tadv, state, number_conc, t_out, dt_out, state_out, team_conf, kmcd, amcd),
      runHostBatch(...)                   src/core/TChem_AerosolChemistry.hpp:51-103
The aerosol problem's ODE vector is [active gas species, particle 0's aerosol species, particle
1's, ...]; its state row is [rho, p, T, active gas, constant gas, particles]. The advance is the
engine's CUDA kernel behind the C ABI (tchem_gb_aero_time_advance); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _capi
from .atmospheric_chemistry import _ptr, _stream_ptr, _torch
from .e3sm import _check_tensors
from .mechanism import KineticModel, set_scenario_conditions


class AerosolModel:
    """Owns a tchem_gb_aero handle. Construct with ``from_file`` or ``from_string`` next to the
    gas KineticModel it refers to (which must outlive it)."""

    def __init__(self, handle: int, gas: KineticModel):
        self._h = C.c_void_p(handle)
        self.gas = gas
        self._refresh()

    def _refresh(self):
        v = _capi.AeroView()
        _capi.check(_capi.lib().tchem_gb_aero_host_view(self._h, C.byref(v)), "tchem_gb_aero_host_view")
        self._view = v
        self.nSpec, self.nSpec_gas, self.nConstSpec_gas = v.nSpec, v.nSpec_gas, v.nConstSpec_gas
        self.nParticles, self.nSimpol = v.nParticles, v.nSimpol
        buf = C.create_string_buffer(256)
        names = []
        for i in range(self.nSpec):
            _capi.check(_capi.lib().tchem_gb_aero_species_name(self._h, i, buf, 256), "tchem_gb_aero_species_name")
            names.append(buf.value.decode())
        self.species_names = names

    @classmethod
    def from_file(cls, yaml_path: str | Path, gas: KineticModel) -> "AerosolModel":
        h = C.c_void_p()
        _capi.check(_capi.lib().tchem_gb_aero_create_from_file(str(yaml_path).encode(), gas.handle, C.byref(h)),
                    "tchem_gb_aero_create_from_file")
        return cls(h.value, gas)

    @classmethod
    def from_string(cls, text: str, gas: KineticModel) -> "AerosolModel":
        h = C.c_void_p()
        _capi.check(_capi.lib().tchem_gb_aero_create_from_string(text.encode(), gas.handle, C.byref(h)),
                    "tchem_gb_aero_create_from_string")
        return cls(h.value, gas)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def view(self) -> _capi.AeroView:
        return self._view

    @property
    def n_ode(self) -> int:
        return self.nSpec_gas + self.nSpec * self.nParticles

    @property
    def state_dim(self) -> int:
        return 3 + self.gas.nSpec + self.nSpec * self.nParticles

    def set_number_of_particles(self, n: int) -> None:
        _capi.check(_capi.lib().tchem_gb_aero_set_number_of_particles(self._h, int(n)),
                    "tchem_gb_aero_set_number_of_particles")
        self._refresh()

    def simpol_table(self) -> tuple[np.ndarray, np.ndarray]:
        """(index [nSimpol, 3]: aerosol ODE index, gas index, compute_alpha;
        param [nSimpol, 7]: B1..B4, diffusion coeff, N star, gas molecular weight)."""
        n = self.nSimpol
        if n == 0:
            return np.zeros((0, 3), np.int32), np.zeros((0, 7))
        idx = np.ctypeslib.as_array(self._view.simpol_index, shape=(3 * n,)).reshape(n, 3).copy()
        par = np.ctypeslib.as_array(self._view.simpol_param, shape=(7 * n,)).reshape(n, 7).copy()
        return idx, par

    def scenario(self, gas_yaml: str | Path, particles_yaml: str | Path) -> tuple[np.ndarray, np.ndarray]:
        """(state [B, state_dim], number_conc [B, nParticles]): the gas scenario
        (setScenarioConditions) and the particles' (scenarioConditionParticles)."""
        gas_state = set_scenario_conditions(gas_yaml, self.gas)
        B = gas_state.shape[0]
        state = np.zeros((B, self.state_dim))
        state[:, :gas_state.shape[1]] = gas_state
        nc = np.zeros((B, max(self.nParticles, 1)))
        found = C.c_int(0)
        _capi.check(_capi.lib().tchem_gb_aero_scenario_particles(
            str(particles_yaml).encode(), self._h, B, nc.ctypes.data_as(C.c_void_p),
            state.ctypes.data_as(C.c_void_p), self.state_dim, C.byref(found)), "tchem_gb_aero_scenario_particles")
        return state, nc

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().tchem_gb_aero_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


class AerosolChemistry:
    """Batched TR-BDF2 advance of the gas-aerosol problem (TChem::AerosolChemistry), plain FP64."""

    @staticmethod
    def getWorkSpaceSize(kmcd: KineticModel, amcd: AerosolModel, nbatch: int = 1) -> int:
        n = _capi.lib().tchem_gb_aero_workspace_bytes(kmcd.handle, amcd.handle, int(nbatch))
        if n == 0:
            _capi.check(1, "tchem_gb_aero_workspace_bytes")
        return int(n)

    @staticmethod
    def runDeviceBatch(tol_newton, tol_time, fac, tadv, state, number_conc, t_out, dt_out, state_out,
                       kmcd: KineticModel, amcd: AerosolModel, *, status=None, stats=None, workspace=None,
                       stream=None):
        """Advances every sample whose t_out < tadv.tend; returns the status tensor.
        tol_time [n_ode, 2], state / state_out [B, state_dim] (may be the same tensor),
        number_conc [B, nParticles]: contiguous float64 CUDA tensors; tadv on the device
        (tadv_to_device); fac is not read (the Jacobian's difference step is fixed)."""
        torch = _torch()
        _check_tensors(tol_newton, tol_time, state, number_conc, t_out, dt_out, state_out)
        B = int(state.shape[0])
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=state.device)
        ws_ptr, ws_bytes = C.c_void_p(0), 0
        if workspace is not None:
            ws_ptr, ws_bytes = _ptr(workspace), workspace.numel() * workspace.element_size()
        rc = _capi.lib().tchem_gb_aero_time_advance(
            kmcd.handle, amcd.handle, B, _ptr(tol_newton), _ptr(tol_time), _ptr(fac), _ptr(tadv), _ptr(state),
            _ptr(number_conc), _ptr(t_out), _ptr(dt_out), _ptr(state_out), _ptr(status), _ptr(stats), ws_ptr,
            ws_bytes, _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_aero_time_advance")
        return status

    @staticmethod
    def runHostBatch(tol_newton, tol_time, tadv: np.ndarray, state: np.ndarray, number_conc: np.ndarray,
                     t_out: np.ndarray, kmcd: KineticModel, amcd: AerosolModel):
        """Host-array variant (runHostBatch): copies in, advances on the GPU, copies out
        (synchronous). Returns (state_out, t_out, dt_out, status) as numpy arrays."""
        torch = _torch()
        from .atmospheric_chemistry import tadv_to_device
        dev = torch.device("cuda", torch.cuda.current_device())

        def d(a):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        d_state = d(state)
        out = d_state.clone()  # rows the advance does not write (skipped samples) come back unchanged
        t = d(t_out)
        dt = torch.zeros_like(t)
        status = AerosolChemistry.runDeviceBatch(d(tol_newton), d(tol_time), None, tadv_to_device(tadv, dev), d_state,
                                                 d(number_conc), t, dt, out, kmcd, amcd)
        torch.cuda.synchronize(dev)
        return out.cpu().numpy(), t.cpu().numpy(), dt.cpu().numpy(), status.cpu().numpy()


class AerosolRHS:
    """The aerosol problem's right-hand side omega[B, n_ode] at each sample's state row
    (src/core/impl/TChem_Impl_Aerosol_RHS.hpp:57-100)."""

    @staticmethod
    def runDeviceBatch(state, number_conc, omega, kmcd: KineticModel, amcd: AerosolModel, *, stream=None):
        _check_tensors(state, number_conc, omega)
        rc = _capi.lib().tchem_gb_aero_rhs(kmcd.handle, amcd.handle, int(state.shape[0]), _ptr(state),
                                           _ptr(number_conc), _ptr(omega), _stream_ptr(stream))
        _capi.check(rc, "tchem_gb_aero_rhs")
        return omega
