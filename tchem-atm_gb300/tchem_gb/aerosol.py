"""Aerosol model handle: SIMPOL.1 gas-particle phase transfer over a parsed gas mechanism.

Mirrors TChem::AerosolModelData (src/core/TChem_AerosolModelData.hpp:30-80): the aerosol species
with their molecular weights, densities and kappa, the number of computational particles, the
SIMPOL_PHASE_TRANSFER entries, setNumberofParticles and scenarioConditionParticles. The aerosol
problem's ODE vector is [active gas species, particle 0's aerosol species, particle 1's, ...];
its state row is [rho, p, T, active gas, constant gas, particles].
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _capi
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
