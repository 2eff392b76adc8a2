"""Kinetic model handle: NCAR-format YAML parsed by the engine's C++ front end.

Mirrors TChem::KineticModelData (src/core/TChem_KineticModelData.hpp:98-99) plus the const
data bundle of createNCAR_KineticModelConstData
(src/core/TChem_KineticModelNCAR_ConstData.hpp:115-148).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _capi


class KineticModel:
    """Owns a tchem_gb_mech handle. Construct with ``from_file`` or ``from_string``."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        v = _capi.KmcdView()
        _capi.check(_capi.lib().tchem_gb_mech_host_view(self._h, C.byref(v)), "tchem_gb_mech_host_view")
        self._view = v
        e = _capi.E3smView()
        _capi.check(_capi.lib().tchem_gb_mech_e3sm_view(self._h, C.byref(e)), "tchem_gb_mech_e3sm_view")
        self._e3sm_view = e
        self.nSpec = v.nSpec
        self.nConstSpec = v.nConstSpec
        self.nReac = v.nReac
        self.maxSpecInReac = v.maxSpecInReac
        self.M_index = v.M_index
        buf = C.create_string_buffer(64)
        names = []
        for i in range(self.nSpec):
            _capi.check(_capi.lib().tchem_gb_mech_species_name(self._h, i, buf, 64), "tchem_gb_mech_species_name")
            names.append(buf.value.decode())
        self.species_names = names

    @classmethod
    def from_file(cls, yaml_path: str | Path, echo_path: str | Path | None = None) -> "KineticModel":
        h = C.c_void_p()
        _capi.check(_capi.lib().tchem_gb_mech_create_from_file(
            str(yaml_path).encode(), None if echo_path is None else str(echo_path).encode(), C.byref(h)),
            "tchem_gb_mech_create_from_file")
        return cls(h.value)

    @classmethod
    def from_string(cls, text: str) -> "KineticModel":
        h = C.c_void_p()
        _capi.check(_capi.lib().tchem_gb_mech_create_from_string(text.encode(), C.byref(h)),
                    "tchem_gb_mech_create_from_string")
        return cls(h.value)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def view(self) -> _capi.KmcdView:
        """Reference-layout host tables (valid while this object lives)."""
        return self._view

    @property
    def e3sm_view(self) -> _capi.E3smView:
        """The E3SM rate tables (JPL, R_JPL_ARRHENIUS, adjust_reaction, prod_O1D), same lifetime."""
        return self._e3sm_view

    @property
    def n_active(self) -> int:
        return self.nSpec - self.nConstSpec

    @property
    def state_dim(self) -> int:
        return self.nSpec + 3

    def stoichiometry(self) -> tuple[np.ndarray, np.ndarray]:
        """(reacSidx, reacNuki) as [nReac, maxSpecInReac] arrays."""
        v = self._view
        n = self.nReac * self.maxSpecInReac
        sidx = np.ctypeslib.as_array(v.reacSidx, shape=(n,)).reshape(self.nReac, self.maxSpecInReac).copy()
        nuki = np.ctypeslib.as_array(v.reacNuki, shape=(n,)).reshape(self.nReac, self.maxSpecInReac).copy()
        return sidx, nuki

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().tchem_gb_mech_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


def scenario_batch_size(yaml_path: str | Path) -> int:
    n = C.c_int()
    _capi.check(_capi.lib().tchem_gb_scenario_batch_size(str(yaml_path).encode(), C.byref(n)),
                "tchem_gb_scenario_batch_size")
    return n.value


def set_scenario_conditions(yaml_path: str | Path, km: KineticModel) -> np.ndarray:
    """state[nBatch, nSpec+3] from a scenario file (AtmChemistry::setScenarioConditions)."""
    nb = scenario_batch_size(yaml_path)
    state = np.zeros((nb, km.state_dim), dtype=np.float64)
    _capi.check(_capi.lib().tchem_gb_scenario_read(str(yaml_path).encode(), km.handle,
                                                   state.ctypes.data_as(C.c_void_p), nb),
                "tchem_gb_scenario_read")
    return state


def set_scenario_photolysis_rates(yaml_path: str | Path, nbatch: int) -> np.ndarray:
    """photo_rates[nBatch, nPhoto] from a scenario file's photolysis_rates section
    (AtmChemistry::setScenarioConditionsPhotolysisReactions); nPhoto = 0 without one."""
    n = C.c_int()
    _capi.check(_capi.lib().tchem_gb_scenario_photolysis_rates(str(yaml_path).encode(), nbatch, None, C.byref(n)),
                "tchem_gb_scenario_photolysis_rates")
    photo = np.zeros((nbatch, n.value), dtype=np.float64)
    _capi.check(_capi.lib().tchem_gb_scenario_photolysis_rates(str(yaml_path).encode(), nbatch,
                                                               photo.ctypes.data_as(C.c_void_p), C.byref(n)),
                "tchem_gb_scenario_photolysis_rates")
    return photo


def set_scenario_external_forcing(yaml_path: str | Path, km: KineticModel, nbatch: int) -> np.ndarray:
    """external_sources[nBatch, m] from a scenario file's external_forcing section
    (AtmChemistry::setScenarioConditionsExternalForcing); zero where none is given."""
    ext = np.zeros((nbatch, km.n_active), dtype=np.float64)
    count = C.c_int()
    _capi.check(_capi.lib().tchem_gb_scenario_external_forcing(str(yaml_path).encode(), km.handle, nbatch,
                                                               ext.ctypes.data_as(C.c_void_p), C.byref(count)),
                "tchem_gb_scenario_external_forcing")
    return ext
