"""Python face of the host-model driver interface (include/tchem_gb_driver.h,
libtchem_gb_driver.so): the reference's TChem_Driver functions (src/core/TChem_Driver.hpp:106-132)
that a host model such as PartMC binds, one driver per process.

  d = Driver(gas_yaml, aero_yaml, solver_yaml, n_batch)
  d.set_state(row, i); d.set_number_concentration(nc, i); d.do_timestep(30.0); d.state(i)

TChem_doTimestep runs the engine's gas-aerosol TR-BDF2 kernel on the current CUDA device.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _capi

DRIVER_LIB_PATH = Path(__file__).resolve().parent / "libtchem_gb_driver.so"
_lib = None


def lib() -> C.CDLL:
    """Loads libtchem_gb_driver.so (after libtchem_gb.so, which it links) and sets the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    _capi.lib()
    if not DRIVER_LIB_PATH.exists():
        raise RuntimeError(f"{DRIVER_LIB_PATH} is missing: build the engine first (tchem_gb.build.build())")
    L = C.CDLL(str(DRIVER_LIB_PATH))
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "initialize": (None, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]),
        "finalize": (None, []),
        "TChem_getNumberOfSpecies": (C.c_int, []),
        "TChem_getLengthOfStateVector": (C.c_int, []),
        "TChem_getStateVectorSize": (C.c_int, []),
        "TChem_getStateVector": (None, [vp, C.c_int]),
        "TChem_setStateVector": (None, [vp, C.c_int]),
        "TChem_getAllStateVectorHost": (None, [vp]),
        "TChem_getSpeciesName": (C.c_int, [ip, C.c_char_p, C.c_size_t]),
        "TChem_getNumberConcentrationVectorSize": (C.c_int, []),
        "TChem_setNumberConcentrationVector": (None, [vp, C.c_int]),
        "TChem_getNumberOfAeroSpecies": (C.c_int, []),
        "TChem_getAerosolSpeciesName": (C.c_int, [ip, C.c_char_p, C.c_size_t]),
        "TChem_getAerosolSpeciesDensity": (C.c_double, [ip]),
        "TChem_getAerosolSpeciesMW": (C.c_double, [ip]),
        "TChem_getAerosolSpeciesKappa": (C.c_double, [ip]),
        "TChem_doTimestep": (None, [dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    _lib = L
    return L


def _vec(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Driver:
    """initialize() on construction, finalize() on close()."""

    def __init__(self, gas_yaml, aero_yaml, solver_yaml, n_batch: int = 1):
        L = lib()
        L.initialize(str(gas_yaml).encode(), str(aero_yaml).encode(), str(solver_yaml).encode(), int(n_batch))
        self.n_batch = int(n_batch)
        self.length = L.TChem_getLengthOfStateVector()
        if self.length < 0:
            raise RuntimeError("initialize failed: " + _capi.lib().tchem_gb_last_error().decode())
        self.n_particles = L.TChem_getNumberConcentrationVectorSize()

    @staticmethod
    def _name(f, i: int) -> str:
        buf = C.create_string_buffer(256)
        idx = C.c_int(i)
        f(C.byref(idx), buf, 256)
        return buf.value.decode()

    def species_names(self) -> list[str]:
        L = lib()
        return [self._name(L.TChem_getSpeciesName, i) for i in range(L.TChem_getNumberOfSpecies())]

    def aerosol_species(self) -> list[tuple[str, float, float, float]]:
        """(name, density, molecular weight, kappa) per aerosol species."""
        L = lib()
        out = []
        for i in range(L.TChem_getNumberOfAeroSpecies()):
            idx = C.c_int(i)
            out.append((self._name(L.TChem_getAerosolSpeciesName, i), L.TChem_getAerosolSpeciesDensity(C.byref(idx)),
                        L.TChem_getAerosolSpeciesMW(C.byref(idx)), L.TChem_getAerosolSpeciesKappa(C.byref(idx))))
        return out

    def set_state(self, row, i: int = 0) -> None:
        a = _vec(row)
        assert a.size == self.length
        lib().TChem_setStateVector(a.ctypes.data_as(C.c_void_p), int(i))

    def state(self, i: int = 0) -> np.ndarray:
        a = np.zeros(self.length)
        lib().TChem_getStateVector(a.ctypes.data_as(C.c_void_p), int(i))
        return a

    def all_states(self) -> np.ndarray:
        a = np.zeros((self.n_batch, self.length))
        lib().TChem_getAllStateVectorHost(a.ctypes.data_as(C.c_void_p))
        return a

    def set_number_concentration(self, nc, i: int = 0) -> None:
        a = _vec(nc)
        assert a.size == self.n_particles
        lib().TChem_setNumberConcentrationVector(a.ctypes.data_as(C.c_void_p), int(i))

    def do_timestep(self, del_t: float) -> None:
        v = C.c_double(float(del_t))
        lib().TChem_doTimestep(C.byref(v))

    def close(self) -> None:
        lib().finalize()
