"""ctypes binding of libtchem_gb.so (declarations in include/tchem_gb.h).

The library is loaded from this package directory; there is no fallback: if it is missing
the import fails with the build command to run.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libtchem_gb.so"

# numpy mirrors of the C structs -------------------------------------------------------------
TIME_ADVANCE_DTYPE = np.dtype(
    [("tbeg", "<f8"), ("tend", "<f8"), ("dt", "<f8"), ("dtmin", "<f8"), ("dtmax", "<f8"),
     ("max_num_newton_iterations", "<i4"), ("num_time_iterations_per_interval", "<i4"),
     ("num_outer_time_iterations_per_interval", "<i4"), ("jacobian_interval", "<i4")],
    align=True)
assert TIME_ADVANCE_DTYPE.itemsize == 56

SAMPLE_STATS_DTYPE = np.dtype(
    [("n_steps", "<i4"), ("n_rejected", "<i4"), ("n_newton_fail", "<i4"), ("n_newton_iter", "<i4"),
     ("n_lu", "<i4"), ("n_solve", "<i4"), ("n_rhs", "<i4"), ("n_jac", "<i4")])
assert SAMPLE_STATS_DTYPE.itemsize == 32


class KmcdView(C.Structure):
    _fields_ = [
        ("nSpec", C.c_int32), ("nConstSpec", C.c_int32), ("nReac", C.c_int32), ("maxSpecInReac", C.c_int32),
        ("M_index", C.c_int32), ("CONV_PPM", C.c_double),
        ("reacNreac", C.POINTER(C.c_int32)), ("reacNprod", C.POINTER(C.c_int32)),
        ("reacSidx", C.POINTER(C.c_int32)), ("reacNuki", C.POINTER(C.c_double)),
        ("convExponent", C.POINTER(C.c_int32)), ("reacType", C.POINTER(C.c_int32)),
        ("nArrhenius", C.c_int32), ("arrhenius_reaction", C.POINTER(C.c_int32)),
        ("arrhenius_param", C.POINTER(C.c_double)),
        ("nTroe", C.c_int32), ("reacPfal", C.POINTER(C.c_int32)), ("reacPpar", C.POINTER(C.c_double)),
        ("nCMAQ_H2O2", C.c_int32), ("cmaq_reaction", C.POINTER(C.c_int32)), ("cmaq_param", C.POINTER(C.c_double)),
        ("nEmission", C.c_int32), ("emission_species", C.POINTER(C.c_int32)),
        ("emission_rate", C.POINTER(C.c_double)),
    ]


class E3smView(C.Structure):
    _fields_ = [
        ("nJPL", C.c_int32), ("jpl_reaction", C.POINTER(C.c_int32)), ("jpl_param", C.POINTER(C.c_double)),
        ("nRJPL", C.c_int32), ("rjpl_reaction", C.POINTER(C.c_int32)), ("rjpl_param", C.POINTER(C.c_double)),
        ("nAdjust", C.c_int32), ("adjust_pair", C.POINTER(C.c_int32)),
        ("nProdO1D", C.c_int32), ("o1d_index", C.POINTER(C.c_int32)), ("o1d_param", C.POINTER(C.c_double)),
    ]


class AeroView(C.Structure):
    _fields_ = [
        ("nSpec", C.c_int32), ("nSpec_gas", C.c_int32), ("nConstSpec_gas", C.c_int32), ("nParticles", C.c_int32),
        ("nSimpol", C.c_int32), ("molecular_weights", C.POINTER(C.c_double)),
        ("aerosol_density", C.POINTER(C.c_double)), ("aerosol_kappa", C.POINTER(C.c_double)),
        ("simpol_index", C.POINTER(C.c_int32)), ("simpol_param", C.POINTER(C.c_double)),
    ]


class Numerics(C.Structure):
    """tchem_gb_numerics: the solver settings of the host-model driver interface."""
    _fields_ = [("atol_newton", C.c_double), ("rtol_newton", C.c_double), ("dtmin", C.c_double),
                ("atol_time", C.c_double), ("rtol_time", C.c_double), ("max_newton_iterations", C.c_int32),
                ("max_num_time_iterations", C.c_int32), ("team_size", C.c_int32), ("vector_size", C.c_int32),
                ("verbose", C.c_int32)]


class AdvanceOpts(C.Structure):
    _fields_ = [("form", C.c_int32), ("threads_per_sample", C.c_int32), ("reserved", C.c_int32 * 6)]


class TChemGBError(RuntimeError):
    """Error returned by the engine's C ABI (message from tchem_gb_last_error)."""

    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where} failed (code {code}): {message}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the engine first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(str(LIB_PATH))
    vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double
    sig = {
        "tchem_gb_last_error": (C.c_char_p, []),
        "tchem_gb_abi_version": (C.c_int, []),
        "tchem_gb_mech_create_from_file": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(vp)]),
        "tchem_gb_mech_create_from_string": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "tchem_gb_mech_destroy": (None, [vp]),
        "tchem_gb_mech_host_view": (C.c_int, [vp, C.POINTER(KmcdView)]),
        "tchem_gb_mech_species_name": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int]),
        "tchem_gb_mech_sparse_lu": (C.c_int, [vp, vp, vp, C.c_int]),
        "tchem_gb_scenario_batch_size": (C.c_int, [C.c_char_p, C.POINTER(C.c_int)]),
        "tchem_gb_scenario_read": (C.c_int, [C.c_char_p, vp, vp, C.c_int]),
        "tchem_gb_mech_e3sm_view": (C.c_int, [vp, C.POINTER(E3smView)]),
        "tchem_gb_scenario_photolysis_rates": (C.c_int, [C.c_char_p, C.c_int, vp, C.POINTER(C.c_int)]),
        "tchem_gb_scenario_external_forcing": (C.c_int, [C.c_char_p, vp, C.c_int, vp, C.POINTER(C.c_int)]),
        "tchem_gb_aero_create_from_file": (C.c_int, [C.c_char_p, vp, C.POINTER(vp)]),
        "tchem_gb_aero_create_from_string": (C.c_int, [C.c_char_p, vp, C.POINTER(vp)]),
        "tchem_gb_aero_destroy": (None, [vp]),
        "tchem_gb_aero_host_view": (C.c_int, [vp, C.POINTER(AeroView)]),
        "tchem_gb_aero_set_number_of_particles": (C.c_int, [vp, C.c_int]),
        "tchem_gb_aero_species_name": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int]),
        "tchem_gb_aero_scenario_particles": (C.c_int, [C.c_char_p, vp, C.c_int, vp, vp, C.c_int,
                                                       C.POINTER(C.c_int)]),
    }
    popts = C.POINTER(AdvanceOpts)
    optional = {
        "tchem_gb_workspace_bytes": (C.c_size_t, [C.POINTER(vp), C.c_int, C.c_int, popts]),
        "tchem_gb_time_advance": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                            vp, vp, C.c_size_t, popts, vp]),
        "tchem_gb_time_advance_hostbuf": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp,
                                                    vp, vp, popts, vp]),
        "tchem_gb_device_error": (C.c_int, [vp, vp, C.POINTER(C.c_int32)]),
        "tchem_gb_time_advance_carry_over": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, vp, vp]),
        "tchem_gb_kernel_launches": (C.c_longlong, []),
        "tchem_gb_kforward": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp]),
        "tchem_gb_reaction_rates": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp]),
        "tchem_gb_jacobian": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, vp, vp, vp]),
        "tchem_gb_time_advance_record": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                                   C.c_int, vp]),
        "tchem_gb_adjoint_workspace_bytes": (C.c_size_t, [vp, C.c_int]),
        "tchem_gb_autotune": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_size_t, vp,
                                        C.POINTER(C.c_int), C.POINTER(C.c_float)]),
        "tchem_gb_mech_set_threads_per_sample": (C.c_int, [vp, C.c_int, C.c_int]),
        "tchem_gb_adjoint": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp,
                                       C.c_size_t, vp]),
        "tchem_gb_e3sm_reaction_rates": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, vp, vp]),
        "tchem_gb_e3sm_rate_of_progress": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, vp, vp]),
        "tchem_gb_e3sm_net_production_rates": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, vp, vp, vp]),
        "tchem_gb_e3sm_workspace_bytes": (C.c_size_t, [vp, C.c_int, popts]),
        "tchem_gb_e3sm_time_advance": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp,
                                                 vp, vp, C.c_size_t, popts, vp]),
        "tchem_gb_aero_workspace_bytes": (C.c_size_t, [vp, vp, C.c_int]),
        "tchem_gb_aero_time_advance": (C.c_int, [vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                                 vp, C.c_size_t, vp]),
        "tchem_gb_aero_rhs": (C.c_int, [vp, vp, C.c_int, vp, vp, vp, vp]),
        "tchem_gb_numerics_read": (C.c_int, [C.c_char_p, C.POINTER(Numerics)]),
        "tchem_gb_tc_tile_update_tf32": (C.c_int, [C.c_int, C.c_int, vp, vp, vp, vp]),
        "tchem_gb_tc_lu_factor_tf32": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    for name, (res, args) in optional.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    _ = (i32, dbl)
    _lib = L
    return L


def check(code: int, where: str) -> None:
    if code != 0:
        msg = lib().tchem_gb_last_error()
        raise TChemGBError(code, where, msg.decode() if msg else "")
