"""C-ABI argument checking without a GPU: bad arguments come back as TCHEM_GB_ERR_ARG with a
message, before any device work."""
from __future__ import annotations

import ctypes as C

from tchem_gb import KineticModel, _capi
from tchem_gb.generator import MechanismSpec, mechanism_yaml

ERR_ARG = 1
ERR_UNSUPPORTED = 4


def _km():
    return KineticModel.from_string(mechanism_yaml(MechanismSpec(n_species=20, n_reactions=40, seed=5)))


def test_threads_per_sample_preference_is_checked():
    L = _capi.lib()
    km = _km()
    assert L.tchem_gb_mech_set_threads_per_sample(km.handle, 2, 64) == 0
    assert L.tchem_gb_mech_set_threads_per_sample(km.handle, 2, 0) == 0
    assert L.tchem_gb_mech_set_threads_per_sample(km.handle, 2, 48) == ERR_ARG
    assert L.tchem_gb_mech_set_threads_per_sample(km.handle, 7, 32) == ERR_ARG
    assert L.tchem_gb_mech_set_threads_per_sample(None, 0, 32) == ERR_ARG


def test_adjoint_and_record_reject_missing_arrays():
    L = _capi.lib()
    km = _km()
    nul = C.c_void_p(0)
    rc = L.tchem_gb_adjoint(km.handle, 4, nul, nul, nul, nul, nul, nul, nul, 16, nul, nul, nul, nul, nul, 0, nul)
    assert rc == ERR_ARG and b"null" in L.tchem_gb_last_error()
    assert L.tchem_gb_adjoint(km.handle, 0, nul, nul, nul, nul, nul, nul, nul, 16, nul, nul, nul, nul, nul, 0,
                              nul) == 0  # empty batch
    rc = L.tchem_gb_time_advance_record(km.handle, 4, nul, nul, nul, nul, nul, nul, nul, nul, nul, nul, nul, nul,
                                        nul, 0, nul)
    assert rc == ERR_ARG and b"tape_cap" in L.tchem_gb_last_error()


def test_autotune_and_noalloc_reject_bad_arguments():
    L = _capi.lib()
    km = _km()
    nul = C.c_void_p(0)
    chosen = C.c_int(0)
    assert L.tchem_gb_autotune(km.handle, 5, 8, nul, nul, nul, nul, nul, nul, nul, nul, nul, 0, nul,
                               C.byref(chosen), None) == ERR_ARG
    assert L.tchem_gb_autotune(km.handle, 2, 0, nul, nul, nul, nul, nul, nul, nul, nul, nul, 0, nul,
                               C.byref(chosen), None) == ERR_ARG
    f = L.tchem_gb_time_advance_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 10 + \
        [C.POINTER(_capi.AdvanceOpts), C.c_void_p]
    assert f(None, 1, None, 4, *([None] * 10), None, None) == ERR_ARG
    handles = (C.c_void_p * 1)(km.handle.value)
    assert f(handles, 1, None, 0, *([None] * 10), None, None) == 0  # empty batch: nothing to do


def test_e3sm_entry_points_reject_bad_arguments():
    L = _capi.lib()
    km = _km()
    nul = C.c_void_p(0)
    buf = C.c_void_p(1 << 20)  # never dereferenced: every call below returns before device work
    for name in ("tchem_gb_e3sm_reaction_rates", "tchem_gb_e3sm_rate_of_progress"):
        f = getattr(L, name)
        assert f(km.handle, -1, buf, nul, 0, buf, nul) == ERR_ARG
        assert f(km.handle, 4, buf, nul, 3, buf, nul) == ERR_ARG  # n_photo > 0 without photolysis rates
        assert f(km.handle, 4, nul, nul, 0, buf, nul) == ERR_ARG and b"null" in L.tchem_gb_last_error()
        assert f(None, 4, buf, nul, 0, buf, nul) == ERR_ARG
        assert f(km.handle, 0, nul, nul, 0, nul, nul) == 0  # empty batch
    f = L.tchem_gb_e3sm_net_production_rates
    assert f(km.handle, 4, buf, nul, 0, nul, nul, nul) == ERR_ARG
    assert f(km.handle, 4, buf, nul, -1, nul, buf, nul) == ERR_ARG
    f = L.tchem_gb_e3sm_time_advance
    o = _capi.AdvanceOpts()
    assert f(km.handle, 4, *([nul] * 6), 0, nul, nul, nul, nul, nul, nul, nul, 0, C.byref(o), nul) == ERR_ARG
    assert f(km.handle, 4, *([buf] * 5), nul, 2, nul, *([buf] * 4), nul, nul, 0, C.byref(o), nul) == ERR_ARG
    assert f(None, 4, *([buf] * 6), 0, nul, *([buf] * 4), nul, nul, 0, C.byref(o), nul) == ERR_ARG
    assert f(km.handle, 0, *([nul] * 6), 0, nul, nul, nul, nul, nul, nul, nul, 0, C.byref(o), nul) == 0
    o.form = 9
    assert f(km.handle, 4, *([buf] * 6), 0, nul, *([buf] * 4), nul, nul, 0, C.byref(o), nul) == ERR_ARG


def test_aerosol_entry_points_reject_bad_arguments():
    """tchem_gb_aero_time_advance / _rhs / _workspace_bytes: host-side checks of the model pair
    (mechanism tables built on the host, including a mechanism without reactions) before any
    device work."""
    from helpers import GOLDEN
    from tchem_gb.aerosol import AerosolModel
    A = GOLDEN / "aerosol"
    L = _capi.lib()
    nul = C.c_void_p(0)
    gas = KineticModel.from_file(A / "simpol_config_gas.yaml")  # no gas reactions
    am = AerosolModel.from_file(A / "simpol_phase_transfer.yaml", gas)
    adv = L.tchem_gb_aero_time_advance
    assert adv(gas.handle, am.handle, 0, *([nul] * 12), 0, nul) == 0  # empty batch
    assert adv(gas.handle, am.handle, 4, *([nul] * 12), 0, nul) == ERR_ARG
    assert b"null" in L.tchem_gb_last_error()
    assert adv(nul, am.handle, 4, *([nul] * 12), 0, nul) == ERR_ARG
    assert L.tchem_gb_aero_rhs(gas.handle, am.handle, 0, nul, nul, nul, nul) == 0
    assert L.tchem_gb_aero_rhs(gas.handle, am.handle, 2, nul, nul, nul, nul) == ERR_ARG
    cb = KineticModel.from_file(A / "cb05_soa_config_full_gas.yaml")
    cb_am = AerosolModel.from_file(A / "cb05_soa_mechanism_aero.yaml", cb)
    assert adv(cb.handle, cb_am.handle, 0, *([nul] * 12), 0, nul) == 0
    assert adv(cb.handle, am.handle, 0, *([nul] * 12), 0, nul) == ERR_ARG  # model built on another gas mechanism
    assert b"another gas mechanism" in L.tchem_gb_last_error()
    assert L.tchem_gb_aero_workspace_bytes(cb.handle, am.handle, 4) == 0
    am.set_number_of_particles(200)  # 1 + 2 * 200 ODEs
    assert adv(gas.handle, am.handle, 4, *([nul] * 12), 0, nul) == ERR_UNSUPPORTED
    assert b"at most 320" in L.tchem_gb_last_error()
    # a SIMPOL gas species held constant: the transfer would change a constant species
    const_gas = KineticModel.from_string((A / "simpol_config_gas.yaml").read_text().replace(
        "constant_species:\n- description: tracer-CONSTANT\n  name: M\nspecies:\n- description: ETHANOL\n  name: ethanol",
        "constant_species:\n- description: tracer-CONSTANT\n  name: M\n- description: ETHANOL\n  name: ethanol\n"
        "species:\n- description: tracer\n  name: X"))
    assert const_gas.nConstSpec == 2
    const_am = AerosolModel.from_file(A / "simpol_phase_transfer.yaml", const_gas)
    assert adv(const_gas.handle, const_am.handle, 0, *([nul] * 12), 0, nul) == ERR_UNSUPPORTED
    assert b"not an active species" in L.tchem_gb_last_error()


def test_tensor_core_tile_update_checks_its_shape():
    L = _capi.lib()
    nul = C.c_void_p(0)
    assert L.tchem_gb_tc_tile_update_tf32(0, 64, nul, nul, nul, nul) == 0  # no tiles
    for n in (0, 8, 24, 272):
        assert L.tchem_gb_tc_tile_update_tf32(1, n, nul, nul, nul, nul) == ERR_ARG
    assert L.tchem_gb_tc_tile_update_tf32(2, 64, nul, nul, nul, nul) == ERR_ARG
    assert b"null" in L.tchem_gb_last_error()
    lu = L.tchem_gb_tc_lu_factor_tf32
    assert lu(0, 300, 304, nul, nul, nul, nul) == 0  # no matrices
    assert lu(1, 0, 1, nul, nul, nul, nul) == ERR_ARG
    assert lu(1, 300, 299, nul, nul, nul, nul) == ERR_ARG  # lda < m
    assert lu(4, 300, 304, nul, nul, nul, nul) == ERR_ARG and b"null" in L.tchem_gb_last_error()
