"""The engine's front end against a second, independent reading of the same mechanism files
(oracle/mechanism_text.py: its own YAML-subset reader and a numpy restatement of initChemNCAR's
table rules, KForwardAerosol and ReactionRatesAerosol). The CPU oracle computes on the tables the
engine's parser builds, so this is what pins the parser and the generated encodings (Troe,
photolysis as ARRHENIUS with A = J) independently: species order, stoichiometry layout,
convExponent and rate parameters must be equal, and the oracle's rate constants and net production
rates must match the independent ones at random states."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import mech_path
from oracle import Oracle
from oracle.mechanism_text import kforward, net_production, tables
from tchem_gb import KineticModel
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states

CASES = {
    "generated_51": lambda: mechanism_yaml(MechanismSpec()),
    "generated_51_night": lambda: mechanism_yaml(MechanismSpec(), night=True),
    "generated_120": lambda: mechanism_yaml(MechanismSpec(n_species=120, n_reactions=330, seed=20251204)),
    "generated_300": lambda: mechanism_yaml(MechanismSpec(n_species=300, n_reactions=1000, seed=20251205)),
    "cb05cl_ae5": lambda: mech_path("cb05cl_ae5.yaml").read_text(),
    "troe": lambda: mech_path("troe.yaml").read_text(),
    "arrhenius": lambda: mech_path("arrhenius.yaml").read_text(),
    "photolysis": lambda: mech_path("photolysis.yaml").read_text(),
    "cmaq_h2o2": lambda: mech_path("cmaq_h2o2.yaml").read_text(),
    "emission": lambda: mech_path("emission.yaml").read_text(),
}


def _view_arrays(km):
    v = km.view
    R, S = v.nReac, v.maxSpecInReac
    arr = lambda p, n: np.ctypeslib.as_array(p, (n,)).copy() if n > 0 else np.zeros(0, dtype=np.int32)  # noqa: E731
    return (R, S, arr(v.reacNreac, R), arr(v.reacNprod, R), arr(v.reacSidx, R * S).reshape(R, S),
            arr(v.reacNuki, R * S).reshape(R, S), arr(v.convExponent, R))


@pytest.mark.parametrize("case", sorted(CASES))
def test_engine_tables_match_the_independent_reading(case):
    text = CASES[case]()
    km = KineticModel.from_string(text)
    tb = tables(text)
    assert km.species_names == tb["names"]
    assert km.n_active == tb["n_active"] and km.view.nConstSpec == tb["n_const"]
    assert km.view.M_index == tb["M_index"]
    R, S, nreac, nprod, sidx, nuki, conv = _view_arrays(km)
    assert R == len(tb["rate"]) and S == tb["S"]
    np.testing.assert_array_equal(nreac, tb["nreac"])
    np.testing.assert_array_equal(nprod, tb["nprod"])
    np.testing.assert_array_equal(conv, tb["conv_exp"])
    v = km.view
    emis = np.zeros(km.nSpec)
    if v.nEmission > 0:
        sp = np.ctypeslib.as_array(v.emission_species, (v.nEmission,))
        rt = np.ctypeslib.as_array(v.emission_rate, (v.nEmission,))
        np.add.at(emis, sp, rt)
    np.testing.assert_array_equal(emis, tb["emis"])
    for r in range(R):
        n_r, n_p = tb["nreac"][r], tb["nprod_found"][r]
        np.testing.assert_array_equal(sidx[r, :n_r], tb["sidx"][r, :n_r])
        np.testing.assert_array_equal(nuki[r, :n_r], tb["nuki"][r, :n_r])
        np.testing.assert_array_equal(sidx[r, S // 2:S // 2 + n_p], tb["sidx"][r, S // 2:S // 2 + n_p])
        np.testing.assert_array_equal(nuki[r, S // 2:S // 2 + n_p], tb["nuki"][r, S // 2:S // 2 + n_p])


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_rates_match_the_independent_reading(case):
    text = CASES[case]()
    km = KineticModel.from_string(text)
    tb = tables(text)
    o = Oracle([km])
    m = km.n_active
    states = sample_states(8, m, n_const=km.view.nConstSpec, seed=17,
                           const_values=tuple([1.0e6] * km.view.nConstSpec))
    for st in states:
        T, p, x = st[2], st[1], st[3:3 + km.nSpec]
        k_ref = kforward(tb, T, p)
        k_or = o.kforward(T, p)
        np.testing.assert_allclose(k_or, k_ref, rtol=1e-13, atol=0)
        w_ref = net_production(tb, T, p, x)
        w_or = o.reaction_rates(T, p, x)
        assert np.abs(w_or - w_ref).max() <= 1e-12 * max(np.abs(w_ref).max(), 1e-300)
