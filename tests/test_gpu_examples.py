"""The example drivers (tchem_gb.examples) through the engine on the GPU, with the reference's gtest
command lines: the box-model driver against the CB05CL_AE5 golden (compare_tchem <= 1e-8) and the
E3SM driver against the uci_col golden (within 10 step-tolerance units per species; the reference's
file criterion measures 1.0e-6 as for the CPU restatement in tests/test_examples.py)."""
from __future__ import annotations

import numpy as np
import pytest

pytest.importorskip("torch")

from helpers import GOLDEN, compare_files_values, compare_tchem, mech_path, tolerance_units  # noqa: E402
from tchem_gb.examples import atmospheric_chemistry, atmospheric_chemistry_e3sm  # noqa: E402
from test_examples import CB05_ARGS, UCI_COL_ARGS  # noqa: E402

pytestmark = pytest.mark.gpu


def test_box_example_on_the_engine(tmp_path):
    out = tmp_path / "full_gas.dat"
    assert atmospheric_chemistry.main([f"--chemfile={mech_path('cb05cl_ae5.yaml')}", f"--outputfile={out}",
                                       f"--outputfile_times={tmp_path / 't.json'}", "--form=plain", *CB05_ARGS]) == 0
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(GOLDEN / "cb05cl_ae5_full_gas.npy")
    assert rows.shape == golden.shape
    assert compare_tchem(rows, golden) <= 1e-8


def test_e3sm_example_on_the_engine(tmp_path):
    out = tmp_path / "full_gas.dat"
    assert atmospheric_chemistry_e3sm.main([f"--chemfile={mech_path('uci_v2_test3.yaml')}",
                                            f"--inputfile={GOLDEN / 'e3sm' / 'uci_col_input_conditions.yaml'}",
                                            f"--outputfile={out}", f"--outputfile_times={tmp_path / 't.json'}",
                                            "--form=plain", *UCI_COL_ARGS]) == 0
    rows = np.genfromtxt(out, skip_header=1)
    golden = np.load(GOLDEN / "e3sm" / "uci_col_full_gas.npy")
    assert rows.shape == golden.shape
    np.testing.assert_allclose(rows[:80], golden[:80], rtol=1e-10, atol=0)
    assert compare_files_values(rows[80:, 3:], golden[80:, 3:]) <= 2e-6
    assert tolerance_units(rows[80:, 6:59], golden[80:, 6:59], 1e-12, 1e-6).max() <= 10.0
