"""Shared test utilities: fixture loading, the reference's host time loop and its comparison norms."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def manifest() -> dict:
    return json.loads((GOLDEN / "manifest.json").read_text())


def mech_path(name: str) -> Path:
    return GOLDEN / "mechanisms" / name


def compare_tchem(test: np.ndarray, ref: np.ndarray) -> float:
    """Largest of the per-column L1/L2/Linf norms of (test - ref) divided by the column's L2
    norm (floored at 1e-23), the criterion of src/unit-tests/scripts/compare_tchem.py:8-77."""
    diff = test - ref
    den = np.linalg.norm(ref, 2, axis=0)
    den = np.where(den > 1e-23, den, 1.0)
    worst = 0.0
    for ordn in (1, 2, np.inf):
        e = np.linalg.norm(diff, ordn, axis=0) / den
        e = np.where(np.all(diff == 0, axis=0), 0.0, e)
        worst = max(worst, float(e.max()))
    return worst


def rel_error(test: np.ndarray, ref: np.ndarray, floor: float) -> np.ndarray:
    """Elementwise |test - ref| / max(|ref|, floor)."""
    return np.abs(test - ref) / np.maximum(np.abs(ref), floor)


def host_time_loop(advance, state: np.ndarray, tadv: np.ndarray, tend: float, max_intervals: int, dtmax: float):
    """The reference box model's host loop (src/examples/TChem_AtmosphericChemistry.cpp:312-352):
    calls `advance(tadv, state, t) -> (state, t, dt)` until the mean t exceeds 0.9999 tend,
    carrying t and dt into tadv. Returns the rows (iter, t, dt, state...) of sample 0."""
    B = state.shape[0]
    t = np.array(tadv["tbeg"], dtype=np.float64)
    dt = np.full(B, dtmax)
    rows = [np.concatenate([[-1, t[0], dt[0]], state[0]])]
    it = 0
    tsum = 0.0
    while it < max_intervals and tsum <= tend * 0.9999:
        state, t, dt = advance(tadv, state, t)
        rows.append(np.concatenate([[it, t[0], dt[0]], state[0]]))
        tadv["tbeg"] = t
        tadv["dt"] = dt
        tsum = float(np.mean(t))
        it += 1
    return np.array(rows), state


def printed(x) -> np.ndarray:
    """Values as the reference's example drivers write them (%15.10e) and read back."""
    return np.vectorize(lambda v: float(f"{v:15.10e}"))(np.asarray(x, dtype=np.float64))


def compare_files_values(test: np.ndarray, ref: np.ndarray) -> float:
    """The criterion of TChem::Test::compareFilesValues (src/core/TChem_Util.hpp:1130-1180) on two
    written files: the relative error |test - ref| / ref at the element with the largest absolute
    difference. Pass both as written (printed()); comparing full-precision values with printed ones
    instead measures the printing rounding of the largest values."""
    d = np.abs(np.asarray(test, dtype=np.float64) - np.asarray(ref, dtype=np.float64))
    i = np.unravel_index(int(d.argmax()), d.shape)
    return float(d[i] / abs(ref[i])) if d[i] > 0 else 0.0


def format_reaction_rates(values, n: int) -> str:
    """Text of TChem::Test::writeReactionRates (src/core/TChem_Util.hpp:1036-1049): a header
    naming n and the vector length, then 'index   value' lines in std::scientific (6 digits)."""
    return f"## nSpec({n})    Omega({len(values)})\n" + "".join(f"{i}   {v:e}\n" for i, v in enumerate(values))


def format_2d_matrix(mat: np.ndarray) -> str:
    """Text of TChem::Test::write2DMatrix (src/core/TChem_Util.hpp:1098-1118): two header lines, then
    each row's values in std::scientific, each followed by one space."""
    r, c = mat.shape
    return (f"## nRows({r})    ({r})\n## nCols({c})    ({c})\n" +
            "".join("".join(f"{v:e} " for v in row) + "\n" for row in mat))


def tolerance_units(test: np.ndarray, ref: np.ndarray, atol: float, rtol: float) -> np.ndarray:
    """|test - ref| in units of the time-step tolerance atol + rtol |ref|."""
    return np.abs(test - ref) / (atol + rtol * np.abs(ref))
