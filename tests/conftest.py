"""Test configuration: markers, import paths, and one-time builds of the engine and the oracle."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "tchem-atm_gb300", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the engine's kernels")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds libtchem_gb.so and the oracle when missing or stale (nvcc cross-compiles without a GPU)."""
    from tchem_gb import build as engine_build
    from oracle import build as oracle_build
    engine_build.build()
    oracle_build.build()
    yield
