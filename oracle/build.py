"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.cpp into oracle/liboracle.so with g++ and OpenMP. FP contraction is
disabled so the x86 and Arm builds round identically.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"


def build(force: bool = False) -> Path:
    src = ORACLE_DIR / "oracle.cpp"
    deps = [src, ORACLE_DIR / "oracle.h", ORACLE_DIR.parent / "include" / "tchem_gb.h"]
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return LIB_PATH
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler found for the oracle")
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall", str(src), "-o",
           str(LIB_PATH)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
