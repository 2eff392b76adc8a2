"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.cpp with g++ and OpenMP into
  liboracle.so         the accuracy reference: FP contraction disabled, so the x86 and Arm builds
                       round identically;
  liboracle_native.so  the timed CPU baseline: tuned for the host CPU (-march=native on x86,
                       -mcpu=native on Arm) with contraction allowed.
"""
from __future__ import annotations

import platform
import shutil
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"
NATIVE_LIB_PATH = ORACLE_DIR / "liboracle_native.so"


def _native_flags() -> list[str]:
    return ["-mcpu=native"] if platform.machine().lower() in ("aarch64", "arm64") else ["-march=native"]


def build(force: bool = False, native: bool = False) -> Path:
    out = NATIVE_LIB_PATH if native else LIB_PATH
    src = ORACLE_DIR / "oracle.cpp"
    deps = [src, ORACLE_DIR / "oracle.h", ORACLE_DIR.parent / "include" / "tchem_gb.h"]
    if not force and out.exists() and out.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return out
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler found for the oracle")
    flags = _native_flags() if native else ["-ffp-contract=off"]
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", *flags, "-Wall", str(src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build(force="--force" in sys.argv, native=True))
