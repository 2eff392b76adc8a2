"""Builds libtchem_gb.so (the engine: sm_103a CUDA kernels + C ABI) in-tree, and beside it
libtchem_gb_driver.so (the host-model driver interface of include/tchem_gb_driver.h, host code
over libtchem_gb.so) and libtchem_gb_probe.so (the benchmark's FMA-throughput probe, kept out of
the engine library).

Translation units are compiled in parallel with nvcc and linked into
``tchem-atm_gb300/tchem_gb/libtchem_gb.so``. Nothing here depends on torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC_DIR = PKG_DIR.parent / "csrc"
BUILD_DIR = PKG_DIR.parent / "_build"
LIB_PATH = PKG_DIR / "libtchem_gb.so"
PROBE_LIB_PATH = PKG_DIR / "libtchem_gb_probe.so"  # the benchmark's FMA-peak probe, not the engine
PROBE_SRC = SRC_DIR / "probe" / "fma_peak.cu"
DRIVER_LIB_PATH = PKG_DIR / "libtchem_gb_driver.so"
DRIVER_DIR = SRC_DIR / "driver"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")
    return cand


def sources() -> list[Path]:
    return sorted(list(SRC_DIR.glob("*.cu")) + list(SRC_DIR.glob("*.cpp")))


def _compile(nvcc: str, src: Path, extra: list[str]) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, *extra, "-I", str(SRC_DIR), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, extra_flags: list[str] | None = None, force: bool = False) -> Path:
    """Compiles every translation unit and links the shared library; returns its path."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = sources()
    extra = list(extra_flags or [])
    driver_srcs = sorted(DRIVER_DIR.glob("*.cpp"))
    outs = (LIB_PATH, DRIVER_LIB_PATH, PROBE_LIB_PATH)
    if not force and all(p.exists() for p in outs):
        deps = srcs + driver_srcs + [PROBE_SRC] + list(SRC_DIR.glob("*.h*")) + list(SRC_DIR.glob("*.cuh"))
        deps += [h for h in (PKG_DIR.parent.parent / "include").glob("tchem_gb*.h")]
        newest = max(p.stat().st_mtime for p in deps)
        if min(p.stat().st_mtime for p in outs) > newest and not extra:
            return LIB_PATH
    workers = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs + [PROBE_SRC]))
    probe_obj = objs.pop()
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(PROBE_LIB_PATH), str(probe_obj), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(LIB_PATH), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    # the driver interface: host code linked against the engine, found beside it at run time
    dobjs = [_compile(nvcc, s, extra) for s in driver_srcs]
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(DRIVER_LIB_PATH), *map(str, dobjs), "-L", str(PKG_DIR),
           "-ltchem_gb", "-lcudart", "-Xlinker", "-rpath=$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
