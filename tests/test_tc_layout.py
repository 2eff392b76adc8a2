"""Host-side checks of the tensor-core kernels' encodings (csrc/tc_tile.cuh), compiled by nvcc
into a small host program: the K-major no-swizzle operand layout is a bijection of the tile onto
its bytes, made of 8-row x 16-byte core matrices (LBO 128 B along K, SBO 32 * K bytes along M/N);
the instruction descriptor of kind::tf32 and the shared-memory descriptor carry each field at the
bit position of the PTX ISA's tables. (What the tensor cores do with them is checked on a GPU.)"""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT


def _run(tmp_path) -> list[str]:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.os.path.exists(nvcc):
        pytest.skip("no nvcc")
    src = tmp_path / "tc_layout.cu"
    src.write_text(f'''#include <cstdio>
#include "{ROOT / "tchem-atm_gb300" / "csrc" / "tc_tile.cuh"}"
using namespace tchem_gb::tc;
int main() {{
  for (int r = 0; r < 256; ++r)
    for (int k = 0; k < 32; ++k) std::printf("o %d %d %u\\n", r, k, kmajor_offset(r, k, 32));
  std::printf("i %u\\n", idesc_tf32(128, 64, true));
  std::printf("i2 %u\\n", idesc_tf32(128, 256, false));
  std::printf("d %llu\\n", (unsigned long long)smem_desc(0x1230u, 128u, 1024u));
  return 0;
}}
''')
    exe = tmp_path / "tc_layout"
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()


def test_tc_encodings(tmp_path):
    out = _run(tmp_path)
    offs = {}
    for line in out:
        if line.startswith("o "):
            _, r, k, o = line.split()
            offs[(int(r), int(k))] = int(o)
    vals = list(offs.values())
    assert len(set(vals)) == len(vals) == 256 * 32  # one byte slot per element
    assert min(vals) == 0 and max(vals) == 256 * 32 * 4 - 4 and all(v % 4 == 0 for v in vals)
    for (r, k), o in offs.items():
        base = offs[(r - r % 8, k - k % 4)]
        assert o - base == (r % 8) * 16 + (k % 4) * 4  # inside a core matrix: 16-byte rows
        assert base == (r // 8) * 1024 + (k // 4) * 128  # SBO 1024 (32 x 4 B per row), LBO 128
    assert offs[(0, 8)] == 256  # K = 8 (one kind::tf32 MMA) later starts 256 B further
    kv = dict(line.split() for line in out if not line.startswith("o "))
    i = int(kv["i"])
    assert (i >> 4) & 3 == 1 and (i >> 7) & 7 == 2 and (i >> 10) & 7 == 2  # D f32, A and B tf32
    assert (i >> 13) & 1 == 1 and (i >> 14) & 1 == 0 and (i >> 15) & 3 == 0  # -A, K-major A and B
    assert (i >> 17) & 63 == 64 >> 3 and (i >> 24) & 31 == 128 >> 4 and (i >> 23) & 1 == 0
    i2 = int(kv["i2"])
    assert (i2 >> 17) & 63 == 256 >> 3 and (i2 >> 13) & 1 == 0
    d = int(kv["d"])
    assert d & 0x3FFF == 0x1230 >> 4 and (d >> 16) & 0x3FFF == 128 >> 4 and (d >> 32) & 0x3FFF == 1024 >> 4
    assert (d >> 46) & 7 == 1 and (d >> 49) & 7 == 0 and (d >> 61) & 7 == 0  # version 1, no swizzle
