"""The gas-aerosol kernel's right-hand-side source (csrc/aero_rhs.cuh: the rate-of-progress,
particle, transfer and row-gather loops and their indexing) built for the host with one lane,
on the engine's own packed mechanism tables (build_host_tables), against the oracle's aerosol RHS
on the CPU: the Simpol model with 1 and 3 particles and CB05CL_AE5 with four SIMPOL SOA
transfers, at perturbed states with every transfer active. The device build of the same source
runs in tests/test_zzz_gpu_aerosol.py."""
from __future__ import annotations

import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from helpers import GOLDEN
from oracle import AerosolOracle, Oracle
from tchem_gb import _capi
from test_zzz_gpu_aerosol import models, perturbed

PROGRAM = r'''
#include <cstdio>
#include <iostream>
#include <vector>

#include "aero_rhs.cuh"
#include "aerosol_model.hpp"
#include "device_tables.hpp"
#include "kinetic_model.hpp"

using namespace tchem_gb;

int main(int argc, char** argv) {
  const KineticModel km = KineticModel::fromYamlFile(argv[1], nullptr);
  AerosolModel am = AerosolModel::fromYamlFile(argv[2], km);
  am.nParticles = std::atoi(argv[3]);
  const HostTables ht = build_host_tables(km);
  const MechLayout& L = ht.L;
  const unsigned char* b = ht.blob.data();
  const int mg = km.nSpec - km.nConstSpec, nA = am.nSpec, nP = am.nParticles, nS = (int)am.simpol.size();
  const int M = mg + nP * nA, R = L.R, nc_ = km.nConstSpec;
  std::vector<int32_t> sidx;
  std::vector<double> spar;
  for (const auto& s : am.simpol) {
    sidx.insert(sidx.end(), {s.aerosol_sp_index, s.gas_sp_index, s.compute_alpha ? 1 : 0});
    spar.insert(spar.end(), {s.B1, s.B2, s.B3, s.B4, s.diffusion_coeff, s.N_star, s.molecular_weight});
  }
  double T, p;
  std::cin >> T >> p;
  std::vector<double> kfor(R), x(M), xc(nc_), nc(nP), keff(R), q(R), f(M), simc(4 * nS + 1), part(3 * nP),
      dsim(nP * nS + 1);
  for (auto& v : kfor) std::cin >> v;
  for (auto& v : x) std::cin >> v;
  for (auto& v : xc) std::cin >> v;
  for (auto& v : nc) std::cin >> v;
  for (int r = 0; r < R; ++r) {  // the constant-species factors, as the kernel's compute_keff folds them
    double k = kfor[r];
    for (int c = ht.cf_ptr[r]; c < ht.cf_ptr[r + 1]; ++c) k *= xc[ht.cf_idx[c]];
    keff[r] = k;
  }
  fp64::AeroEval E;
  E.x = x.data(); E.keff = keff.data(); E.q = q.data(); E.f = f.data(); E.simc = simc.data();
  E.part = part.data(); E.dsim = dsim.data(); E.nc = nc.data();
  E.rf_ptr = reinterpret_cast<const int32_t*>(b + L.off_rf_ptr);
  E.rf_sp = reinterpret_cast<const int16_t*>(b + L.off_rf_sp);
  E.pr_ptr = reinterpret_cast<const int32_t*>(b + L.off_pr_ptr);
  E.pr_r = reinterpret_cast<const int16_t*>(b + L.off_pr_r);
  E.pr_nu = reinterpret_cast<const double*>(b + L.off_pr_nu);
  E.emis = reinterpret_cast<const double*>(b + L.off_emis);
  E.A = AeroDev{nA, nP, nS, mg, M, sidx.data(), spar.data(), am.aerosol_density.data(), am.molecular_weights.data(),
                (double)(1.0e-25L / 1800.0L), (double)1.0e-25L, (double)(1.0e-25L / 0.1L)};
  E.R = R;
  fp64::aero_setup<1>(E, 0, T, p);
  fp64::aero_eval<1>(E, 0);
  for (double v : f) std::printf("%.17g\n", v);
  return 0;
}
'''


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.os.path.exists(nvcc):
        pytest.skip("no nvcc")
    d = tmp_path_factory.mktemp("aero_rhs")
    src = d / "aero_rhs_host.cu"
    src.write_text(PROGRAM)
    exe = d / "aero_rhs_host"
    csrc = ROOT / "tchem-atm_gb300" / "csrc"
    pkg = _capi.LIB_PATH.parent
    r = subprocess.run([shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc", "-std=c++17", "-O2",
                        "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(csrc), str(src), "-o", str(exe),
                        "-L", str(pkg), "-ltchem_gb", "-Xlinker", f"-rpath={pkg}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("case,particles", [("simpol", 1), ("simpol", 3), ("cb05", 1)])
def test_kernel_rhs_source_matches_oracle(program, case, particles):
    km, am, gf, pf = models(case)
    am.set_number_of_particles(particles)
    state, nc = perturbed(km, am, gf, pf, 4, 7)
    mg, n = km.n_active, km.nSpec
    files = {"simpol": ("simpol_config_gas.yaml", "simpol_phase_transfer.yaml"),
             "cb05": ("cb05_soa_config_full_gas.yaml", "cb05_soa_mechanism_aero.yaml")}[case]
    o = Oracle([km])
    for b in range(state.shape[0]):
        row = state[b]
        T, p = row[2], row[1]
        x = np.concatenate([row[3:3 + mg], row[3 + n:]])
        xconst = row[3 + mg:3 + n]
        kfor = o.kforward(T, p) if km.nReac else np.zeros(0)
        stdin = " ".join(f"{v:.17g}" for v in [T, p, *kfor, *x, *xconst, *nc[b]])
        r = subprocess.run([str(program), str(GOLDEN / "aerosol" / files[0]), str(GOLDEN / "aerosol" / files[1]),
                            str(particles)], input=stdin, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        f = np.array([float(v) for v in r.stdout.split()])
        ref = AerosolOracle(km, am).rhs(T, p, nc[b], x, xconst)
        assert f.shape == ref.shape
        assert np.abs(f[:mg] - ref[:mg]).max() <= 1e-13 * max(np.abs(ref[:mg]).max(), 1e-300)
        aero = ref[mg:]
        scale = np.maximum(np.abs(aero), max(1e-12 * np.abs(aero).max(), 1e-300))
        assert (np.abs(f[mg:] - aero) / scale).max() <= 1e-12
