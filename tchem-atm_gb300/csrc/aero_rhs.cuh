// Right-hand side of the gas-aerosol problem (SIMPOL.1 phase transfer), shared by the kernel
// (csrc/kernels_aero.cu, a warp of 32 lanes per sample) and a host build of the same source
// (one lane) that the tests run against the oracle on the CPU.
//
// Per sample, the temperature and pressure terms of each SIMPOL entry (accommodation coefficient,
// mean free path, partitioning constant, kg m-3 -> ppm factor;
// src/core/impl/TChem_Impl_SIMPOL_constant.hpp:50-130) are evaluated once. Per RHS evaluation the
// lanes run over reactions (rates of progress), then over particles (radius, mean molecular weight
// and mass; TChem_Impl_SingleParticleUtils.hpp:50-170), then over (particle, entry) pairs (the
// transfers, TChem_Impl_SIMPOL_phase_transfer.hpp:60-150), and each row gathers its terms in the
// reference's order (particles outer, entries inner), so no atomics are needed.
#pragma once

#include <cmath>
#include <cstdint>

#include "kernels.hpp"

namespace tchem_gb {
namespace fp64 {

__host__ __device__ inline void aero_sync() {
#ifdef __CUDA_ARCH__
  __syncwarp();
#endif
}

constexpr double kAeroPi = 3.141592653589793;
constexpr double kAeroRuniv = 8.314472;  // J/(mol K), src/core/TChem_Util.hpp
constexpr double kAeroAtmPa = 101325.0;  // Pa

// Everything one right-hand-side evaluation reads and writes (built once per sample, passed by
// reference to the one out-of-line evaluation routine, which keeps the kernels small to compile).
struct AeroEval {
  const double* x;       // [M] ODE vector (shared memory)
  const double* keff;    // [R]
  double* q;             // [R] rates of progress
  double* f;             // [M] result
  double* simc;          // [nS][4]: accommodation coefficient, mean free path, partitioning constant, kg m-3 -> ppm
  double* part;          // [nP][3]: radius, mean molecular weight, mass
  double* dsim;          // [nP][nS]: cond - evap of each (particle, entry) pair
  double* nc;            // [nP]: number concentrations of the sample
  const int32_t* rf_ptr;
  const int16_t* rf_sp;
  const int32_t* pr_ptr;
  const int16_t* pr_r;
  const double* pr_nu;
  const double* emis;
  AeroDev A;
  int32_t R;
};

// Temperature and pressure terms of every SIMPOL entry, NL lanes over entries (lane in [0, NL)).
template <int NL>
__host__ __device__ inline void aero_setup(const AeroEval& E, int lane, double t, double p) {
  const AeroDev& A = E.A;
  for (int is = lane; is < A.nS; is += NL) {
    const int32_t* I = A.sim_idx + 3 * is;
    const double* P = A.sim_par + 7 * is;
    const double B1 = P[0], B2 = P[1], B3 = P[2], B4 = P[3], D = P[4], N_star = P[5], MW = P[6];
    double alpha = 0.1;
    if (I[2]) {
      const double n23 = pow(N_star, 2.0 / 3.0);
      double dh = -10.0 * (N_star - 1.0) + 7.53 * (n23 - 1.0) - 1.0;
      double ds = -32.0 * (N_star - 1.0) + 9.21 * (n23 - 1.0) - 1.3;
      dh = dh * 4184.0;
      ds = ds * 4.184;
      const double dg = dh - t * ds;
      alpha = exp(-dg / (kAeroRuniv * t));
      alpha = alpha / (1.0 + alpha);
    }
    double vp = B1 / t + B2 + B3 * t + B4 * log(t);
    vp = kAeroAtmPa * pow(10.0, vp);
    double* sc = E.simc + 4 * is;
    sc[0] = alpha;
    sc[1] = 3.0 * D / sqrt(8.0 * kAeroRuniv * t / (kAeroPi * MW));
    sc[2] = vp / p / MW * 1.0e6;
    sc[3] = kAeroRuniv / MW * 1.0e6 * t / p;
  }
}

// E.f = RHS at the ODE vector in E.x, NL lanes (a whole warp on the device, NL = 32; one host
// thread, NL = 1); ends with a warp barrier on the device.
template <int NL>
__host__ __device__ __noinline__ void aero_eval(const AeroEval& E, int lane) {
  const AeroDev& A = E.A;
  const double* x = E.x;
  const int mg = A.m_gas, nA = A.nA, nS = A.nS, nP = A.nP, M = A.M;
  for (int r = lane; r < E.R; r += NL) {
    double q = E.keff[r];
    for (int g = E.rf_ptr[r]; g < E.rf_ptr[r + 1]; ++g) q *= x[E.rf_sp[g]];
    E.q[r] = q;
  }
  for (int ip = lane; ip < nP; ip += NL) {
    const double* xp = x + mg + ip * nA;
    double volume = A.vol0, mass = A.mass0, moles = A.moles0;
    for (int k = 0; k < nA; ++k) volume += xp[k] / A.density[k];
    for (int k = 0; k < nA; ++k) {
      mass += xp[k];
      moles += xp[k] / A.mw[k];
    }
    E.part[3 * ip] = pow(volume * 3.0 / 4.0 / kAeroPi, 1.0 / 3.0);
    E.part[3 * ip + 1] = mass / moles;
    E.part[3 * ip + 2] = mass;
  }
  aero_sync();
  for (int e = lane; e < nP * nS; e += NL) {
    const int ip = e / nS, is = e - ip * nS;
    const int aero = A.sim_idx[3 * is] + ip * nA, gas = A.sim_idx[3 * is + 1];
    const double* sc = E.simc + 4 * is;
    const double alpha = sc[0], mfp = sc[1], keq = sc[2];
    const double D = A.sim_par[7 * is + 4];
    const double radius = E.part[3 * ip], avg_mw = E.part[3 * ip + 1], mass = E.part[3 * ip + 2];
    const double kn = mfp / radius;
    const double ffs = (0.75 * alpha * (1.0 + kn)) / (kn * kn + (1.0 + 0.283 * alpha) * kn + 0.75 * alpha);
    double cond = 4.0 * kAeroPi * radius * D * ffs;
    double evap = cond * 1.0 * (keq * avg_mw / mass);
    // the host admits gas in [0, m_gas) and aero in [m_gas, M) only; the guards keep reads in bounds
    cond *= (gas >= 0 && gas < mg) ? x[gas] : 0.0;
    evap *= (aero >= mg && aero < M) ? x[aero] : 0.0;
    E.dsim[e] = -evap + cond;
  }
  aero_sync();
  for (int i = lane; i < M; i += NL) {
    double acc = 0.0;
    if (i < mg) {
      acc = E.emis[i];
      for (int e = E.pr_ptr[i]; e < E.pr_ptr[i + 1]; ++e) acc += E.pr_nu[e] * E.q[E.pr_r[e]];
      bool any = false;
      for (int is = 0; is < nS; ++is) any |= A.sim_idx[3 * is + 1] == i;
      if (any)
        for (int ip = 0; ip < nP; ++ip)
          for (int is = 0; is < nS; ++is)
            if (A.sim_idx[3 * is + 1] == i) acc += -E.nc[ip] * E.dsim[ip * nS + is];
    } else {
      const int ip = (i - mg) / nA;
      for (int is = 0; is < nS; ++is)
        if (A.sim_idx[3 * is] + ip * nA == i) acc += E.dsim[ip * nS + is] / E.simc[4 * is + 3];
    }
    E.f[i] = acc;
  }
  aero_sync();
}

}  // namespace fp64
}  // namespace tchem_gb
