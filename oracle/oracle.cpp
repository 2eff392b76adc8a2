// CPU oracle: FP64 restatement of the reference's box-model RHS and a TR-BDF2 integrator.
// TEST INFRASTRUCTURE ONLY (see oracle.h for scope and citations).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// --- rate constants: src/core/impl/TChem_Impl_KForwardAerosol.hpp:44-145 -----------------
void kforward(const tchem_gb_kmcd_view& km, double t, double p, double* kfor) {
  const double t_1 = 1.0 / t;
  const double one = 1.0;
  const double conv = km.CONV_PPM * p * t_1;
  for (int r = 0; r < km.nReac; ++r) kfor[r] = 0.0;  // types outside the box path stay 0
  for (int i = 0; i < km.nArrhenius; ++i) {
    const double* P = km.arrhenius_param + 5 * i;
    const double E = P[0], A = P[1], B = P[2], C = P[3], D = P[4];
    const int r = km.arrhenius_reaction[i];
    kfor[r] = A * std::exp(C * t_1) * (B == 0.0 ? one : std::pow(t / D, B)) * (E == 0.0 ? one : (one + E * p)) *
              std::pow(conv, static_cast<double>(km.convExponent[r]));
  }
  for (int i = 0; i < km.nTroe; ++i) {
    const double* rp = km.reacPpar + 8 * i;
    const int r = km.reacPfal[i];
    const double k0_A = rp[0], k0_B = rp[1], k0_C = rp[2];
    const double kinf_A = rp[3], kinf_B = rp[4], kinf_C = rp[5], Fc = rp[6], N = rp[7];
    const double k0 = k0_A * (k0_C == 0.0 ? one : std::exp(k0_C * t_1)) *
                      (k0_B == 0.0 ? one : std::pow(t / 300.0, k0_B)) * conv;
    const double k0_kinf = k0 / (kinf_A * (kinf_C == 0.0 ? one : std::exp(kinf_C * t_1)) *
                                 (kinf_B == 0.0 ? one : std::pow(t / 300.0, kinf_B)));
    kfor[r] = k0 / (1.0 + k0_kinf) * std::pow(Fc, 1.0 / (1.0 + std::pow(std::log10(k0_kinf) / N, 2.0))) *
              std::pow(conv, static_cast<double>(km.convExponent[r]));
  }
  for (int i = 0; i < km.nCMAQ_H2O2; ++i) {
    const double* P = km.cmaq_param + 6 * i;
    const double A1 = P[0], B1 = P[1], C1 = P[2], A2 = P[3], B2 = P[4], C2 = P[5];
    const int r = km.cmaq_reaction[i];
    kfor[r] = (A1 * std::exp(C1 * t_1) * (B1 == 0.0 ? one : std::pow(t / 300.0, B1)) +
               A2 * std::exp(C2 * t_1) * (B2 == 0.0 ? one : std::pow(t / 300.0, B2)) * conv) *
              std::pow(conv, static_cast<double>(km.convExponent[r]));
  }
}

// --- E3SM rate constants ---------------------------------------------------------------------
// Order of src/core/impl/TChem_Impl_RateofProgress.hpp:70-80 and
// src/core/impl/TChem_Impl_ReactionRates.hpp:54-79: photolysis rates into kfor[0, n_photo), then
// KForward (src/core/impl/TChem_Impl_KForward.hpp:44-147: ARRHENIUS and TROE without the ppm
// conversion, CMAQ_H2O2 with it), KForwardJPL (src/core/impl/TChem_Impl_KForwardJPL.hpp:45-147,
// [M] = x(M_index)) and AdjustReactions (src/core/impl/TChem_Impl_AdjustReactions.hpp:45-100:
// the adjust pairs serially in file order, then the prod_O1D modifier). x[nSpec]. Reactions
// that neither list nor the photolysis input reaches stay 0.
void e3sm_kforward(const tchem_gb_kmcd_view& km, const tchem_gb_e3sm_view& e3, double t, double p, const double* x,
                   const double* photo, int n_photo, double* kfor) {
  const double t_1 = 1.0 / t;
  const double one = 1.0;
  const double conv = km.CONV_PPM * p * t_1;
  for (int r = 0; r < km.nReac; ++r) kfor[r] = (photo && r < n_photo) ? photo[r] : 0.0;
  for (int i = 0; i < km.nArrhenius; ++i) {
    const double* P = km.arrhenius_param + 5 * i;
    const double E = P[0], A = P[1], B = P[2], C = P[3], D = P[4];
    kfor[km.arrhenius_reaction[i]] =
        A * std::exp(C * t_1) * (B == 0.0 ? one : std::pow(t / D, B)) * (E == 0.0 ? one : (one + E * p));
  }
  for (int i = 0; i < km.nTroe; ++i) {
    const double* rp = km.reacPpar + 8 * i;
    const double k0_A = rp[0], k0_B = rp[1], k0_C = rp[2];
    const double kinf_A = rp[3], kinf_B = rp[4], kinf_C = rp[5], Fc = rp[6], N = rp[7];
    const double k0 = k0_A * (k0_C == 0.0 ? one : std::exp(k0_C * t_1)) * (k0_B == 0.0 ? one : std::pow(t / 300.0, k0_B));
    const double k0_kinf = k0 / (kinf_A * (kinf_C == 0.0 ? one : std::exp(kinf_C * t_1)) *
                                 (kinf_B == 0.0 ? one : std::pow(t / 300.0, kinf_B)));
    kfor[km.reacPfal[i]] = k0 / (1.0 + k0_kinf) * std::pow(Fc, 1.0 / (1.0 + std::pow(std::log10(k0_kinf) / N, 2.0)));
  }
  for (int i = 0; i < km.nCMAQ_H2O2; ++i) {
    const double* P = km.cmaq_param + 6 * i;
    const double A1 = P[0], B1 = P[1], C1 = P[2], A2 = P[3], B2 = P[4], C2 = P[5];
    const int r = km.cmaq_reaction[i];
    kfor[r] = (A1 * std::exp(C1 * t_1) * (B1 == 0.0 ? one : std::pow(t / 300.0, B1)) +
               A2 * std::exp(C2 * t_1) * (B2 == 0.0 ? one : std::pow(t / 300.0, B2)) * conv) *
              std::pow(conv, static_cast<double>(km.convExponent[r]));
  }
  const double mM = x[km.M_index];
  // k0 and kinf of the JPL forms: A exp(C/T) (T/300)^B with the exp and pow skipped at C, B = 0
  auto arr = [&](double A, double B, double C) {
    return A * (C == 0.0 ? one : std::exp(C * t_1)) * (B == 0.0 ? one : std::pow(t / 300.0, B));
  };
  auto falloff = [&](const double* P) {  // k0_A, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc
    const double k0 = arr(P[0], P[1], P[2]);
    const double kinf = arr(P[3], P[4], P[5]);
    const double xpo = k0 * mM / kinf;
    const double lg = std::log10(xpo);
    const double factor = P[6] == one ? one : std::pow(P[6], one / (one + lg * lg));
    return k0 / (one + xpo) * factor;
  };
  for (int i = 0; i < e3.nJPL; ++i) kfor[e3.jpl_reaction[i]] = falloff(e3.jpl_param + 7 * i);
  for (int i = 0; i < e3.nRJPL; ++i) {
    const double* P = e3.rjpl_param + 10 * i;
    kfor[e3.rjpl_reaction[i]] = falloff(P) / arr(P[7], P[8], P[9]);
  }
  for (int i = 0; i < e3.nAdjust; ++i) kfor[e3.adjust_pair[2 * i]] *= x[e3.adjust_pair[2 * i + 1]];
  for (int i = 0; i < e3.nProdO1D; ++i) {
    const int32_t* I = e3.o1d_index + 7 * i;
    const double* P = e3.o1d_param + 6 * i;
    const double k1 = P[0] * std::exp(P[1] * t_1), k2 = P[2] * std::exp(P[3] * t_1), k3 = P[4] * std::exp(P[5] * t_1);
    const double fc = k1 * x[I[4]] + k2 * x[I[5]] + k3 * x[I[6]];
    for (int j = 0; j < 3; ++j) kfor[I[j]] *= kfor[I[3]] / fc;
  }
}

// True when an active species scales a rate constant ([M] of the JPL forms, an adjust or a
// prod_O1D species): the rate constants then change with the state.
bool e3sm_kfor_depends_on_state(const tchem_gb_kmcd_view& km, const tchem_gb_e3sm_view& e3) {
  const int m = km.nSpec - km.nConstSpec;
  if ((e3.nJPL > 0 || e3.nRJPL > 0) && km.M_index < m) return true;
  for (int i = 0; i < e3.nAdjust; ++i)
    if (e3.adjust_pair[2 * i + 1] < m) return true;
  for (int i = 0; i < e3.nProdO1D; ++i)
    for (int j = 4; j < 7; ++j)
      if (e3.o1d_index[7 * i + j] < m) return true;
  return false;
}

// --- SIMPOL.1 gas-particle phase transfer ----------------------------------------------------
// src/core/impl/TChem_Impl_SIMPOL_constant.hpp:50-130 (accommodation coefficient, mean free path,
// vapour pressure, kg/m3 -> ppm factor, partitioning constant),
// src/core/impl/TChem_Impl_SingleParticleUtils.hpp:50-170 (particle volume, radius, mass and mean
// molecular weight with the reference's floor values; Fuchs-Sutugin transition-regime rate),
// src/core/impl/TChem_Impl_SIMPOL_phase_transfer.hpp:60-150 (condensation minus evaporation per
// particle). Constants of src/core/TChem_Util.hpp: RUNIV 8.314472 J/mol/K, PI, ATMPA 101325 Pa.
constexpr double kRuniv = 8.314472;
constexpr double kPi = 3.141592653589793;
constexpr double kAtmPa = 101325.0;
constexpr long double kMinMass = 1.0e-25L;     // kg/m3
constexpr long double kMinMw = 0.1L;           // kg/mol
constexpr long double kMinDensity = 1800.0L;   // kg/m3

// Adds SIMPOL entry i_simpol's transfer for particle i_part to omega (ODE vector x).
void simpol_particle(const tchem_gb_aero_view& av, int i_simpol, int i_part, double t, double p,
                     const double* number_conc, const double* x, double* omega) {
  const int32_t* I = av.simpol_index + 3 * i_simpol;
  const double* P = av.simpol_param + 7 * i_simpol;
  const int aero = I[0], gas = I[1];
  const double B1 = P[0], B2 = P[1], B3 = P[2], B4 = P[3], D = P[4], N_star = P[5], MW = P[6];
  double alpha = 0.1;
  if (I[2]) {
    const double n23 = std::pow(N_star, 2.0 / 3.0);
    double dh = -10.0 * (N_star - 1.0) + 7.53 * (n23 - 1.0) - 1.0;
    double ds = -32.0 * (N_star - 1.0) + 9.21 * (n23 - 1.0) - 1.3;
    dh = dh * 4184.0;
    ds = ds * 4.184;
    const double dg = dh - t * ds;
    alpha = std::exp(-dg / (kRuniv * t));
    alpha = alpha / (1.0 + alpha);
  }
  const double mfp = 3.0 * D / std::sqrt(8.0 * kRuniv * t / (kPi * MW));
  double vp = B1 / t + B2 + B3 * t + B4 * std::log(t);
  vp = kAtmPa * std::pow(10.0, vp);
  const double kgm3_to_ppm = kRuniv / MW * 1.0e6 * t / p;
  const double keq = vp / p / MW * 1.0e6;
  const int first = av.nSpec_gas + i_part * av.nSpec;
  double volume = static_cast<double>(kMinMass / kMinDensity);
  double mass = static_cast<double>(kMinMass);
  double moles = static_cast<double>(kMinMass / kMinMw);
  for (int k = 0; k < av.nSpec; ++k) volume += x[first + k] / av.aerosol_density[k];
  for (int k = 0; k < av.nSpec; ++k) {
    mass += x[first + k];
    moles += x[first + k] / av.molecular_weights[k];
  }
  const double radius = std::pow(volume * 3.0 / 4.0 / kPi, 1.0 / 3.0);
  const double avg_mw = mass / moles;
  const double kn = mfp / radius;
  const double ffs = (0.75 * alpha * (1.0 + kn)) / (kn * kn + (1.0 + 0.283 * alpha) * kn + 0.75 * alpha);
  double cond = 4.0 * kPi * radius * D * ffs;
  double evap = cond * 1.0 * (keq * avg_mw / mass);
  cond *= x[gas];
  evap *= x[aero + i_part * av.nSpec];
  const double diff = -evap + cond;
  omega[gas] += -number_conc[i_part] * diff;
  omega[aero + i_part * av.nSpec] += diff / kgm3_to_ppm;
}

// --- RHS: src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:57-143 --------------------------
// concX[nSpec] (constant species last), kfor precomputed; omega[m]. src[m] (E3SM external
// sources, src/core/impl/TChem_Impl_NetProductionRates.hpp:73-77) replaces the emissions.
void reaction_rates(const tchem_gb_kmcd_view& km, const double* kfor, const double* concX, double* omega,
                    double* rop, const double* src = nullptr) {
  const int m = km.nSpec - km.nConstSpec;
  const int S = km.maxSpecInReac;
  for (int i = 0; i < m; ++i) omega[i] = src ? src[i] : 0.0;
  for (int i = 0; i < km.nEmission && !src; ++i) {
    const int k = km.emission_species[i];
    if (k < m) omega[k] = km.emission_rate[i];
  }
  for (int r = 0; r < km.nReac; ++r) {
    double q = kfor[r];
    for (int j = 0; j < km.reacNreac[r]; ++j) {
      const int ks = km.reacSidx[r * S + j];
      const int niup = std::abs(static_cast<int>(km.reacNuki[r * S + j]));
      q *= std::pow(concX[ks], static_cast<double>(niup));
    }
    rop[r] = q;
  }
  const int joff = S / 2;
  for (int r = 0; r < km.nReac; ++r) {
    const double q = rop[r];
    for (int j = 0; j < km.reacNreac[r]; ++j) {
      const int ks = km.reacSidx[r * S + j];
      if (ks < m) omega[ks] += km.reacNuki[r * S + j] * q;
    }
    for (int j = 0; j < km.reacNprod[r]; ++j) {
      const int ks = km.reacSidx[r * S + j + joff];
      if (ks < m) omega[ks] += km.reacNuki[r * S + j + joff] * q;
    }
  }
}

// --- analytic Jacobian of reaction_rates with respect to the active species ---------------
void jacobian(const tchem_gb_kmcd_view& km, const double* kfor, const double* concX, double* J) {
  const int m = km.nSpec - km.nConstSpec;
  const int S = km.maxSpecInReac;
  const int joff = S / 2;
  std::fill(J, J + static_cast<size_t>(m) * m, 0.0);
  for (int r = 0; r < km.nReac; ++r) {
    const int nr = km.reacNreac[r];
    for (int j = 0; j < nr; ++j) {
      const int sj = km.reacSidx[r * S + j];
      if (sj >= m) continue;
      const int nj = std::abs(static_cast<int>(km.reacNuki[r * S + j]));
      double dq = kfor[r] * nj * std::pow(concX[sj], static_cast<double>(nj - 1));
      for (int l = 0; l < nr; ++l) {
        if (l == j) continue;
        const int sl = km.reacSidx[r * S + l];
        const int nl = std::abs(static_cast<int>(km.reacNuki[r * S + l]));
        dq *= std::pow(concX[sl], static_cast<double>(nl));
      }
      for (int k = 0; k < nr; ++k) {
        const int sk = km.reacSidx[r * S + k];
        if (sk < m) J[static_cast<size_t>(sk) * m + sj] += km.reacNuki[r * S + k] * dq;
      }
      for (int k = 0; k < km.reacNprod[r]; ++k) {
        const int sk = km.reacSidx[r * S + k + joff];
        if (sk < m) J[static_cast<size_t>(sk) * m + sj] += km.reacNuki[r * S + k + joff] * dq;
      }
    }
  }
}

// Mantissa bits kept in the operands of the blocked trailing update of FP32 factorizations
// (oracle_set_lu_tile_bits): 0 = unblocked FP32 LU; 10 = TF32 tiles, 7 = BF16 tiles.
int g_lu_tile_bits = 0;

// Static symmetric elimination order without pivoting for FP32 factorizations of matrices of its
// size (oracle_set_lu_static_order): row and column k of the factored matrix are species
// g_lu_order[k]. A sparse factorization in that order performs exactly these operations on the
// structural nonzeros (the skipped ones only ever add 0 to 0).
std::vector<int> g_lu_order;

// Test settings of the full-Newton integrator (oracle_set_newton_min_iterations,
// oracle_set_step_sequence): a minimum number of Newton iterations per stage before the
// convergence test may end it, and an imposed sequence of accepted step sizes (step k takes
// g_step_seq[k], the last entry repeating, each clipped to t_end as usual) in place of the error
// control.
int g_newton_min_iters = 1;
std::vector<double> g_step_seq;

// Round-to-nearest-even of an FP32 value to `keep` mantissa bits (TF32: 10, BF16: 7).
float round_mantissa(float x, int keep) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf, nan
  const int drop = 23 - keep;
  const uint32_t lsb = (u >> drop) & 1u;
  u += (1u << (drop - 1)) - 1u + lsb;
  u &= ~((1u << drop) - 1u);
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}

// --- dense LU with partial pivoting (row swaps; first maximum in the current row order) ---
template <typename T>
struct DenseLU {
  int n = 0;
  std::vector<T> a;
  std::vector<int> piv;
  std::vector<T> w;
  std::vector<T> dinv;   // ordered factors: reciprocals of the pivots
  bool ordered = false;  // the factors are of the static order (g_lu_order)
  void resize(int n_) {
    n = n_;
    dinv.assign(n_, T(0));
    a.assign(static_cast<size_t>(n) * n, T(0));
    piv.assign(n, 0);
    w.assign(n, T(0));
  }
  // Blocked right-looking LU as a tensor-core factorization computes it: 32-column panels factored
  // with partial pivoting in FP32, U12 = L11^-1 A12 in FP32, and the trailing update
  // A22 -= L21 U12 with both operands rounded to `keep` mantissa bits and FP32 accumulation of each
  // panel's 32 products.
  bool factor_blocked(int keep) {
    const int NB = 32;
    for (int p0 = 0; p0 < n; p0 += NB) {
      const int p1 = std::min(n, p0 + NB);
      for (int k = p0; k < p1; ++k) {
        int p = k;
        T amax = std::abs(a[static_cast<size_t>(k) * n + k]);
        for (int i = k + 1; i < n; ++i) {
          const T v = std::abs(a[static_cast<size_t>(i) * n + k]);
          if (v > amax) { amax = v; p = i; }
        }
        if (!(amax > T(0)) || !std::isfinite(static_cast<double>(amax))) return false;
        piv[k] = p;
        if (p != k)
          for (int j = 0; j < n; ++j) std::swap(a[static_cast<size_t>(k) * n + j], a[static_cast<size_t>(p) * n + j]);
        const T inv = T(1) / a[static_cast<size_t>(k) * n + k];
        for (int i = k + 1; i < n; ++i) {
          const T l = a[static_cast<size_t>(i) * n + k] * inv;
          a[static_cast<size_t>(i) * n + k] = l;
          for (int j = k + 1; j < p1; ++j) a[static_cast<size_t>(i) * n + j] -= l * a[static_cast<size_t>(k) * n + j];
        }
      }
      for (int k = p0; k < p1; ++k)
        for (int i = k + 1; i < p1; ++i) {
          const T l = a[static_cast<size_t>(i) * n + k];
          for (int j = p1; j < n; ++j) a[static_cast<size_t>(i) * n + j] -= l * a[static_cast<size_t>(k) * n + j];
        }
      for (int i = p1; i < n; ++i)
        for (int j = p1; j < n; ++j) {
          float acc = 0.f;
          for (int k = p0; k < p1; ++k)
            acc += round_mantissa(static_cast<float>(a[static_cast<size_t>(i) * n + k]), keep) *
                   round_mantissa(static_cast<float>(a[static_cast<size_t>(k) * n + j]), keep);
          a[static_cast<size_t>(i) * n + j] -= acc;
        }
    }
    return true;
  }
  // A = I - c J, built in double and rounded to T.
  bool factor(const double* J, double c) {
    ordered = sizeof(T) == 4 && static_cast<int>(g_lu_order.size()) == n;
    if (ordered) return factor_ordered(J, c);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        a[static_cast<size_t>(i) * n + j] = static_cast<T>((i == j ? 1.0 : 0.0) - c * J[static_cast<size_t>(i) * n + j]);
    if (sizeof(T) == 4 && g_lu_tile_bits > 0) return factor_blocked(g_lu_tile_bits);
    for (int k = 0; k < n; ++k) {
      int p = k;
      T amax = std::abs(a[static_cast<size_t>(k) * n + k]);
      for (int i = k + 1; i < n; ++i) {
        const T v = std::abs(a[static_cast<size_t>(i) * n + k]);
        if (v > amax) { amax = v; p = i; }
      }
      if (!(amax > T(0)) || !std::isfinite(static_cast<double>(amax))) return false;
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; ++j) std::swap(a[static_cast<size_t>(k) * n + j], a[static_cast<size_t>(p) * n + j]);
      const T inv = T(1) / a[static_cast<size_t>(k) * n + k];
      for (int i = k + 1; i < n; ++i) {
        const T l = a[static_cast<size_t>(i) * n + k] * inv;
        a[static_cast<size_t>(i) * n + k] = l;
        for (int j = k + 1; j < n; ++j) a[static_cast<size_t>(i) * n + j] -= l * a[static_cast<size_t>(k) * n + j];
      }
    }
    return true;
  }
  // x = A^{-T} b with the same factors: U^T z = b, L^T v = z, x = P^T v.
  void solve_t(const double* b, double* x) {
    for (int i = 0; i < n; ++i) w[i] = static_cast<T>(b[i]);
    for (int j = 0; j < n; ++j) {
      w[j] /= a[static_cast<size_t>(j) * n + j];
      for (int l = j + 1; l < n; ++l) w[l] -= a[static_cast<size_t>(j) * n + l] * w[j];
    }
    for (int k = n - 1; k > 0; --k)
      for (int i = 0; i < k; ++i) w[i] -= a[static_cast<size_t>(k) * n + i] * w[k];
    for (int k = n - 1; k >= 0; --k)
      if (piv[k] != k) std::swap(w[k], w[piv[k]]);
    for (int i = 0; i < n; ++i) x[i] = static_cast<double>(w[i]);
  }
  // P (I - c J) P^T = L U with P the static order, no row exchanges.
  bool factor_ordered(const double* J, double c) {
    const int* o = g_lu_order.data();
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        a[static_cast<size_t>(i) * n + j] =
            static_cast<T>((o[i] == o[j] ? 1.0 : 0.0) - c * J[static_cast<size_t>(o[i]) * n + o[j]]);
    for (int k = 0; k < n; ++k) {
      piv[k] = k;
      const T akk = a[static_cast<size_t>(k) * n + k];
      if (!(std::abs(akk) > T(0)) || !std::isfinite(static_cast<double>(akk))) return false;
      const T inv = T(1) / akk;
      dinv[k] = inv;
      for (int i = k + 1; i < n; ++i) {
        const T l = a[static_cast<size_t>(i) * n + k] * inv;
        a[static_cast<size_t>(i) * n + k] = l;
        for (int j = k + 1; j < n; ++j) a[static_cast<size_t>(i) * n + j] -= l * a[static_cast<size_t>(k) * n + j];
      }
    }
    return true;
  }
  // Column-oriented substitutions of the ordered factors on w: L z = w, then U x = z with
  // x_k = z_k * (1 / u_kk) and the column of x_k eliminated from the rows above.
  void substitute() {
    for (int k = 0; k < n; ++k) {
      const T wk = w[k];
      for (int i = k + 1; i < n; ++i) w[i] -= a[static_cast<size_t>(i) * n + k] * wk;
    }
    for (int k = n - 1; k >= 0; --k) {
      const T xk = w[k] * dinv[k];
      w[k] = xk;
      for (int i = 0; i < k; ++i) w[i] -= a[static_cast<size_t>(i) * n + k] * xk;
    }
  }
  // x = A^{-1} b (b and x in double, arithmetic in T).
  void solve(const double* b, double* x) {
    if (ordered) {
      const int* o = g_lu_order.data();
      for (int k = 0; k < n; ++k) w[k] = static_cast<T>(b[o[k]]);
      substitute();
      for (int k = 0; k < n; ++k) x[o[k]] = static_cast<double>(w[k]);
      return;
    }
    for (int i = 0; i < n; ++i) w[i] = static_cast<T>(b[i]);
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(w[k], w[piv[k]]);
    for (int k = 0; k < n; ++k) {
      const T wk = w[k];
      for (int i = k + 1; i < n; ++i) w[i] -= a[static_cast<size_t>(i) * n + k] * wk;
    }
    for (int k = n - 1; k >= 0; --k) {
      T s = w[k];
      for (int j = k + 1; j < n; ++j) s -= a[static_cast<size_t>(k) * n + j] * w[j];
      w[k] = s / a[static_cast<size_t>(k) * n + k];
    }
    for (int i = 0; i < n; ++i) x[i] = static_cast<double>(w[i]);
  }
};

struct Settings {
  int max_newton, jac_interval, max_iters, refine;
  bool simplified;  // simplified-Newton form (tchem_gb.h, TCHEM_GB_FORM_MIXED_SIMPLIFIED)
  double atol_newton, rtol_newton;
  const double* tol_time;  // [m][2]
};

// One sample: RHS/Jacobian closure over the fixed T, p and constant concentrations.
template <typename LU_T>
struct Sample {
  const tchem_gb_kmcd_view& km;
  int m, n;
  std::vector<double> kfor, rop, concX, J;
  DenseLU<LU_T> lu;
  tchem_gb_sample_stats st{};
  std::vector<double> res, corr;  // refinement residual and correction
  // simplified-Newton form: factors valid / formed in the current stage, and their coefficient
  bool have_lu = false, fresh = false;
  double c_lu = 0.0;

  // trajectory record (adjoint): accepted step sizes, or null
  double* tape_dt = nullptr;
  int tape_cap = 0;

  // E3SM inputs: rate constants given per sample (kfor_in) and external sources (src) in place of
  // the emissions.
  const double* src = nullptr;
  // Aerosol problem (src/core/problems/TChem_Impl_AerosolChemistry_Problem.hpp:70-160): the ODE
  // vector is [active gas, particles]; the RHS is the gas RHS plus the SIMPOL transfers of every
  // particle (src/core/impl/TChem_Impl_Aerosol_RHS.hpp:60-105); the Jacobian is a forward
  // difference of it, as the reference's (computeJacobian -> computeNumericalJacobian).
  const tchem_gb_aero_view* aero = nullptr;
  const double* number_conc = nullptr;
  double T_aero = 0.0, p_aero = 0.0;
  int m_gas = 0;
  std::vector<double> f0, fh, yh;

  Sample(const tchem_gb_kmcd_view& km_, double T, double p, const double* xconst, const double* k_scale = nullptr,
         const double* kfor_in = nullptr, const double* src_ = nullptr)
      : km(km_), m(km_.nSpec - km_.nConstSpec), n(km_.nSpec), src(src_) {
    kfor.assign(km.nReac, 0.0);
    rop.assign(km.nReac, 0.0);
    concX.assign(n, 0.0);
    J.assign(static_cast<size_t>(m) * m, 0.0);
    for (int i = 0; i < n - m; ++i) concX[m + i] = xconst[i];
    if (kfor_in)
      std::copy(kfor_in, kfor_in + km.nReac, kfor.begin());
    else
      kforward(km, T, p, kfor.data());
    if (k_scale)
      for (int r = 0; r < km.nReac; ++r) kfor[r] *= k_scale[r];
    lu.resize(m);
    res.assign(m, 0.0);
    corr.assign(m, 0.0);
  }
  // Switches this sample to the aerosol problem of av with number concentrations nc[nParticles].
  void set_aerosol(const tchem_gb_aero_view* av, const double* nc, double T, double p) {
    aero = av;
    number_conc = nc;
    T_aero = T;
    p_aero = p;
    m_gas = m;
    m = av->nSpec_gas + av->nSpec * av->nParticles;
    J.assign(static_cast<size_t>(m) * m, 0.0);
    lu.resize(m);
    res.assign(m, 0.0);
    corr.assign(m, 0.0);
    f0.assign(m, 0.0);
    fh.assign(m, 0.0);
    yh.assign(m, 0.0);
  }
  void aerosol_rhs(const double* y, double* out) {
    std::copy(y, y + m_gas, concX.begin());
    reaction_rates(km, kfor.data(), concX.data(), out, rop.data(), src);
    for (int i = m_gas; i < m; ++i) out[i] = 0.0;
    for (int ip = 0; ip < aero->nParticles; ++ip)
      for (int is = 0; is < aero->nSimpol; ++is) simpol_particle(*aero, is, ip, T_aero, p_aero, number_conc, y, out);
  }
  void f(const double* y, double* out) {
    if (aero) {
      aerosol_rhs(y, out);
    } else {
      std::copy(y, y + m, concX.begin());
      reaction_rates(km, kfor.data(), concX.data(), out, rop.data(), src);
    }
    ++st.n_rhs;
  }
  void jac(const double* y) {
    if (aero) {
      // forward differences, column j with step 1e-8 max(|y_j|, 1e-20)
      aerosol_rhs(y, f0.data());
      std::copy(y, y + m, yh.begin());
      for (int j = 0; j < m; ++j) {
        const double h = 1e-8 * std::max(std::abs(y[j]), 1e-20);
        yh[j] = y[j] + h;
        aerosol_rhs(yh.data(), fh.data());
        const double hh = yh[j] - y[j];
        for (int i = 0; i < m; ++i) J[static_cast<size_t>(i) * m + j] = (fh[i] - f0[i]) / hh;
        yh[j] = y[j];
      }
    } else {
      std::copy(y, y + m, concX.begin());
      jacobian(km, kfor.data(), concX.data(), J.data());
    }
    ++st.n_jac;
  }

  // Simplified Newton: the factors of I - c_lu J (carried, or formed at the first iterate) serve
  // every iteration; they are re-formed once per stage at the current iterate when the max-norm
  // of the correction (rounded to FP32) shrinks by less than half. Converged when every
  // |dx_i| <= atol / sqrt(m) + rtol |y_i|, which implies the 2-norm test of the full Newton
  // method (||dx|| <= atol + rtol ||y||, by Minkowski's inequality).
  bool newton_simplified(double* y, const double* rhs, double c, const Settings& s, std::vector<double>& fy,
                         std::vector<double>& g, std::vector<double>& dx) {
    float prev = 0.f;
    bool refresh = !have_lu;
    const double atol_c = s.atol_newton / std::sqrt(static_cast<double>(m));
    for (int it = 0; it < s.max_newton; ++it) {
      f(y, fy.data());
      for (int i = 0; i < m; ++i) g[i] = -((y[i] - c * fy[i]) - rhs[i]);
      if (refresh) {
        jac(y);
        if (!lu.factor(J.data(), c)) return false;
        ++st.n_lu;
        have_lu = fresh = true;
        refresh = false;
        c_lu = c;
      }
      lu.solve(g.data(), dx.data());
      ++st.n_solve;
      ++st.n_newton_iter;
      bool finite = true, conv = true;
      float dmax = 0.f;
      for (int i = 0; i < m; ++i) {
        y[i] += dx[i];
        finite = finite && std::isfinite(dx[i]) && std::isfinite(y[i]);
        conv = conv && std::abs(dx[i]) <= atol_c + s.rtol_newton * std::abs(y[i]);
        dmax = std::max(dmax, static_cast<float>(std::abs(dx[i])));
      }
      if (!finite) return false;
      if (it > 0 && !fresh && dmax > 0.5f * prev) refresh = true;
      prev = dmax;
      if (conv) return true;
    }
    return false;
  }

  // Solves y - c f(y) = rhs by Newton from the guess in y.
  bool newton(double* y, const double* rhs, double c, const Settings& s, std::vector<double>& fy,
              std::vector<double>& g, std::vector<double>& dx) {
    if (s.simplified) {
      fresh = false;
      return newton_simplified(y, rhs, c, s, fy, g, dx);
    }
    for (int it = 0; it < s.max_newton; ++it) {
      f(y, fy.data());
      for (int i = 0; i < m; ++i) g[i] = -((y[i] - c * fy[i]) - rhs[i]);
      if (it % s.jac_interval == 0) {
        jac(y);
        if (!lu.factor(J.data(), c)) return false;
        ++st.n_lu;
      }
      lu.solve(g.data(), dx.data());
      ++st.n_solve;
      // Iterative refinement of the linear solve: FP64 residual with the FP64 Jacobian the
      // factors were built from, correction through the (FP32) factors.
      for (int k = 0; k < s.refine; ++k) {
        for (int i = 0; i < m; ++i) {
          double jd = 0.0;
          for (int j = 0; j < m; ++j) jd += J[static_cast<size_t>(i) * m + j] * dx[j];
          res[i] = g[i] - (dx[i] - c * jd);
        }
        lu.solve(res.data(), corr.data());
        ++st.n_solve;
        ++st.n_rhs;  // the Jacobian-vector product, counted like a right-hand side
        for (int i = 0; i < m; ++i) dx[i] += corr[i];
      }
      ++st.n_newton_iter;
      double sdx = 0.0, sy = 0.0;
      for (int i = 0; i < m; ++i) {
        y[i] += dx[i];
        sdx += dx[i] * dx[i];
        sy += y[i] * y[i];
      }
      const double ndx = std::sqrt(sdx), ny = std::sqrt(sy);
      if (!std::isfinite(ndx) || !std::isfinite(ny)) return false;
      if (it + 1 >= g_newton_min_iters && ndx <= s.atol_newton + s.rtol_newton * ny) return true;
    }
    return false;
  }

  int integrate(double* y, double t_beg, double t_end, double dt_in, double dt_min, double dt_max, const Settings& s,
                double& t_out, double& dt_out) {
    if (dt_in < 0.0) return TCHEM_GB_SAMPLE_NEGATIVE_DT;
    const double gamma = 2.0 - std::sqrt(2.0);
    const double d = 0.5 * gamma;                                  // diagonal coefficient of both stages
    const double cg = 1.0 / (gamma * (2.0 - gamma));               // BDF2 stage: weight of y_gamma
    const double cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));  // and of y_n
    const double kappa = (-3.0 * gamma * gamma + 4.0 * gamma - 2.0) / (12.0 * (2.0 - gamma));
    const double e0 = 1.0 / gamma, e1 = -1.0 / (gamma * (1.0 - gamma)), e2 = 1.0 / (1.0 - gamma);

    std::vector<double> fn(m), fg(m), f1(m), yg(m), y1(m), rhs(m), fy(m), g(m), dx(m), est(m), estf(m);
    double t = t_beg, dt = dt_in;
    int status = TCHEM_GB_SAMPLE_OK;
    std::vector<double> yp(m), ygp(m);  // simplified form: last accepted step's y_n and y_gamma
    double dtp = 0.0;
    bool have_prev = false;
    f(y, fn.data());
    for (int iter = 0; iter < s.max_iters && t < t_end; ++iter) {
      bool converged = false, last = false;
      for (int ntry = 0; ntry < 4; ++ntry) {
        if (!g_step_seq.empty() && ntry == 0)
          dt = g_step_seq[std::min<size_t>(static_cast<size_t>(st.n_steps), g_step_seq.size() - 1)];
        dt = std::min(std::max(dt, dt_min), dt_max);
        last = dt >= t_end - t;
        if (last) dt = t_end - t;
        if (!(dt > 0.0)) { status = TCHEM_GB_SAMPLE_DT_UNDERFLOW; break; }
        const double c = d * dt;
        // simplified form: keep the carried factors while c moved by at most 30%
        if (s.simplified && !(have_lu && std::abs(c / c_lu - 1.0) <= 0.3)) have_lu = false;
        // stage 1 (trapezoidal rule to t + gamma dt)
        for (int i = 0; i < m; ++i) { rhs[i] = y[i] + c * fn[i]; yg[i] = y[i]; }
        if (s.simplified && have_prev) {
          // stage-1 guess: the quadratic through the last step's y_{n-1}, y_{n-1+gamma}, y_n
          const double t0 = -dtp, t1 = -(1.0 - gamma) * dtp, tt = gamma * dt;
          const double l0 = (tt - t1) * tt / ((t0 - t1) * t0);
          const double l1 = (tt - t0) * tt / ((t1 - t0) * t1);
          const double l2 = (tt - t0) * (tt - t1) / (t0 * t1);
          for (int i = 0; i < m; ++i) yg[i] = l0 * yp[i] + l1 * ygp[i] + l2 * y[i];
        }
        bool ok = newton(yg.data(), rhs.data(), c, s, fy, g, dx);
        if (ok) {
          // stage 2 (BDF2 through t, t + gamma dt, t + dt)
          f(yg.data(), fg.data());
          for (int i = 0; i < m; ++i) { rhs[i] = cg * yg[i] - cn * y[i]; y1[i] = yg[i]; }
          if (s.simplified) {
            // stage-2 guess: the quadratic with p(t) = y_n, p'(t) = f_n, p(t + gamma dt) = y_gamma
            const double a = 1.0 / (gamma * gamma), b = dt * (1.0 - 1.0 / gamma);
            for (int i = 0; i < m; ++i) y1[i] = (1.0 - a) * y[i] + a * yg[i] + b * fn[i];
          }
          ok = newton(y1.data(), rhs.data(), c, s, fy, g, dx);
        }
        if (ok) { converged = true; break; }
        ++st.n_newton_fail;
        dt *= 0.5;
      }
      if (status != TCHEM_GB_SAMPLE_OK) break;
      if (!converged) { status = TCHEM_GB_SAMPLE_NEWTON_FAIL; break; }
      f(y1.data(), f1.data());
      // local error estimate, filtered through (I - d dt J)^{-1}
      for (int i = 0; i < m; ++i) est[i] = 2.0 * kappa * dt * (e0 * fn[i] + e1 * fg[i] + e2 * f1[i]);
      if (s.simplified) {
        // filter with the factors of I - c J(y_{n+1}), carried into the next step
        jac(y1.data());
        have_lu = lu.factor(J.data(), d * dt);
        c_lu = d * dt;
        if (have_lu) {
          ++st.n_lu;
          lu.solve(est.data(), estf.data());
          ++st.n_solve;
        } else {
          std::fill(estf.begin(), estf.end(), std::numeric_limits<double>::quiet_NaN());
        }
      } else {
        lu.solve(est.data(), estf.data());
        ++st.n_solve;
      }
      double err = 0.0;
      for (int i = 0; i < m; ++i) {
        const double w = s.tol_time[2 * i] + s.tol_time[2 * i + 1] * std::max(std::abs(y[i]), std::abs(y1[i]));
        err = std::max(err, std::abs(estf[i]) / w);
      }
      if (!std::isfinite(err)) { status = TCHEM_GB_SAMPLE_NONFINITE; break; }
      if (!g_step_seq.empty()) err = 0.0;  // the imposed step is accepted
      if (err <= 1.0 || dt <= dt_min) {
        if (tape_dt) {
          if (st.n_steps >= tape_cap) { status = TCHEM_GB_SAMPLE_TAPE_FULL; break; }
          tape_dt[st.n_steps] = dt;
        }
        t = last ? t_end : t + dt;
        if (s.simplified) {
          std::copy(y, y + m, yp.begin());
          ygp = yg;
          dtp = dt;
          have_prev = true;
        }
        std::copy(y1.begin(), y1.end(), y);
        fn.swap(f1);
        ++st.n_steps;
        double fac = err > 0.0 ? 0.9 * std::cbrt(1.0 / err) : 2.0;
        fac = std::max(0.2, std::min(2.0, fac));
        dt = std::min(dt * fac, dt_max);
        if (t + dt > t_end) dt = t_end - t;
      } else {
        ++st.n_rejected;
        dt *= std::max(0.2, 0.9 * std::cbrt(1.0 / err));
      }
    }
    t_out = t;
    dt_out = dt;
    if (status != TCHEM_GB_SAMPLE_OK) {
      for (int i = 0; i < m; ++i) y[i] = 0.0;
      t_out = t_end;
      dt_out = -1.0;
    }
    return status;
  }
};

template <typename LU_T>
void run_batch(const tchem_gb_kmcd_view* const* kms, const int32_t* mech_of_sample, int nbatch, const double* tol_newton,
               const double* tol_time, const tchem_gb_tadv* tadv, const double* state, double* t_out,
               double* dt_out, double* state_out, int32_t* status, tchem_gb_sample_stats* stats, int dim, int refine,
               bool simplified, const tchem_gb_e3sm_view* e3 = nullptr, const double* photo = nullptr,
               int n_photo = 0, const double* ext = nullptr) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const tchem_gb_kmcd_view& km = *kms[mech_of_sample ? mech_of_sample[b] : 0];
    const int n = km.nSpec, m = km.nSpec - km.nConstSpec;
    const tchem_gb_tadv& ta = tadv[b];
    tchem_gb_sample_stats st0{};
    if (stats) stats[b] = st0;
    if (t_out[b] >= ta.tend) {
      if (status) status[b] = TCHEM_GB_SAMPLE_SKIPPED;
      continue;
    }
    const double* row = state + static_cast<size_t>(b) * dim;
    double* out = state_out + static_cast<size_t>(b) * dim;
    const double rho = row[0], p = row[1], T = row[2];
    std::vector<double> y(row + 3, row + 3 + m);
    std::vector<double> xconst(row + 3 + m, row + 3 + n);
    // E3SM: rate constants once per sample at the initial state (they depend on constant
    // species only), external sources (zero when none are given) in place of the emissions.
    std::vector<double> kfor_e3, src_e3;
    if (e3) {
      kfor_e3.assign(km.nReac, 0.0);
      e3sm_kforward(km, *e3, T, p, row + 3, photo ? photo + static_cast<size_t>(b) * n_photo : nullptr, n_photo,
                    kfor_e3.data());
      src_e3.assign(m, 0.0);
      if (ext) std::copy(ext + static_cast<size_t>(b) * m, ext + static_cast<size_t>(b + 1) * m, src_e3.begin());
    }
    Sample<LU_T> smp(km, T, p, xconst.data(), nullptr, e3 ? kfor_e3.data() : nullptr, e3 ? src_e3.data() : nullptr);
    Settings s{ta.max_num_newton_iterations, std::max(1, ta.jacobian_interval), ta.num_time_iterations_per_interval,
               refine, simplified, tol_newton[0], tol_newton[1], tol_time};
    double to = 0.0, dto = 0.0;
    const int st = smp.integrate(y.data(), ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax, s, to, dto);
    if (status) status[b] = st;
    if (stats) stats[b] = smp.st;
    if (st == TCHEM_GB_SAMPLE_NEGATIVE_DT) continue;  // outputs untouched
    out[0] = rho;
    out[1] = p;
    out[2] = T;
    for (int i = 0; i < m; ++i) out[3 + i] = y[i];
    for (int i = 0; i < n - m; ++i) out[3 + m + i] = xconst[i];
    t_out[b] = to;
    dt_out[b] = dto;
  }
}

// --- discrete adjoint and forward sensitivities of the plain form ------------------------------
// On a recorded step sequence (the step-size control is not differentiated). Stages per step, with
// c = gamma/2 dt: (1) y_g - c f(y_g) = y_n + c f(y_n); (2) y_1 - c f(y_1) = cg y_g - cn y_n.

// nu_r . mu over the active species of reaction r.
double nu_dot(const tchem_gb_kmcd_view& km, int r, const double* mu) {
  const int m = km.nSpec - km.nConstSpec, S = km.maxSpecInReac, joff = S / 2;
  double d = 0.0;
  for (int j = 0; j < km.reacNreac[r]; ++j) {
    const int k = km.reacSidx[r * S + j];
    if (k < m) d += km.reacNuki[r * S + j] * mu[k];
  }
  for (int j = 0; j < km.reacNprod[r]; ++j) {
    const int k = km.reacSidx[r * S + j + joff];
    if (k < m) d += km.reacNuki[r * S + j + joff] * mu[k];
  }
  return d;
}

// out += scale * sum_r nu_r q_r dtheta_r (the rates of progress q from the last f()).
void add_ftheta(const tchem_gb_kmcd_view& km, const double* rop, const double* dth, double scale, double* out) {
  const int m = km.nSpec - km.nConstSpec, S = km.maxSpecInReac, joff = S / 2;
  for (int r = 0; r < km.nReac; ++r) {
    const double q = scale * rop[r] * dth[r];
    for (int j = 0; j < km.reacNreac[r]; ++j) {
      const int k = km.reacSidx[r * S + j];
      if (k < m) out[k] += km.reacNuki[r * S + j] * q;
    }
    for (int j = 0; j < km.reacNprod[r]; ++j) {
      const int k = km.reacSidx[r * S + j + joff];
      if (k < m) out[k] += km.reacNuki[r * S + j + joff] * q;
    }
  }
}

// Replays the recorded steps from y0: yn[j], yg[j] (m each) per step and the end state.
bool replay(Sample<double>& S, const double* y0, const double* dts, int nsteps, const Settings& s,
            std::vector<double>& yn, std::vector<double>& yg, std::vector<double>& yend) {
  const int m = S.m;
  const double gamma = 2.0 - std::sqrt(2.0), d = 0.5 * gamma;
  const double cg = 1.0 / (gamma * (2.0 - gamma)), cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
  std::vector<double> y(y0, y0 + m), fn(m), rv(m), g1(m), fy(m), g(m), dx(m);
  yn.assign(static_cast<size_t>(nsteps) * m, 0.0);
  yg.assign(static_cast<size_t>(nsteps) * m, 0.0);
  S.f(y.data(), fn.data());
  for (int j = 0; j < nsteps; ++j) {
    const double c = d * dts[j];
    std::copy(y.begin(), y.end(), yn.begin() + static_cast<size_t>(j) * m);
    for (int i = 0; i < m; ++i) { rv[i] = y[i] + c * fn[i]; g1[i] = y[i]; }
    if (!S.newton(g1.data(), rv.data(), c, s, fy, g, dx)) return false;
    std::copy(g1.begin(), g1.end(), yg.begin() + static_cast<size_t>(j) * m);
    for (int i = 0; i < m; ++i) { rv[i] = cg * g1[i] - cn * y[i]; y[i] = g1[i]; }
    if (!S.newton(y.data(), rv.data(), c, s, fy, g, dx)) return false;
    S.f(y.data(), fn.data());
  }
  yend = y;
  return true;
}

// lambda (in: dL/dy_end, out: dL/dy0) and gk += dL/dtheta over the recorded steps.
bool adjoint_sweep(Sample<double>& S, const std::vector<double>& yn, const std::vector<double>& yg,
                   const std::vector<double>& yend, const double* dts, int nsteps, double* lam, double* gk) {
  const int m = S.m, R = S.km.nReac;
  const double gamma = 2.0 - std::sqrt(2.0), d = 0.5 * gamma;
  const double cg = 1.0 / (gamma * (2.0 - gamma)), cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
  std::vector<double> mu1(m), mu2(m), tmp(m), y1(yend);
  for (int j = nsteps - 1; j >= 0; --j) {
    const double c = d * dts[j];
    const double* ynj = yn.data() + static_cast<size_t>(j) * m;
    const double* ygj = yg.data() + static_cast<size_t>(j) * m;
    S.jac(y1.data());
    if (!S.lu.factor(S.J.data(), c)) return false;
    S.lu.solve_t(lam, mu2.data());
    S.f(y1.data(), tmp.data());
    for (int r = 0; r < R; ++r) gk[r] += c * S.rop[r] * nu_dot(S.km, r, mu2.data());
    for (int i = 0; i < m; ++i) tmp[i] = cg * mu2[i];
    S.jac(ygj);
    if (!S.lu.factor(S.J.data(), c)) return false;
    S.lu.solve_t(tmp.data(), mu1.data());
    S.f(ygj, tmp.data());
    for (int r = 0; r < R; ++r) gk[r] += c * S.rop[r] * nu_dot(S.km, r, mu1.data());
    S.f(ynj, tmp.data());
    for (int r = 0; r < R; ++r) gk[r] += c * S.rop[r] * nu_dot(S.km, r, mu1.data());
    S.jac(ynj);
    for (int jj = 0; jj < m; ++jj) {
      double acc = 0.0;
      for (int i = 0; i < m; ++i) acc += S.J[static_cast<size_t>(i) * m + jj] * mu1[i];
      lam[jj] = -cn * mu2[jj] + mu1[jj] + c * acc;
    }
    std::copy(ynj, ynj + m, y1.begin());
  }
  return true;
}

// Forward sensitivity: s (in: dy0, out: dy_end) along dtheta over the recorded steps.
bool tangent_sweep(Sample<double>& S, const std::vector<double>& yn, const std::vector<double>& yg,
                   const std::vector<double>& yend, const double* dts, int nsteps, const double* dth, double* sv) {
  const int m = S.m;
  const double gamma = 2.0 - std::sqrt(2.0), d = 0.5 * gamma;
  const double cg = 1.0 / (gamma * (2.0 - gamma)), cn = (1.0 - gamma) * (1.0 - gamma) / (gamma * (2.0 - gamma));
  std::vector<double> b(m), sg(m), tmp(m);
  for (int j = 0; j < nsteps; ++j) {
    const double c = d * dts[j];
    const double* ynj = yn.data() + static_cast<size_t>(j) * m;
    const double* ygj = yg.data() + static_cast<size_t>(j) * m;
    const double* y1 = j + 1 < nsteps ? yn.data() + static_cast<size_t>(j + 1) * m : yend.data();
    S.jac(ynj);
    for (int i = 0; i < m; ++i) {
      double acc = 0.0;
      for (int k = 0; k < m; ++k) acc += S.J[static_cast<size_t>(i) * m + k] * sv[k];
      b[i] = sv[i] + c * acc;
    }
    S.f(ynj, tmp.data());
    add_ftheta(S.km, S.rop.data(), dth, c, b.data());
    S.f(ygj, tmp.data());
    add_ftheta(S.km, S.rop.data(), dth, c, b.data());
    S.jac(ygj);
    if (!S.lu.factor(S.J.data(), c)) return false;
    S.lu.solve(b.data(), sg.data());
    for (int i = 0; i < m; ++i) b[i] = cg * sg[i] - cn * sv[i];
    S.f(y1, tmp.data());
    add_ftheta(S.km, S.rop.data(), dth, c, b.data());
    S.jac(y1);
    if (!S.lu.factor(S.J.data(), c)) return false;
    S.lu.solve(b.data(), sv);
  }
  return true;
}

struct SampleSetup {
  std::vector<double> y0, xconst;
  double T = 0.0, p = 0.0;
};

SampleSetup setup_row(const tchem_gb_kmcd_view& km, const double* state, int b) {
  const int n = km.nSpec, m = n - km.nConstSpec;
  const double* row = state + static_cast<size_t>(b) * (n + 3);
  SampleSetup u;
  u.p = row[1];
  u.T = row[2];
  u.y0.assign(row + 3, row + 3 + m);
  u.xconst.assign(row + 3 + m, row + 3 + n);
  return u;
}

Settings replay_settings(const tchem_gb_tadv& ta, const double* tol_newton) {
  return Settings{ta.max_num_newton_iterations, std::max(1, ta.jacobian_interval), ta.num_time_iterations_per_interval,
                  0, false, tol_newton[0], tol_newton[1], nullptr};
}

}  // namespace

extern "C" {

// One FP32 matrix factored as the tensor-core LU does (DenseLU::factor_blocked with `keep`
// mantissa bits in the trailing-update operands; 23 = no rounding): lu[n][n] holds the unit-lower
// L below the diagonal and U on and above it, piv[k] the row swapped with row k.
int oracle_lu_factor_blocked(int n, const float* a_in, int keep, float* lu, int32_t* piv) {
  if (n < 1 || !a_in || !lu || !piv || keep < 1 || keep > 23) return TCHEM_GB_ERR_ARG;
  DenseLU<float> f;
  f.resize(n);
  std::copy(a_in, a_in + static_cast<size_t>(n) * n, f.a.begin());
  if (!f.factor_blocked(keep)) return TCHEM_GB_ERR_DEVICE;
  std::copy(f.a.begin(), f.a.end(), lu);
  for (int k = 0; k < n; ++k) piv[k] = f.piv[k];
  return TCHEM_GB_OK;
}

int oracle_set_lu_tile_bits(int bits) {
  if (bits != 0 && (bits < 1 || bits > 23)) return TCHEM_GB_ERR_ARG;
  g_lu_tile_bits = bits;
  return TCHEM_GB_OK;
}

// Static elimination order of FP32 factorizations of n x n matrices (n = 0: partial pivoting).
int oracle_set_newton_min_iterations(int k) {
  if (k < 1 || k > 20) return TCHEM_GB_ERR_ARG;
  g_newton_min_iters = k;
  return TCHEM_GB_OK;
}

int oracle_set_step_sequence(int n, const double* dt) {
  if (n < 0 || (n > 0 && !dt)) return TCHEM_GB_ERR_ARG;
  for (int k = 0; k < n; ++k)
    if (!(dt[k] > 0.0)) return TCHEM_GB_ERR_ARG;
  g_step_seq.assign(dt, dt + n);
  return TCHEM_GB_OK;
}

int oracle_set_lu_static_order(int n, const int32_t* order) {
  if (n < 0 || (n > 0 && !order)) return TCHEM_GB_ERR_ARG;
  std::vector<int> o(order, order + n), seen(n, 0);
  for (int k = 0; k < n; ++k) {
    if (o[k] < 0 || o[k] >= n || seen[o[k]]) return TCHEM_GB_ERR_ARG;
    seen[o[k]] = 1;
  }
  g_lu_order = o;
  return TCHEM_GB_OK;
}

int oracle_kforward(const tchem_gb_kmcd_view* km, double T, double p, double* kfor) {
  if (!km || !kfor) return TCHEM_GB_ERR_ARG;
  kforward(*km, T, p, kfor);
  return TCHEM_GB_OK;
}

int oracle_reaction_rates(const tchem_gb_kmcd_view* km, double T, double p, const double* x, double* omega) {
  if (!km || !x || !omega) return TCHEM_GB_ERR_ARG;
  std::vector<double> kfor(km->nReac), rop(km->nReac);
  kforward(*km, T, p, kfor.data());
  reaction_rates(*km, kfor.data(), x, omega, rop.data());
  return TCHEM_GB_OK;
}

int oracle_jacobian(const tchem_gb_kmcd_view* km, double T, double p, const double* x, double* J) {
  if (!km || !x || !J) return TCHEM_GB_ERR_ARG;
  std::vector<double> kfor(km->nReac);
  kforward(*km, T, p, kfor.data());
  jacobian(*km, kfor.data(), x, J);
  return TCHEM_GB_OK;
}

int oracle_time_advance(const tchem_gb_kmcd_view* const* kms, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                        const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                        const double* state, double* t_out, double* dt_out, double* state_out, int32_t* status,
                        tchem_gb_sample_stats* stats, int lu_fp32, int simplified, int nthreads) {
  if (!kms || n_mechs <= 0 || nbatch < 0 || !tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out ||
      !state_out)
    return TCHEM_GB_ERR_ARG;
  if (mech_of_sample)
    for (int b = 0; b < nbatch; ++b)
      if (mech_of_sample[b] < 0 || mech_of_sample[b] >= n_mechs) return TCHEM_GB_ERR_ARG;
  // Every row has the width of the widest mechanism (one state array for all samples).
  int dim = 0;
  for (int i = 0; i < n_mechs; ++i) dim = std::max(dim, kms[i]->nSpec + 3);
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  if (lu_fp32)
    run_batch<float>(kms, mech_of_sample, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, status,
                     stats, dim, lu_fp32 - 1, simplified != 0);
  else
    run_batch<double>(kms, mech_of_sample, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, status,
                      stats, dim, 0, simplified != 0);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return TCHEM_GB_OK;
}

int oracle_e3sm_kforward(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                         const double* x, const double* photo, int n_photo, double* kfor) {
  if (!km || !e3 || !x || !kfor || n_photo < 0) return TCHEM_GB_ERR_ARG;
  e3sm_kforward(*km, *e3, T, p, x, photo, photo ? n_photo : 0, kfor);
  return TCHEM_GB_OK;
}

int oracle_e3sm_rate_of_progress(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                                 const double* x, const double* photo, int n_photo, double* rop) {
  if (!km || !e3 || !x || !rop || n_photo < 0) return TCHEM_GB_ERR_ARG;
  std::vector<double> kfor(km->nReac), omega(km->nSpec - km->nConstSpec), zero(km->nSpec - km->nConstSpec, 0.0);
  e3sm_kforward(*km, *e3, T, p, x, photo, photo ? n_photo : 0, kfor.data());
  reaction_rates(*km, kfor.data(), x, omega.data(), rop, zero.data());
  return TCHEM_GB_OK;
}

int oracle_e3sm_net_production_rates(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, double T, double p,
                                     const double* x, const double* photo, int n_photo, const double* ext,
                                     double* omega) {
  if (!km || !e3 || !x || !omega || n_photo < 0) return TCHEM_GB_ERR_ARG;
  const int m = km->nSpec - km->nConstSpec;
  std::vector<double> kfor(km->nReac), rop(km->nReac), zero(m, 0.0);
  e3sm_kforward(*km, *e3, T, p, x, photo, photo ? n_photo : 0, kfor.data());
  reaction_rates(*km, kfor.data(), x, omega, rop.data(), ext ? ext : zero.data());
  return TCHEM_GB_OK;
}

int oracle_e3sm_time_advance(const tchem_gb_kmcd_view* km, const tchem_gb_e3sm_view* e3, int nbatch,
                             const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                             const double* state, const double* photo, int n_photo, const double* ext, double* t_out,
                             double* dt_out, double* state_out, int32_t* status, tchem_gb_sample_stats* stats,
                             int lu_fp32, int simplified, int nthreads) {
  if (!km || !e3 || nbatch < 0 || n_photo < 0 || !tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out ||
      !state_out)
    return TCHEM_GB_ERR_ARG;
  if (e3sm_kfor_depends_on_state(*km, *e3)) return TCHEM_GB_ERR_UNSUPPORTED;
  const tchem_gb_kmcd_view* kms[1] = {km};
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  if (lu_fp32)
    run_batch<float>(kms, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, status, stats,
                     km->nSpec + 3, lu_fp32 - 1, simplified != 0, e3, photo, photo ? n_photo : 0, ext);
  else
    run_batch<double>(kms, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out, status, stats,
                      km->nSpec + 3, 0, simplified != 0, e3, photo, photo ? n_photo : 0, ext);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return TCHEM_GB_OK;
}

int oracle_simpol_rhs(const tchem_gb_aero_view* av, int i_simpol, double T, double p, const double* number_conc,
                      const double* x, double* omega) {
  if (!av || !number_conc || !x || !omega || i_simpol < 0 || i_simpol >= av->nSimpol) return TCHEM_GB_ERR_ARG;
  for (int ip = 0; ip < av->nParticles; ++ip) simpol_particle(*av, i_simpol, ip, T, p, number_conc, x, omega);
  return TCHEM_GB_OK;
}

int oracle_aerosol_rhs(const tchem_gb_kmcd_view* km, const tchem_gb_aero_view* av, double T, double p,
                       const double* number_conc, const double* x, const double* xconst, double* omega) {
  if (!km || !av || !number_conc || !x || !omega || (km->nConstSpec > 0 && !xconst)) return TCHEM_GB_ERR_ARG;
  Sample<double> smp(*km, T, p, xconst);
  smp.set_aerosol(av, number_conc, T, p);
  smp.f(x, omega);
  return TCHEM_GB_OK;
}

int oracle_aerosol_time_advance(const tchem_gb_kmcd_view* km, const tchem_gb_aero_view* av, int nbatch,
                                const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                                const double* state, const double* number_conc, double* t_out, double* dt_out,
                                double* state_out, int32_t* status, tchem_gb_sample_stats* stats, int nthreads) {
  if (!km || !av || nbatch < 0 || !tol_newton || !tol_time || !tadv || !state || !number_conc || !t_out || !dt_out ||
      !state_out || av->nParticles < 1)
    return TCHEM_GB_ERR_ARG;
  const int n = km->nSpec, mg = n - km->nConstSpec;
  const int npart = av->nParticles * av->nSpec;
  const int dim = 3 + n + npart;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const tchem_gb_tadv& ta = tadv[b];
    if (stats) stats[b] = tchem_gb_sample_stats{};
    if (t_out[b] >= ta.tend) {
      if (status) status[b] = TCHEM_GB_SAMPLE_SKIPPED;
      continue;
    }
    const double* row = state + static_cast<size_t>(b) * dim;
    double* out = state_out + static_cast<size_t>(b) * dim;
    const double p = row[1], T = row[2];
    // ODE vector [active gas, particles]; the constant gas species sit between them in the row
    std::vector<double> y(mg + npart);
    std::copy(row + 3, row + 3 + mg, y.begin());
    std::copy(row + 3 + n, row + 3 + n + npart, y.begin() + mg);
    Sample<double> smp(*km, T, p, row + 3 + mg);
    smp.set_aerosol(av, number_conc + static_cast<size_t>(b) * av->nParticles, T, p);
    Settings s{ta.max_num_newton_iterations, std::max(1, ta.jacobian_interval), ta.num_time_iterations_per_interval,
               0, false, tol_newton[0], tol_newton[1], tol_time};
    double to = 0.0, dto = 0.0;
    const int st = smp.integrate(y.data(), ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax, s, to, dto);
    if (status) status[b] = st;
    if (stats) stats[b] = smp.st;
    if (st == TCHEM_GB_SAMPLE_NEGATIVE_DT) continue;
    // src/core/TChem_AerosolChemistry.cpp:168-172: active gas and particles back, T; rho, p and the
    // constant species are left as they are (copied through here)
    std::copy(row, row + dim, out);
    std::copy(y.begin(), y.begin() + mg, out + 3);
    std::copy(y.begin() + mg, y.end(), out + 3 + n);
    t_out[b] = to;
    dt_out[b] = dto;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return TCHEM_GB_OK;
}

int oracle_time_advance_record(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton,
                               const double* tol_time, const double* k_scale, const tchem_gb_tadv* tadv,
                               const double* state, double* t_out, double* dt_out, double* state_out,
                               int32_t* status, double* tape_dt, int32_t* tape_nsteps, int tape_cap, int nthreads) {
  if (!km || nbatch < 0 || !tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out || !state_out || !status ||
      !tape_dt || !tape_nsteps || tape_cap < 1)
    return TCHEM_GB_ERR_ARG;
  const int n = km->nSpec, m = n - km->nConstSpec;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const tchem_gb_tadv& ta = tadv[b];
    const SampleSetup u = setup_row(*km, state, b);
    Sample<double> smp(*km, u.T, u.p, u.xconst.data(), k_scale);
    smp.tape_dt = tape_dt + static_cast<size_t>(b) * tape_cap;
    smp.tape_cap = tape_cap;
    Settings s{ta.max_num_newton_iterations, std::max(1, ta.jacobian_interval), ta.num_time_iterations_per_interval,
               0, false, tol_newton[0], tol_newton[1], tol_time};
    std::vector<double> y(u.y0);
    double to = 0.0, dto = 0.0;
    status[b] = smp.integrate(y.data(), ta.tbeg, ta.tend, ta.dt, ta.dtmin, ta.dtmax, s, to, dto);
    tape_nsteps[b] = smp.st.n_steps;
    double* out = state_out + static_cast<size_t>(b) * (n + 3);
    const double* row = state + static_cast<size_t>(b) * (n + 3);
    std::copy(row, row + n + 3, out);
    for (int i = 0; i < m; ++i) out[3 + i] = y[i];
    t_out[b] = to;
    dt_out[b] = dto;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return TCHEM_GB_OK;
}

int oracle_replay(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                  const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                  int tape_cap, double* y_end, int nthreads) {
  if (!km || nbatch < 0 || !tol_newton || !tadv || !state || !tape_dt || !tape_nsteps || !y_end) return TCHEM_GB_ERR_ARG;
  const int m = km->nSpec - km->nConstSpec;
  int rc = TCHEM_GB_OK;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const SampleSetup u = setup_row(*km, state, b);
    Sample<double> smp(*km, u.T, u.p, u.xconst.data(), k_scale);
    std::vector<double> yn, yg, ye;
    if (!replay(smp, u.y0.data(), tape_dt + static_cast<size_t>(b) * tape_cap, tape_nsteps[b],
                replay_settings(tadv[b], tol_newton), yn, yg, ye))
      rc = TCHEM_GB_ERR_DEVICE;
    else
      std::copy(ye.begin(), ye.end(), y_end + static_cast<size_t>(b) * m);
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return rc;
}

int oracle_adjoint(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                   const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                   int tape_cap, const double* lambda, double* grad_x0, double* grad_k, int nthreads) {
  if (!km || nbatch < 0 || !tol_newton || !tadv || !state || !tape_dt || !tape_nsteps || !lambda || !grad_x0 ||
      !grad_k)
    return TCHEM_GB_ERR_ARG;
  const int m = km->nSpec - km->nConstSpec, R = km->nReac;
  int rc = TCHEM_GB_OK;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const SampleSetup u = setup_row(*km, state, b);
    Sample<double> smp(*km, u.T, u.p, u.xconst.data(), k_scale);
    std::vector<double> yn, yg, ye;
    const double* dts = tape_dt + static_cast<size_t>(b) * tape_cap;
    double* lam = grad_x0 + static_cast<size_t>(b) * m;
    double* gk = grad_k + static_cast<size_t>(b) * R;
    std::copy(lambda + static_cast<size_t>(b) * m, lambda + static_cast<size_t>(b + 1) * m, lam);
    std::fill(gk, gk + R, 0.0);
    if (!replay(smp, u.y0.data(), dts, tape_nsteps[b], replay_settings(tadv[b], tol_newton), yn, yg, ye) ||
        !adjoint_sweep(smp, yn, yg, ye, dts, tape_nsteps[b], lam, gk))
      rc = TCHEM_GB_ERR_DEVICE;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return rc;
}

int oracle_tangent(const tchem_gb_kmcd_view* km, int nbatch, const double* tol_newton, const double* k_scale,
                   const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const int32_t* tape_nsteps,
                   int tape_cap, const double* dx0, const double* dtheta, double* dy_end, int nthreads) {
  if (!km || nbatch < 0 || !tol_newton || !tadv || !state || !tape_dt || !tape_nsteps || !dx0 || !dtheta || !dy_end)
    return TCHEM_GB_ERR_ARG;
  const int m = km->nSpec - km->nConstSpec, R = km->nReac;
  int rc = TCHEM_GB_OK;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nbatch; ++b) {
    const SampleSetup u = setup_row(*km, state, b);
    Sample<double> smp(*km, u.T, u.p, u.xconst.data(), k_scale);
    std::vector<double> yn, yg, ye;
    const double* dts = tape_dt + static_cast<size_t>(b) * tape_cap;
    double* sv = dy_end + static_cast<size_t>(b) * m;
    std::copy(dx0 + static_cast<size_t>(b) * m, dx0 + static_cast<size_t>(b + 1) * m, sv);
    if (!replay(smp, u.y0.data(), dts, tape_nsteps[b], replay_settings(tadv[b], tol_newton), yn, yg, ye) ||
        !tangent_sweep(smp, yn, yg, ye, dts, tape_nsteps[b], dtheta + static_cast<size_t>(b) * R, sv))
      rc = TCHEM_GB_ERR_DEVICE;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return rc;
}

}  // extern "C"
