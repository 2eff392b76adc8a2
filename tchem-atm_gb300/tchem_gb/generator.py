"""Seeded generator of CB05-shaped mechanisms and box-model sample batches.

Mechanisms are written as reference-format (NCAR-version) YAML, so they go through the same
front end as any user mechanism. The shape follows the CB05 example mechanism of the
reference (src/examples/runs/atmospheric_chemistry/CB05CL_AE5/config_full_gas.yaml and
docs/CB5_example.md:5-14): Arrhenius, Troe and photolysis reactions, the latter encoded as
ARRHENIUS with A = J and B = C = 0, plus the constant species M.

Per reaction: 1-2 reactants and 1-4 products with integer stoichiometry. Species carry an
integer weight and no reaction creates weight, so every mechanism is mass-non-increasing and
concentrations stay bounded over long horizons.

Rate parameters (the benchmark's distributions): Arrhenius log10 A ~ U[-16, -10], B ~ U[-3, 3],
C ~ U[-2000, 2000] (the reference's form is exp(+C/T); the range is symmetric), D = 300, E = 0;
Troe with CB05-like falloff parameters; photolysis J log-uniform in [1e-6, 1e-2] s^-1
(J = 0 for a "night" variant).

Samples: T ~ U[260, 310] K, p ~ U[0.8, 1.05] atm (stored in Pa), number densities
log-uniform in [1e2, 1e12] molecules cm^-3 stored as x = n / conv with conv = CONV_PPM p / T
(the unit the reference's rate law uses), M = 1e6.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

CONV_PPM = 7.24296358205307e10
ATM = 101325.0


@dataclass
class MechanismSpec:
    n_species: int = 51
    n_reactions: int = 156
    frac_troe: float = 0.10
    frac_photolysis: float = 0.30
    seed: int = 20251203
    max_reactants: int = 2
    max_products: int = 4


def _fmt(x: float) -> str:
    return repr(float(x))


def mechanism_yaml(spec: MechanismSpec = MechanismSpec(), night: bool = False) -> str:
    """Reference-format YAML of a seeded CB05-shaped mechanism.

    ``night=True`` writes the same mechanism with every photolysis rate set to 0 (the
    per-sample mechanism variant of the reference's kmcds overload).
    """
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    m, R = spec.n_species, spec.n_reactions
    names = [f"S{i:03d}" for i in range(m)]
    weight = rng.integers(1, 5, size=m)
    weight[: max(1, m // 8)] = 1  # a pool of light end products
    n_troe = int(round(spec.frac_troe * R))
    n_photo = int(round(spec.frac_photolysis * R))
    types = np.array(["TROE"] * n_troe + ["PHOTO"] * n_photo + ["ARRHENIUS"] * (R - n_troe - n_photo))
    rng.shuffle(types)

    def pick_products(budget: int, exclude: set[int], kmax: int) -> dict[int, int]:
        k_target = int(rng.choice(np.arange(1, kmax + 1), p=[0.35, 0.35, 0.2, 0.1][:kmax] /
                                  np.sum([0.35, 0.35, 0.2, 0.1][:kmax])))
        prods: dict[int, int] = {}
        for _ in range(k_target):
            cand = [s for s in range(m) if weight[s] <= budget and s not in exclude and s not in prods]
            if not cand:
                break
            s = int(rng.choice(cand))
            coef = 2 if (weight[s] * 2 <= budget and rng.random() < 0.1) else 1
            prods[s] = coef
            budget -= coef * int(weight[s])
            if budget <= 0:
                break
        if not prods:  # always at least one product: the lightest species not among the reactants
            cand = [s for s in range(m) if s not in exclude]
            s = int(min(cand, key=lambda i: weight[i]))
            prods[s] = 1
        return prods

    lines = ["NCAR-version: v1.0", "constant_species:", "- description: third body", "  name: M", "species:"]
    for n in names:
        lines += [f"- name: {n}"]
    lines.append("reactions:")
    for r in range(R):
        t = types[r]
        if t == "PHOTO":
            s = int(rng.integers(m))
            reac = {s: 1}
        elif t == "TROE":
            a, b = rng.choice(m, size=2, replace=False)
            reac = {int(a): 1, int(b): 1}
        else:
            nr = 1 if rng.random() < 0.3 else 2
            if nr == 1:
                reac = {int(rng.integers(m)): 1}
            elif rng.random() < 0.05:
                reac = {int(rng.integers(m)): 2}
            else:
                a, b = rng.choice(m, size=2, replace=False)
                reac = {int(a): 1, int(b): 1}
        budget = int(sum(weight[s] * c for s, c in reac.items()))
        prods = pick_products(budget, set(reac), 2 if t == "TROE" else spec.max_products)
        lines.append(f"- MUSICA_name: R{r + 1}")
        lines.append("  reactants:")
        lines += [f"    {names[s]}: {c}" for s, c in reac.items()]
        lines.append("  products:")
        lines += [f"    {names[s]}: {c}" for s, c in prods.items()]
        if t == "PHOTO":
            J = 10.0 ** rng.uniform(-6.0, -2.0)
            lines += ["  type: ARRHENIUS", "  coefficients:", f"    A: {_fmt(0.0 if night else J)}",
                      "  note: PHOTOLYSIS (A := photolysis rate)"]
        elif t == "TROE":
            k0_A = 10.0 ** rng.uniform(-33.0, -30.0)
            k0_B = rng.uniform(-4.0, 0.0)
            kinf_A = 10.0 ** rng.uniform(-12.0, -10.0)
            kinf_B = rng.uniform(-1.0, 0.0)
            lines += ["  type: TROE", "  coefficients:", f"    k0_A: {_fmt(k0_A)}", f"    k0_B: {_fmt(k0_B)}",
                      "    k0_C: 0.0", f"    kinf_A: {_fmt(kinf_A)}", f"    kinf_B: {_fmt(kinf_B)}",
                      "    kinf_C: 0.0", "    Fc: 0.6", "    N: 1.0"]
        else:
            A = 10.0 ** rng.uniform(-16.0, -10.0)
            B = rng.uniform(-3.0, 3.0)
            Cc = rng.uniform(-2000.0, 2000.0)
            lines += ["  type: ARRHENIUS", "  coefficients:", f"    A: {_fmt(A)}", f"    B: {_fmt(B)}",
                      f"    C: {_fmt(Cc)}", "    D: 300.0", "    E: 0.0"]
    return "\n".join(lines) + "\n"


def sample_states(n_samples: int, n_active: int, n_const: int = 1, seed: int = 7,
                  const_values: tuple[float, ...] = (1.0e6,)) -> np.ndarray:
    """state[B, n_active + n_const + 3] = [rho=0, p (Pa), T (K), x_active..., x_const...]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    B = int(n_samples)
    T = rng.uniform(260.0, 310.0, size=B)
    p = rng.uniform(0.8, 1.05, size=B) * ATM
    n = 10.0 ** rng.uniform(2.0, 12.0, size=(B, n_active))
    conv = CONV_PPM * p / T
    state = np.zeros((B, n_active + n_const + 3))
    state[:, 1] = p
    state[:, 2] = T
    state[:, 3:3 + n_active] = n / conv[:, None]
    for i in range(n_const):
        state[:, 3 + n_active + i] = const_values[i] if i < len(const_values) else 0.0
    return state


def scenario_yaml(state: np.ndarray, species_names: list[str], n_active: int) -> str:
    """Reference-format scenario (environmental_conditions + initial_state, units mol m-3)."""
    p = ", ".join(_fmt(v) for v in state[:, 1])
    T = ", ".join(_fmt(v) for v in state[:, 2])
    lines = ["NCAR-version: v1.0", "environmental_conditions:", "  pressure:", "    evolving: 'false'",
             f"    initial_value: [{p}]", "    units: Pa", "  temperature:", "    evolving: 'false'",
             f"    initial_value: [{T}]", "    units: K", "initial_state:"]
    for i, name in enumerate(species_names):
        vals = ", ".join(_fmt(v) for v in state[:, 3 + i])
        lines += [f"  {name}:", f"    initial_value: [{vals}]", "    units: mol m-3"]
    return "\n".join(lines) + "\n"
