"""Second reading of an NCAR-format mechanism file, independent of the engine's parser (test
infrastructure only: it checks the engine's front end, it is not part of the product).

The engine parses mechanisms with its own C++ YAML-subset reader (tchem-atm_gb300/csrc/yaml_lite.cpp,
kinetic_model.cpp), and the CPU oracle computes on the tables that parser builds, so a parser bug would
cancel out of every GPU-vs-oracle comparison. This module reads the same files with a separate reader
written here, restates the table rules of KineticModelData::initChemNCAR
(src/core/TChem_KineticModelData.cpp:80-1017) for the box-model rate forms, and evaluates the rate
constants (KForwardAerosol, src/core/impl/TChem_Impl_KForwardAerosol.hpp:44-145) and net production
rates (ReactionRatesAerosol, src/core/impl/TChem_Impl_ReactionRatesAerosol.hpp:80-138) with numpy, so
tests can compare both the engine's tables and the oracle's rates against it.

Rules restated (file:line of the reference):
* species first, then constant_species, in file order (:91-140); M must exist (:142-156);
* reactants and products keyed by species index in increasing order (a std::map, :196-225); reactant
  coefficients negative at columns 0.., products from column maxSpecInReac / 2 (:318-337);
  maxSpecInReac = 2 * max over reactions of max(#reactants, #products) (:246-253, 268);
* ARRHENIUS: A (default 1, /60 when time_unit is min), B (0), C (0) or Ea (C = -Ea / KBOLT), D (300),
  E (0) (:386-433); TROE: k0_A * 1e6, k0_B, k0_C, kinf_A, kinf_B, kinf_C, Fc (0.6), N (1) (:690-755);
  CMAQ_H2O2: k1_A, k1_B, k1_C, k2_A * 1e6, k2_B, k2_C (:454-503);
* convExponent = sum of reactant |nu| - 1 (:939-947); EMISSION sources (:893-936).
"""
from __future__ import annotations

import math
import re

import numpy as np

CONV_PPM = 7.24296358205307e10
KBOLT = 1.3806504e-23  # src/core/TChem_Util.hpp:195


# ---- a reader for the YAML subset of the mechanism files -----------------------------------------

def _scalar(tok: str):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"" and t[-1] == t[0]:
        return t[1:-1]
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [] if not inner else [_scalar(x) for x in inner.split(",")]
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        return t


def _lines(text: str):
    out = []
    for raw in text.splitlines():
        line = raw.split(" #", 1)[0].rstrip() if " #" in raw else raw.rstrip()
        if not line.strip() or line.lstrip().startswith("#"):
            continue
        out.append((len(line) - len(line.lstrip(" ")), line.strip()))
    return out


def _block(lines, i: int, ind: int):
    """Parses the block starting at lines[i] with indentation ind; returns (value, next index)."""
    if lines[i][1].startswith("- ") or lines[i][1] == "-":
        items = []
        while i < len(lines) and lines[i][0] == ind and (lines[i][1].startswith("- ") or lines[i][1] == "-"):
            body = lines[i][1][1:].strip()
            if not body:
                val, i = _block(lines, i + 1, lines[i + 1][0])
                items.append(val)
                continue
            # a list item that starts a map: "- key: value" continues at ind + 2
            sub = [(ind + 2, body)]
            j = i + 1
            while j < len(lines) and lines[j][0] > ind:
                sub.append(lines[j])
                j += 1
            if ":" in body and not body.startswith("["):
                val, _ = _block(sub, 0, ind + 2)
            else:
                val = _scalar(body)
            items.append(val)
            i = j
        return items, i
    d = {}
    while i < len(lines) and lines[i][0] == ind and not lines[i][1].startswith("- "):
        m = re.match(r"^('[^']*'|\"[^\"]*\"|[^:]+):\s*(.*)$", lines[i][1])
        if not m:
            raise ValueError(f"cannot read line: {lines[i][1]!r}")
        key = _scalar(m.group(1))
        rest = m.group(2)
        if rest:
            i += 1
            while i < len(lines) and lines[i][0] > ind:  # a plain scalar continued on deeper lines
                rest += " " + lines[i][1]
                i += 1
            d[key] = _scalar(rest)
        elif i + 1 < len(lines) and lines[i + 1][0] > ind:
            d[key], i = _block(lines, i + 1, lines[i + 1][0])
        elif i + 1 < len(lines) and lines[i + 1][0] == ind and lines[i + 1][1].startswith("- "):
            d[key], i = _block(lines, i + 1, ind)  # a list at the key's own indentation
        else:
            d[key] = None
            i += 1
    return d, i


def read_yaml_subset(text: str):
    lines = _lines(text)
    val, _ = _block(lines, 0, lines[0][0])
    return val


# ---- the tables of initChemNCAR (box-model rate forms) --------------------------------------------

def tables(text: str) -> dict:
    root = read_yaml_subset(text)
    names = [s["name"] for s in root.get("species") or []]
    const = [s["name"] for s in root.get("constant_species") or []]
    allnames = names + const
    index: dict[str, int] = {}
    for i, n in enumerate(allnames):
        index.setdefault(n, i)  # std::map::insert keeps the first index of a repeated name (:110-135)
    if "M" not in index:
        raise ValueError("M species does not exist")
    reactions = root.get("reactions") or []
    R = len(reactions)
    reac_info, prod_info = [], []
    for rx in reactions:
        rs = {index[k]: float(v) for k, v in (rx.get("reactants") or {}).items()}
        ps = {index[k]: float(v) for k, v in (rx.get("products") or {}).items() if k in index}
        reac_info.append(dict(sorted(rs.items())))
        prod_info.append(dict(sorted(ps.items())))
    nreac = np.array([len(rx.get("reactants") or {}) for rx in reactions], dtype=np.int32)
    nprod = np.array([len(rx.get("products") or {}) for rx in reactions], dtype=np.int32)
    S = 2 * int(max(nreac.max(initial=0), nprod.max(initial=0)))
    sidx = np.zeros((R, S), dtype=np.int32)
    nuki = np.zeros((R, S))
    for r in range(R):
        for c, (k, v) in enumerate(reac_info[r].items()):
            sidx[r, c], nuki[r, c] = k, -v
        for c, (k, v) in enumerate(prod_info[r].items()):
            sidx[r, S // 2 + c], nuki[r, S // 2 + c] = k, v
    conv_exp = np.array([int(round(np.abs(nuki[r, :nreac[r]]).sum())) - 1 for r in range(R)], dtype=np.int32)
    rate = []
    for r, rx in enumerate(reactions):
        t = rx["type"]
        co = rx.get("coefficients") or {}
        per_min = rx.get("time_unit") == "min"
        scale = (lambda a: a / 60.0) if per_min else (lambda a: a)
        if t == "ARRHENIUS":
            if "Ea" in co and "C" in co:
                raise ValueError("Ea and C both given")
            C = -float(co["Ea"]) / KBOLT if "Ea" in co else float(co.get("C", 0.0))
            rate.append(("ARRHENIUS", [scale(float(co.get("A", 1.0))), float(co.get("B", 0.0)), C,
                                       float(co.get("D", 300.0)), float(co.get("E", 0.0))]))
        elif t == "TROE":
            rate.append(("TROE", [scale(float(co.get("k0_A", 1.0))) * 1e6, float(co.get("k0_B", 0.0)),
                                  float(co.get("k0_C", 0.0)), scale(float(co.get("kinf_A", 1.0))),
                                  float(co.get("kinf_B", 0.0)), float(co.get("kinf_C", 0.0)),
                                  float(co.get("Fc", 0.6)), float(co.get("N", 1.0))]))
        elif t == "CMAQ_H2O2":
            rate.append(("CMAQ_H2O2", [scale(float(co.get("k1_A", 1.0))), float(co.get("k1_B", 0.0)),
                                       float(co.get("k1_C", 0.0)), scale(float(co.get("k2_A", 1.0))) * 1e6,
                                       float(co.get("k2_B", 0.0)), float(co.get("k2_C", 0.0))]))
        else:
            rate.append((t, []))
    emis = np.zeros(len(allnames))
    for src in root.get("sources") or []:
        if src.get("type") == "EMISSION":
            emis[index[src["species"]]] += float(src["coefficients"]["emission_rate"])
    nfound = np.array([len(pi) for pi in prod_info], dtype=np.int32)  # products naming a known species
    return {"names": allnames, "n_active": len(names), "n_const": len(const), "nreac": nreac, "nprod": nprod,
            "nprod_found": nfound,
            "S": S, "sidx": sidx, "nuki": nuki, "conv_exp": conv_exp, "rate": rate, "emis": emis,
            "M_index": index["M"]}


# ---- rate constants and net production rates ------------------------------------------------------

def kforward(tb: dict, T: float, p: float) -> np.ndarray:
    """Rate constants in the reference's units (k * conv^convExponent, conv = CONV_PPM p / T)."""
    conv = CONV_PPM * p / T
    out = np.zeros(len(tb["rate"]))
    for r, (t, P) in enumerate(tb["rate"]):
        cp = conv ** int(tb["conv_exp"][r])
        if t == "ARRHENIUS":
            A, B, C, D, E = P
            out[r] = A * math.exp(C / T) * (1.0 if B == 0.0 else (T / D) ** B) * (1.0 if E == 0.0 else 1.0 + E * p) * cp
        elif t == "TROE":
            k0A, k0B, k0C, kiA, kiB, kiC, Fc, N = P
            k0 = k0A * (1.0 if k0C == 0.0 else math.exp(k0C / T)) * (1.0 if k0B == 0.0 else (T / 300.0) ** k0B) * conv
            kinf = kiA * (1.0 if kiC == 0.0 else math.exp(kiC / T)) * (1.0 if kiB == 0.0 else (T / 300.0) ** kiB)
            ratio = k0 / kinf
            lg = math.log10(ratio) / N
            out[r] = k0 / (1.0 + ratio) * Fc ** (1.0 / (1.0 + lg * lg)) * cp
        elif t == "CMAQ_H2O2":
            A1, B1, C1, A2, B2, C2 = P
            k1 = A1 * math.exp(C1 / T) * (1.0 if B1 == 0.0 else (T / 300.0) ** B1)
            k2 = A2 * math.exp(C2 / T) * (1.0 if B2 == 0.0 else (T / 300.0) ** B2)
            out[r] = (k1 + k2 * conv) * cp
    return out


def net_production(tb: dict, T: float, p: float, x: np.ndarray) -> np.ndarray:
    """omega[k] for the active species: emissions plus sum over reactions of nu_k q_r, with
    q_r = k_r prod over reactants x^|nu| (x over all species, constant ones included)."""
    k = kforward(tb, T, p)
    S = tb["S"]
    omega = tb["emis"].copy()
    for r in range(len(k)):
        q = k[r]
        for c in range(tb["nreac"][r]):
            q *= x[tb["sidx"][r, c]] ** int(round(-tb["nuki"][r, c]))
        for c in range(tb["nreac"][r]):
            omega[tb["sidx"][r, c]] += tb["nuki"][r, c] * q
        for c in range(tb["nprod_found"][r]):
            j = tb["sidx"][r, S // 2 + c]
            omega[j] += tb["nuki"][r, S // 2 + c] * q
    return omega[:tb["n_active"]]
