"""Box-model time advance of a scenario: the engine's counterpart of the reference's example driver
src/examples/TChem_AtmosphericChemistry.cpp (same options, host time loop and output file).

  python -m tchem_gb.examples.atmospheric_chemistry --chemfile=mech.yaml [--outputfile=...]
      [--tbeg=0 --tend=1 --dtmin=1e-8 --dtmax=0.1 --tol-time=1e-4 --atol-newton=1e-10
       --rtol-newton=1e-6 --time-iterations-per-interval=10 --max-time-iterations=1000
       --max-newton-iterations=100 --jacobian-interval=1] [--batch_size=N --use_cloned_samples=true]
      [--write-time-profiles=true] [--form=plain|mixed|simplified]

The scenario (state rows [rho, p, T, species]) is read from the chemfile, as the reference does;
one scenario sample with --use_cloned_samples and --batch_size > 1 is cloned. The host loop calls
the batch advance (runHostBatch, one call per interval of --time-iterations-per-interval steps)
until the mean time reaches 0.9999 tend or --max-time-iterations calls, carrying t and dt into
the next call (src/examples/TChem_AtmosphericChemistry.cpp:312-352), and writes every sample's row
after every call: "iter t dt rho p T species..." in %15.10e, the first row (iter -1) holding the
initial state with dt = dtmax. --form (not in the reference) selects the engine's numerical form.
The step-time tolerance atol is 1e-12, as the reference fixes it.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def _bool(s: str) -> bool:
    return str(s).lower() in ("1", "true", "yes", "on")


def header_line(species_names) -> str:
    """The reference's header: iter, t, dt, Density[kg/m3], Pressure[Pascal], Temperature[K],
    species names, tab separated."""
    return ("iter \t t \t dt \t Density[kg/m3] \t Pressure[Pascal] \t Temperature[K] \t" +
            "".join(f"{n} \t" for n in species_names) + "\n")


def state_lines(it: int, t, dt, state) -> str:
    """One row per sample as the reference's writeState: iter, t, dt, state, %15.10e."""
    return "".join(f"{it} \t {t[s]:15.10e} \t  {dt[s]:15.10e} \t " + "".join(f"{v:15.10e} \t" for v in state[s]) + "\n"
                   for s in range(state.shape[0]))


def host_loop(advance, tadv, state, t, dt, tend: float, max_iterations: int, write=None):
    """Calls advance(tadv, state, t) -> (state, t, dt) until the mean t exceeds 0.9999 tend or
    max_iterations calls, carrying t and dt into tadv; write(iter, t, dt, state) after each call.
    Returns (state, t, dt, calls)."""
    it, tsum = 0, 0.0
    while it < max_iterations and tsum <= tend * 0.9999:
        state, t, dt = advance(tadv, state, t)
        if write is not None:
            write(it, t, dt, state)
        tadv["tbeg"] = t
        tadv["dt"] = dt
        tsum = float(np.mean(t))
        it += 1
    return state, t, dt, it


def base_parser(doc: str) -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(description=doc, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--chemfile", required=True)
    ap.add_argument("--outputfile", default="AtmosphericChemistry.dat")
    ap.add_argument("--outputfile_times", default="wall_times.json")
    ap.add_argument("--tbeg", type=float, default=0.0)
    ap.add_argument("--tend", type=float, default=1.0)
    ap.add_argument("--dtmin", type=float, default=1e-8)
    ap.add_argument("--dtmax", type=float, default=1e-1)
    ap.add_argument("--tol-time", dest="tol_time", type=float, default=1e-4)
    ap.add_argument("--atol-newton", dest="atol_newton", type=float, default=1e-10)
    ap.add_argument("--rtol-newton", dest="rtol_newton", type=float, default=1e-6)
    ap.add_argument("--time-iterations-per-interval", dest="iters_per_interval", type=int, default=10)
    ap.add_argument("--max-time-iterations", dest="max_time_iterations", type=int, default=1000)
    ap.add_argument("--max-newton-iterations", dest="max_newton", type=int, default=100)
    ap.add_argument("--jacobian-interval", dest="jacobian_interval", type=int, default=1)
    ap.add_argument("--batch_size", type=int, default=1)
    ap.add_argument("--use_cloned_samples", type=_bool, default=False)
    ap.add_argument("--write-time-profiles", dest="write_time_profiles", type=_bool, default=True)
    ap.add_argument("--verbose", type=_bool, default=False)
    ap.add_argument("--form", default="plain", choices=["plain", "mixed", "simplified"])
    return ap


def make_tadv(a, B: int):
    from tchem_gb import time_advance_array
    return time_advance_array(B, tbeg=a.tbeg, tend=a.tend, dt=a.dtmin, dtmin=a.dtmin, dtmax=a.dtmax,
                              max_num_newton_iterations=a.max_newton,
                              num_time_iterations_per_interval=a.iters_per_interval,
                              jacobian_interval=a.jacobian_interval)


def clone(a, *arrays):
    """The reference's --use_cloned_samples: one scenario sample cloned to --batch_size rows."""
    if arrays[0].shape[0] == 1 and a.use_cloned_samples and a.batch_size > 1:
        return tuple(np.tile(x, (a.batch_size, 1)) for x in arrays)
    return arrays


def run(a, km, state, advance, names=None, initial_row_times=None) -> int:
    """The example's main loop and output for a parsed argument set (shared with the E3SM and
    aerosol examples); names: the output columns after T (default: the gas species);
    initial_row_times: (t, dt) written in the iter -1 row (default: tbeg and dtmax)."""
    B = state.shape[0]
    tadv = make_tadv(a, B)
    t = np.full(B, a.tbeg)
    dt = np.full(B, a.dtmax)
    walls = {}
    f = open(a.outputfile, "w") if a.write_time_profiles else None
    try:
        if f:
            f.write(header_line(km.species_names if names is None else names))
            t0, dt0 = (t, dt) if initial_row_times is None else (np.full(B, initial_row_times[0]),
                                                                 np.full(B, initial_row_times[1]))
            f.write(state_lines(-1, t0, dt0, state))
        clock = [time.perf_counter()]

        def write(it, t_, dt_, state_):
            now = time.perf_counter()
            walls[f"wall_time_iter_{it}"] = now - clock[0]
            if f:
                f.write(state_lines(it, t_, dt_, state_))
            clock[0] = time.perf_counter()

        state, t, dt, calls = host_loop(advance, tadv, state, t, dt, a.tend, a.max_time_iterations, write)
    finally:
        if f:
            f.close()
    walls["number_of_time_iters"] = calls
    walls["number_of_samples"] = B
    with open(a.outputfile_times, "w") as g:
        json.dump(walls, g, indent=1)
    return 0


def main(argv=None, make_advance=None) -> int:
    """make_advance(km, tol_newton, tol_time) -> advance(tadv, state, t) -> (state, t, dt) replaces
    the engine's batch advance when given (the tests drive this loop with the CPU oracle)."""
    from tchem_gb import AtmosphericChemistry, KineticModel, set_scenario_conditions

    a = base_parser(__doc__).parse_args(argv)
    km = KineticModel.from_file(a.chemfile)
    (state,) = clone(a, set_scenario_conditions(a.chemfile, km))
    tol_newton = np.array([a.atol_newton, a.rtol_newton])
    tol_time = np.tile([1e-12, a.tol_time], (km.n_active, 1))
    if make_advance is None:
        def advance(tadv, state_, t_):
            out, t2, dt2, _, _ = AtmosphericChemistry.runHostBatch(tol_newton, tol_time, tadv, state_, t_, km,
                                                                   form=a.form)
            return out, t2, dt2
    else:
        advance = make_advance(km, tol_newton, tol_time)
    return run(a, km, state, advance)


if __name__ == "__main__":
    sys.exit(main())
