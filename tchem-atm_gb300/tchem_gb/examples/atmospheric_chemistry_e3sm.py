"""E3SM gas-chemistry time advance of a scenario: the engine's counterpart of the reference's
example driver src/examples/TChem_AtmosphericChemistryE3SM.cpp (same options, host time loop and
output file).

  python -m tchem_gb.examples.atmospheric_chemistry_e3sm --chemfile=mech.yaml [--inputfile=scenario.yaml]
      [options of tchem_gb.examples.atmospheric_chemistry] [--atol-time=1e-12]

The scenario state, photolysis rates and external forcing are read from --inputfile (default: the
chemfile), as the reference does (setScenarioConditions, setScenarioConditionsPhotolysisReactions,
setScenarioConditionsExternalForcing); cloned samples clone all three. The host loop and the
output rows are those of the box-model example; the batch advance is
AtmosphericChemistryE3SM.runHostBatch.
"""
from __future__ import annotations

import sys

import numpy as np

from .atmospheric_chemistry import base_parser, clone, run


def main(argv=None, make_advance=None) -> int:
    """make_advance(km, tol_newton, tol_time, photo_rates, external_sources) -> advance(tadv, state,
    t) -> (state, t, dt) replaces the engine's batch advance when given (the tests drive this loop
    with the CPU oracle)."""
    from tchem_gb import (KineticModel, set_scenario_conditions, set_scenario_external_forcing,
                          set_scenario_photolysis_rates)
    from tchem_gb.e3sm import AtmosphericChemistryE3SM

    ap = base_parser(__doc__)
    ap.add_argument("--inputfile", default="None")
    ap.add_argument("--atol-time", dest="atol_time", type=float, default=1e-12)
    ap.set_defaults(outputfile="AtmosphericChemistryE3SM.dat")
    a = ap.parse_args(argv)
    inputfile = a.chemfile if a.inputfile == "None" else a.inputfile
    km = KineticModel.from_file(a.chemfile)
    state = set_scenario_conditions(inputfile, km)
    nfiles = state.shape[0]
    photo = set_scenario_photolysis_rates(inputfile, nfiles)
    ext = set_scenario_external_forcing(inputfile, km, nfiles)
    state, photo, ext = clone(a, state, photo, ext)
    tol_newton = np.array([a.atol_newton, a.rtol_newton])
    tol_time = np.tile([a.atol_time, a.tol_time], (km.n_active, 1))
    photo_in = photo if photo.shape[1] > 0 else None
    if make_advance is None:
        def advance(tadv, state_, t_):
            out, t2, dt2, _ = AtmosphericChemistryE3SM.runHostBatch(tol_newton, tol_time, tadv, state_, photo_in, ext,
                                                                    t_, km, form=a.form)
            return out, t2, dt2
    else:
        advance = make_advance(km, tol_newton, tol_time, photo_in, ext)
    return run(a, km, state, advance)


if __name__ == "__main__":
    sys.exit(main())
