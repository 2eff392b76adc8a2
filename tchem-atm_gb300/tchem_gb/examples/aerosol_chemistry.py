"""Gas-aerosol (SIMPOL.1 phase transfer) time advance of a scenario: the engine's counterpart of
the reference's example driver src/examples/TChem_AerosolChemistry.cpp (same options, host time
loop and output file).

  python -m tchem_gb.examples.aerosol_chemistry --chemfile=config_gas.yaml --aerofile=aero.yaml
      [--inputfile=... --inputfile_particles=... --number_of_particles=N --outputfile=...]
      [--tbeg=0 --tend=1 --dtmin=1e-8 --dtmax=0.1 --tol-time=1e-4 --atol-time=1e-12
       --atol-newton=1e-10 --rtol-newton=1e-6 --time-iterations-per-interval=10
       --max-time-iterations=1000 --max-newton-iterations=100 --jacobian-interval=1]
      [--batch_size=N --use_cloned_samples=true] [--write-time-profiles=true]

The gas scenario is read from --inputfile (default: the chemfile) and the particles (number
concentrations and aerosol masses) from --inputfile_particles (default: the chemfile); one
scenario sample with --use_cloned_samples and --batch_size > 1 is cloned. The host loop calls
AerosolChemistry.runHostBatch (one call per interval of --time-iterations-per-interval steps)
until the mean time reaches 0.9999 tend or --max-time-iterations calls, carrying t and dt into
the next call (src/examples/TChem_AerosolChemistry.cpp:372-419), and writes every sample's row
after every call: "iter t dt rho p T gas species... particle species..." in %15.10e, the columns
of particle i named <species>_p<i>, the first row (iter -1) holding the initial state with
t = dt = 0 (src/examples/TChem_AerosolChemistry.cpp:332-370). The engine runs the plain FP64 form.
"""
from __future__ import annotations

import sys

import numpy as np

from .atmospheric_chemistry import base_parser, run


def parser():
    ap = base_parser(__doc__)
    ap.set_defaults(outputfile="AerosolChemistry.dat")
    ap.add_argument("--aerofile", required=True)
    ap.add_argument("--inputfile", default="None")
    ap.add_argument("--inputfile_particles", default="None")
    ap.add_argument("--number_of_particles", type=int, default=-1)
    ap.add_argument("--atol-time", dest="atol_time", type=float, default=1e-12)
    ap.add_argument("--team_thread_size", type=int, default=-1)
    ap.add_argument("--vector_thread_size", type=int, default=-1)
    return ap


def main(argv=None, make_advance=None) -> int:
    """make_advance(km, am, tol_newton, tol_time, number_conc) -> advance(tadv, state, t) ->
    (state, t, dt) replaces the engine's batch advance when given (the tests drive this loop with
    the CPU oracle)."""
    from tchem_gb import KineticModel
    from tchem_gb.aerosol import AerosolChemistry, AerosolModel

    a = parser().parse_args(argv)
    if a.form != "plain":
        raise SystemExit("the gas-aerosol advance runs the plain FP64 form")
    inputfile = a.chemfile if a.inputfile == "None" else a.inputfile
    particles = a.chemfile if a.inputfile_particles == "None" else a.inputfile_particles
    km = KineticModel.from_file(a.chemfile)
    am = AerosolModel.from_file(a.aerofile, km)
    if a.number_of_particles > 0:
        am.set_number_of_particles(a.number_of_particles)
    state, nc = am.scenario(inputfile, particles)
    if state.shape[0] == 1 and a.use_cloned_samples and a.batch_size > 1:
        state, nc = np.tile(state, (a.batch_size, 1)), np.tile(nc, (a.batch_size, 1))
    tol_newton = np.array([a.atol_newton, a.rtol_newton])
    tol_time = np.tile([a.atol_time, a.tol_time], (am.n_ode, 1))
    if make_advance is None:
        def advance(tadv, state_, t_):
            out, t2, dt2, status = AerosolChemistry.runHostBatch(tol_newton, tol_time, tadv, state_, nc, t_, km, am)
            return out, t2, dt2
    else:
        advance = make_advance(km, am, tol_newton, tol_time, nc)
    names = list(km.species_names) + [f"{s}_p{ip}" for ip in range(am.nParticles) for s in am.species_names]
    # the reference example writes its freshly made host time views (zeros) in the iter -1 row
    return run(a, km, state, advance, names=names, initial_row_times=(0.0, 0.0))


if __name__ == "__main__":
    sys.exit(main())
