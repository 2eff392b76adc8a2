"""Net production rates of a scenario batch: the engine's counterpart of the reference's example
driver src/examples/TChem_NetProductionRates.cpp (same options, same run and output).

  python -m tchem_gb.examples.net_production_rates --chemfile=mech.yaml [--inputfile=scenario.yaml]
      [--outputfile=net_production_rates.dat] [--outputfile_times=wall_times.json]
      [--batch_size=N --use_cloned_samples=true] [--verbose=true] [--replicate=N]

The scenario's state, photolysis rates and external forcing are read as the reference reads them
(setScenarioConditions, setScenarioConditionsPhotolysisReactions,
setScenarioConditionsExternalForcing); with one scenario sample, --use_cloned_samples and
--batch_size > 1 clone it, as the reference does. --replicate=N (not in the reference) tiles the
scenario's samples to N rows for throughput runs. The device call runs twice, the second one timed
with CUDA events (the reference's example times its second call too); wall_times.json records it.
With --verbose=true the rates are written in the reference's format: sample 0 as
writeReactionRates when samples are cloned, else the [B][nSpec] matrix as write2DMatrix (the
constant species' columns are 0).
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np


def _bool(s: str) -> bool:
    return str(s).lower() in ("1", "true", "yes", "on")


def parse(argv=None) -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--chemfile", required=True)
    ap.add_argument("--inputfile", default="None")
    ap.add_argument("--outputfile", default="net_production_rates.dat")
    ap.add_argument("--outputfile_times", default="wall_times.json")
    ap.add_argument("--batch_size", type=int, default=1)
    ap.add_argument("--use_cloned_samples", type=_bool, default=False)
    ap.add_argument("--verbose", type=_bool, default=True)
    ap.add_argument("--replicate", type=int, default=0)
    return ap.parse_args(argv)


def reaction_rates_text(values, n: int) -> str:
    return f"## nSpec({n})    Omega({len(values)})\n" + "".join(f"{i}   {v:e}\n" for i, v in enumerate(values))


def matrix_text(mat: np.ndarray) -> str:
    r, c = mat.shape
    return (f"## nRows({r})    ({r})\n## nCols({c})    ({c})\n" +
            "".join("".join(f"{v:e} " for v in row) + "\n" for row in mat))


def main(argv=None) -> int:
    import torch

    from tchem_gb import (KineticModel, set_scenario_conditions, set_scenario_external_forcing,
                          set_scenario_photolysis_rates)
    from tchem_gb.e3sm import NetProductionRates

    a = parse(argv)
    inputfile = a.chemfile if a.inputfile == "None" else a.inputfile
    km = KineticModel.from_file(a.chemfile)
    state = set_scenario_conditions(inputfile, km)
    nfiles = state.shape[0]
    photo = set_scenario_photolysis_rates(inputfile, nfiles)
    ext = set_scenario_external_forcing(inputfile, km, nfiles)
    cloned = nfiles == 1 and a.use_cloned_samples and a.batch_size > 1
    if cloned:
        reps = a.batch_size
    elif a.replicate > 0:
        reps = -(-a.replicate // nfiles)
    else:
        reps = 1
    B = a.batch_size if cloned else (a.replicate if a.replicate > 0 else nfiles)
    state, photo, ext = (np.tile(x, (reps, 1))[:B] for x in (state, photo, ext))
    dev = torch.device("cuda", torch.cuda.current_device())
    d_state = torch.as_tensor(state).to(dev)
    d_photo = torch.as_tensor(photo).to(dev) if photo.shape[1] > 0 else None
    d_ext = torch.as_tensor(ext).to(dev)
    omega = torch.zeros(B, km.n_active, dtype=torch.float64, device=dev)
    NetProductionRates.runDeviceBatch(d_state, d_photo, d_ext, omega, km)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    NetProductionRates.runDeviceBatch(d_state, d_photo, d_ext, omega, km)
    e1.record()
    torch.cuda.synchronize(dev)
    seconds = e0.elapsed_time(e1) * 1e-3
    with open(a.outputfile_times, "w") as f:
        json.dump({"Net Production Rates": {"wall_time": seconds, "wall_time_per_sample": seconds / B,
                                            "number_of_samples": B}}, f, indent=1)
    print(f"net production rates: {B} samples in {seconds * 1e3:.3f} ms ({B / seconds:.4g} samples/s)")
    if a.verbose:
        W = np.zeros((B, km.nSpec))
        W[:, :km.n_active] = omega.cpu().numpy()
        with open(a.outputfile, "w") as f:
            f.write(reaction_rates_text(W[0], km.nReac) if cloned else matrix_text(W))
    return 0


if __name__ == "__main__":
    sys.exit(main())
