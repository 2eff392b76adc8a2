"""One batched time advance of the seeded CB05-shaped workload (or of the larger generated
mechanisms) on the GPU: the benchmark's inputs at any size, in any numerical form, as one
runDeviceBatch call -- a small, self-contained case for profiling a single kernel launch.

  python -m tchem_gb.examples.generated_batch [--samples 4096] [--horizon 600] [--form mixed]
      [--threads-per-sample 0] [--species 51 --reactions 156] [--seed 7] [--repeat 1]

The mechanism is the generator's (51 species / 156 reactions by default: 60 % Arrhenius, 10 %
Troe, 30 % fixed-J photolysis); the states are the benchmark's (T ~ U[260, 310] K,
p ~ U[0.8, 1.05] atm, number densities log-uniform in [1e2, 1e12] cm^-3; samples 0..N-1 of the
seeded 1,048,576-sample batch when --species is 51). Settings: dt_in = dt_min = 1e-10,
dt_max = horizon, atol 1e-12, rtol 1e-6, Newton 1e-18 / 1e-8, at most 20 Newton iterations.
Prints the wall time of each call and the mean work counters.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--samples", type=int, default=4096)
    ap.add_argument("--horizon", type=float, default=600.0)
    ap.add_argument("--form", choices=["plain", "mixed", "simplified"], default="mixed")
    ap.add_argument("--threads-per-sample", dest="tps", type=int, default=0)
    ap.add_argument("--species", type=int, default=51)
    ap.add_argument("--reactions", type=int, default=156)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args(argv)

    import torch

    from tchem_gb import AtmosphericChemistry, KineticModel, tadv_to_device, time_advance_array
    from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states

    spec = MechanismSpec() if (a.species, a.reactions) == (51, 156) else \
        MechanismSpec(n_species=a.species, n_reactions=a.reactions, seed=20251205)
    km = KineticModel.from_string(mechanism_yaml(spec))
    m = km.n_active
    if (a.species, a.reactions) == (51, 156) and a.samples <= (1 << 20):
        state = sample_states(1 << 20, m, seed=a.seed)[:a.samples]
    else:
        state = sample_states(a.samples, m, seed=a.seed)
    tadv = time_advance_array(a.samples, tend=a.horizon, dt=1e-10, dtmin=1e-10, dtmax=a.horizon,
                              max_num_newton_iterations=20, num_time_iterations_per_interval=10_000_000)
    dev = torch.device("cuda")
    d_tn = torch.tensor([1e-18, 1e-8], dtype=torch.float64, device=dev)
    d_tt = torch.as_tensor(np.tile([1e-12, 1e-6], (m, 1))).to(dev)
    d_tadv = tadv_to_device(tadv, dev)
    d_state = torch.as_tensor(state).to(dev)
    out = torch.empty_like(d_state)
    t = torch.zeros(a.samples, dtype=torch.float64, device=dev)
    dt = torch.zeros_like(t)
    stats = torch.zeros(a.samples, 8, dtype=torch.int32, device=dev)
    for r in range(a.repeat):
        t.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = AtmosphericChemistry.runDeviceBatch(d_tn, d_tt, None, d_tadv, d_state, t, dt, out, km, stats=stats,
                                                 form=a.form, threads_per_sample=a.tps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        bad = int((st != 0).sum())
        print(f"call {r}: {a.samples} samples, {m} species, {a.horizon} s, form {a.form}: {el * 1e3:.1f} ms, "
              f"{a.samples / el:.1f} samples/s, failed {bad}", flush=True)
        if bad:
            return 1
    s = stats.cpu().numpy().astype(np.float64).mean(axis=0)
    names = ["steps", "rejected", "newton_fail", "newton_iter", "factorizations", "solves", "rhs", "jacobians"]
    print("mean work per sample: " + ", ".join(f"{n} {v:.1f}" for n, v in zip(names, s)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
