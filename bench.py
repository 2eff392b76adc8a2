#!/usr/bin/env python3
"""Benchmark of the batched box-model TR-BDF2 time advance (TChem::AtmosphericChemistry::runDeviceBatch).

Workload: the CB05-shaped batch -- 51 active species, one constant species, 156 reactions (60 %
Arrhenius, 10 % Troe, 30 % fixed-J photolysis), seeded -- advanced from t = 0 to the 3600 s horizon
with adaptive TR-BDF2 steps (dt_in = dt_min = 1e-10, dt_max = 3600, atol 1e-12, rtol 1e-6, Newton
1e-18 / 1e-8, at most 20 Newton iterations). 1,048,576 samples per GPU with T ~ U[260, 310] K,
p ~ U[0.8, 1.05] atm and number densities log-uniform in [1e2, 1e12] cm^-3 (synthetic, seeded). The
state array (1,048,576 x 55 doubles, 461 MB) is larger than L2, so no flush is needed between steps.

The timed loop is the reference's host time loop (src/examples/TChem_AtmosphericChemistry.cpp:312-352):
every "step" is one runDeviceBatch call over the whole batch followed by the carry-over of t and dt
into the time-advance records (one device kernel, tchem_gb_time_advance_carry_over). Each call
advances every sample by at most S steps (num_time_iterations_per_interval; S = the probe's mean step
count / K), the last of the K calls without that limit, so the K timed steps take every sample from
t = 0 to the horizon. The W warm-up steps run the same calls on a separate copy of the batch.

Metric: box-samples/s = samples advanced to the horizon per second (whole job, all ranks).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--form simplified]

--impl engine (default) times the chosen form through the device API (value); the same K calls through
the host-buffer C ABI with the host<->device copies of every call inside the timed region (e2e); the
plain FP64 form and the other mixed form on subsamples, with the chosen form's end-state error against
the plain FP64 results; the CPU oracle on a bounded subsample (cpu_baseline, and the error against the
FP64 oracle); and the side legs: the uneven batch in one graph launch, the discrete adjoint, the
E3SM scenario, the gas-aerosol driver case and the 300-species mechanism.
--impl reference times the reference algorithm's CPU restatement (the oracle, FP64, OpenMP on all
host threads) on a bounded subsample per step; the reference's own Kokkos build cannot be built
here (Kokkos, Tines, Sacado and yaml-cpp are absent).
Under torchrun each rank advances its own batch (samples are independent: weak scaling, no
collective on the data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "tchem-atm_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

from tchem_gb import _capi  # noqa: E402
from tchem_gb.generator import MechanismSpec, mechanism_yaml, sample_states  # noqa: E402
from tchem_gb.mechanism import KineticModel  # noqa: E402

T_START = time.perf_counter()
METRIC = "box-samples/s"
HORIZON = 3600.0
TOL_NEWTON = (1e-18, 1e-8)
ATOL, RTOL = 1e-12, 1e-6
SEED = 7
UNCAPPED = 10_000_000  # step budget of a call that runs every sample to its horizon
# Form names of the C ABI's tchem_gb_form.
FORM_DTYPE = {"plain": "f64", "mixed": "f64 state / f32 Gauss-Jordan inverse or LU + f64-residual refinement",
              "simplified": "f64 state / f32 Gauss-Jordan inverse"}
# DRAM bytes per sample of the time-advance kernel, from one ncu capture of a 4096-sample case of
# the same kernel (dram__bytes_read.sum + dram__bytes_write.sum over the launch, divided by the
# samples). The per-sample traffic (state, time-advance record and times read once, results written
# once) does not depend on the horizon or on the batch size, so it scales by samples.
NCU_DRAM_BYTES_PER_SAMPLE = {"mixed": 820480 / 1216}  # 1,216-sample capture of the two-warp Gauss-Jordan kernel


def parse() -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed runDeviceBatch calls that take the batch to the horizon")
    ap.add_argument("--warmup", type=int, default=5, help="untimed calls on a separate copy of the batch")
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--form", choices=["simplified", "mixed", "plain"], default="mixed",
                    help="mixed (default): full Newton with an FP32 Gauss-Jordan inverse or LU and FP64-residual "
                         "refinement; simplified: simplified Newton on a carried FP32 inverse; plain: FP64 LU")
    ap.add_argument("--samples", type=int, default=1 << 20, help="samples per GPU (the workload is 1,048,576)")
    ap.add_argument("--plain-samples", type=int, default=16384, help="subsample for the plain FP64 form")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU time of one oracle sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--other-samples", type=int, default=65536,
                    help="subsample for the other mixed form (mixed <-> simplified)")
    ap.add_argument("--uneven-samples", type=int, default=262144,
                    help="samples of the uneven-batch leg (262144 in the reference's uneven configuration): 75 %% on "
                         "the 51-species and 25 %% on a 120-species mechanism, half night, horizons 600/1800/3600 s, "
                         "autotuned shapes, one CUDA-graph launch; 0 skips it")
    ap.add_argument("--adjoint-samples", type=int, default=65536,
                    help="samples of the discrete-adjoint leg (1800 s horizon, FP64); 0 skips it")
    ap.add_argument("--e3sm-samples", type=int, default=65536,
                    help="samples of the E3SM leg (the reference's 80-column uci scenario tiled); 0 skips it")
    ap.add_argument("--large-samples", type=int, default=1216,
                    help="samples of the 300-species / 1000-reaction leg in the tensor-core form (with the plain "
                         "FP64 form beside it on 152 samples over 0.1 s); 0 skips it")
    ap.add_argument("--large-horizon", type=float, default=10.0, help="horizon of the 300-species leg (s)")
    ap.add_argument("--tc-lu-matrices", type=int, default=0,
                    help="matrices of the tensor-core LU leg (300 x 300 FP32, TF32 trailing updates on tcgen05): "
                         "factorizations/s and the TF32 rate of the trailing updates; 0 skips it")
    ap.add_argument("--leg-budget-s", type=float, default=1150.0,
                    help="side legs start only while the run's wall time is below this (seconds)")
    ap.add_argument("--aerosol-samples", type=int, default=8192,
                    help="samples of the gas-aerosol (SIMPOL.1) leg: the reference driver test's CB05CL_AE5 + SOA "
                         "sample perturbed, one 30 s driver time step (83 ODEs, plain FP64); 0 skips it")
    return ap.parse_args()


# ---- workload ---------------------------------------------------------------------------------

def workload(B: int, rank: int):
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec()))
    m = km.n_active
    state = sample_states(B, m, seed=SEED + rank)
    tadv = np.zeros(B, dtype=_capi.TIME_ADVANCE_DTYPE)
    tadv["tbeg"], tadv["tend"], tadv["dt"], tadv["dtmin"], tadv["dtmax"] = 0.0, HORIZON, 1e-10, 1e-10, HORIZON
    tadv["max_num_newton_iterations"] = 20
    tadv["num_time_iterations_per_interval"] = 1_000_000
    tadv["jacobian_interval"] = 1
    tol_time = np.tile([ATOL, RTOL], (m, 1))
    return km, state, tadv, tol_time


def flops_per_call(km) -> tuple[float, float, float]:
    """Algorithmic flops of one RHS, one analytic Jacobian and one factorization (m^3 * 2/3)."""
    v = km.view
    R, S = v.nReac, v.maxSpecInReac
    nr = np.ctypeslib.as_array(v.reacNreac, (R,))
    npd = np.ctypeslib.as_array(v.reacNprod, (R,))
    nu = np.ctypeslib.as_array(v.reacNuki, (R * S,)).reshape(R, S)
    nu_reac = np.array([np.abs(nu[r, :nr[r]]).sum() for r in range(R)])
    f_rhs = float(np.sum(2 * nu_reac + 2 * (nr + npd)))
    f_jac = float(np.sum(nr * (2 * nr + 2 * (nr + npd))))
    m = km.n_active
    return f_rhs, f_jac, 2.0 / 3.0 * m ** 3


def work_flops(km, stats: np.ndarray) -> tuple[float, float]:
    """(FP32-side, FP64-side) algorithmic flops of a run from its per-sample counters: LU and
    solves and Jacobians are the linear-algebra side, RHS evaluations the FP64 side."""
    f_rhs, f_jac, f_lu = flops_per_call(km)
    m = km.n_active
    s = stats.astype(np.float64)
    f32 = s[:, 4].sum() * f_lu + s[:, 5].sum() * 2 * m * m + s[:, 7].sum() * f_jac
    f64 = s[:, 6].sum() * f_rhs
    return f32, f64


# ---- clocks -----------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=10)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        return False

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- distributed helpers ----------------------------------------------------------------------

def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        # one GPU per rank over NCCL; gloo where there is no GPU (the CPU-only reference arm)
        dist.init_process_group(backend="nccl" if n_gpus > 0 and torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- CPU legs (the oracle: accuracy reference and CPU restatement) ------------------------------

def cpu_sample_size(km, state, tadv, tol_time, seconds: float) -> tuple[int, float]:
    """Samples of the CPU oracle that take about `seconds` on all host threads."""
    from oracle import Oracle
    o = Oracle([km], native=True)
    n0 = max(2 * (os.cpu_count() or 1), 16)
    t0 = time.perf_counter()
    o.time_advance(tadv[:n0], state[:n0], TOL_NEWTON, tol_time)
    rate = n0 / (time.perf_counter() - t0)
    n = int(max(n0, min(len(state), rate * seconds)))
    return n, rate


def run_oracle(km, state, tadv, tol_time, n: int):
    from oracle import Oracle
    t0 = time.perf_counter()
    res = Oracle([km], native=True).time_advance(tadv[:n], state[:n], TOL_NEWTON, tol_time)
    return res, time.perf_counter() - t0


def bench_config(B: int, form: str, world: int) -> dict:
    """The workload description shared by both arms."""
    return {"workload": f"cb05-shaped 51 species / 156 reactions, {B} samples per GPU, 0 -> 3600 s TR-BDF2",
            "samples_per_gpu": B, "horizon_s": HORIZON, "form": form, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (461 MB state per GPU); no flush"}


def rel_err(test: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """Per-sample max over species of |test - ref| / max(|ref|, atol)."""
    return (np.abs(test - ref) / np.maximum(np.abs(ref), ATOL)).max(axis=1)


# ---- reference arm ----------------------------------------------------------------------------

def reference_arm(args, world: int, rank: int):
    if rank != 0:
        return  # one CPU measurement per node; the other ranks have no work
    km, state, tadv, tol_time = workload(max(args.samples, 1), 0)
    n, _ = cpu_sample_size(km, state, tadv, tol_time, args.cpu_seconds)
    for _ in range(args.warmup):
        run_oracle(km, state, tadv, tol_time, n)
    total = 0.0
    for _ in range(args.steps):
        _, el = run_oracle(km, state, tadv, tol_time, n)
        total += el
    value = n * args.steps / total
    cores = os.cpu_count() or 1
    sample = (f"first {n} of the {args.samples}-sample CB05-shaped batch per step (FP64 TR-BDF2 CPU restatement built for the host CPU, "
              f"OpenMP dynamic over samples on {cores} threads); samples are independent, so box-samples/s "
              f"of the full batch equals this rate")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.samples, args.form, world),
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Kokkos/Tines build is unavailable here (submodules absent, no network); the "
                "oracle restatement of its algorithm is timed instead",
    }
    print(json.dumps(line), flush=True)


# ---- uneven batch -------------------------------------------------------------------------------

def uneven_leg(B: int, form: str, dev, stream) -> dict:
    """Mixed mechanism sizes, day/night variants and three horizons in one graph-captured launch,
    in the chosen form; end states of a stratified subsample against the plain FP64 form."""
    import torch
    from tchem_gb import AtmosphericChemistry, tadv_to_device
    spec120 = MechanismSpec(n_species=120, n_reactions=330, seed=20251204)
    mechs = [KineticModel.from_string(mechanism_yaml(MechanismSpec())),
             KineticModel.from_string(mechanism_yaml(MechanismSpec(), night=True)),
             KineticModel.from_string(mechanism_yaml(spec120)),
             KineticModel.from_string(mechanism_yaml(spec120, night=True))]
    rng = np.random.default_rng(20251205)
    big = rng.random(B) < 0.25
    night = rng.random(B) < 0.5
    mos = (2 * big + night).astype(np.int32)
    dim = mechs[2].state_dim
    state = np.zeros((B, dim))
    s51 = sample_states(B, mechs[0].n_active, seed=SEED + 11)
    s120 = sample_states(B, mechs[2].n_active, seed=SEED + 12)
    state[:, :s51.shape[1]] = s51
    state[big] = s120[big]
    horizon = rng.choice([600.0, 1800.0, 3600.0], size=B)
    tadv = np.zeros(B, dtype=_capi.TIME_ADVANCE_DTYPE)
    tadv["tbeg"], tadv["tend"], tadv["dt"], tadv["dtmin"], tadv["dtmax"] = 0.0, horizon, 1e-10, 1e-10, horizon
    tadv["max_num_newton_iterations"] = 20
    tadv["num_time_iterations_per_interval"] = 1_000_000
    tadv["jacobian_interval"] = 1
    tol_time = np.tile([ATOL, RTOL], (mechs[2].n_active, 1))
    d_tn = torch.tensor(TOL_NEWTON, dtype=torch.float64, device=dev)
    d_tt = torch.as_tensor(tol_time).to(dev)
    tuned = {}
    for k in (0, 2):  # autotune each structure on a probe of its own samples
        sel = np.nonzero(mos == k)[0][:2048]
        km = mechs[k]
        tps, times = AtmosphericChemistry.autotune(km, d_tn, d_tt[:km.n_active], tadv_to_device(tadv[sel], dev),
                                                   torch.as_tensor(state[sel][:, :km.state_dim]).to(dev),
                                                   form=form, stream=stream)
        AtmosphericChemistry.set_threads_per_sample(mechs[k + 1], tps, form=form)
        tuned[f"{km.n_active}_species"] = {"threads_per_sample": tps,
                                           "probe_ms": {str(a): round(b, 1) for a, b in times.items()}}
    d_state = torch.as_tensor(state).to(dev)
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device=dev)
    dt = torch.zeros_like(t)
    g, status = AtmosphericChemistry.capture(d_tn, d_tt, tadv_to_device(tadv, dev), d_state, t, dt, out, mechs,
                                             mech_of_sample=torch.as_tensor(mos).to(dev), form=form)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    g.replay()
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    res = out.cpu().numpy()
    # accuracy: 512 samples of each 51-species variant and 16 of each 120-species variant against the
    # plain FP64 form (one call per mechanism; the plain form is slow at 120 species)
    acc = {}
    for k, n in ((0, 512), (1, 512), (2, 16), (3, 16)):
        sel = np.nonzero(mos == k)[0][:n]
        km = mechs[k]
        st = torch.as_tensor(state[sel][:, :km.state_dim]).to(dev)
        po = torch.empty_like(st)
        pt = torch.zeros(len(sel), dtype=torch.float64, device=dev)
        pdt = torch.zeros_like(pt)
        AtmosphericChemistry.runDeviceBatch(d_tn, d_tt[:km.n_active], None, tadv_to_device(tadv[sel], dev), st, pt,
                                            pdt, po, km, form="plain", stream=stream)
        ref = po.cpu().numpy()[:, 3:3 + km.n_active]
        e = rel_err(res[sel][:, 3:3 + km.n_active], ref)
        acc[f"{km.n_active}_species_{'night' if k % 2 else 'day'}"] = {"samples": len(sel), "max": float(e.max()),
                                                                        "p99": float(np.percentile(e, 99))}
    return {"samples": B, "value": B / (ms * 1e-3), "unit": "samples/s", "ms": ms, "form": form,
            "failed_samples": int((status.cpu().numpy() != 0).sum()),
            "mix": {"51_species": int((~big).sum()), "120_species": int(big.sum()), "night": int(night.sum())},
            "launch": "one CUDA graph replay, timed (t reset, bucketing, one persistent kernel per mechanism "
                      "structure, the structures' kernels concurrent on forked streams)",
            "autotuned": tuned, "accuracy_vs_plain_fp64_gpu": acc}


# ---- E3SM gas chemistry -----------------------------------------------------------------------

E3SM_MECH = ROOT / "tests" / "golden" / "mechanisms" / "uci_v2_test3.yaml"
E3SM_SCENARIO = ROOT / "tests" / "golden" / "e3sm" / "uci_col_input_conditions.yaml"
E3SM_GOLDEN = ROOT / "tests" / "golden" / "e3sm" / "uci_col_full_gas.npy"


def e3sm_leg(B: int, cpu_seconds: float, dev, stream) -> dict:
    """The E3SM TR-BDF2 advance (AtmosphericChemistryE3SM::runDeviceBatch) of the reference's
    80-column uci scenario (53 active species, 106 reactions, 22 photolysis rates, external
    forcing) tiled to B samples, with the settings of the reference's E3SM gtest (1800 s, dt_in =
    dt_min = 1e-20, dt_max = 3600, rtol 1e-6, at most 100 steps per call); the NetProductionRates
    kernel on the same rows; the CPU restatement on the host cores; the first 80 end states against
    the reference's golden."""
    import torch
    from oracle import E3smOracle
    from tchem_gb import (set_scenario_conditions, set_scenario_external_forcing, set_scenario_photolysis_rates,
                          tadv_to_device)
    from tchem_gb.e3sm import AtmosphericChemistryE3SM, NetProductionRates
    km = KineticModel.from_file(E3SM_MECH)
    base = set_scenario_conditions(E3SM_SCENARIO, km)
    nc, m = base.shape[0], km.n_active
    rep = -(-B // nc)
    state = np.tile(base, (rep, 1))[:B]
    photo = np.tile(set_scenario_photolysis_rates(E3SM_SCENARIO, nc), (rep, 1))[:B]
    ext = np.tile(set_scenario_external_forcing(E3SM_SCENARIO, km, nc), (rep, 1))[:B]
    tadv = np.zeros(B, dtype=_capi.TIME_ADVANCE_DTYPE)
    tadv["tbeg"], tadv["tend"], tadv["dt"], tadv["dtmin"], tadv["dtmax"] = 0.0, 1800.0, 1e-20, 1e-20, 3600.0
    tadv["max_num_newton_iterations"] = 20
    tadv["num_time_iterations_per_interval"] = 100
    tadv["jacobian_interval"] = 1
    tol_time = np.tile([ATOL, RTOL], (m, 1))
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_state, d_photo, d_ext, d_tadv = d(state), d(photo), d(ext), tadv_to_device(tadv, dev)
    d_tn, d_tt = torch.tensor(TOL_NEWTON, dtype=torch.float64, device=dev), d(tol_time)
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device=dev)
    dt = torch.zeros_like(t)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(fn, reps: int = 3) -> float:
        fn()  # warm-up: tables on the device, kernel attributes, workspace
        best = float("inf")
        for _ in range(reps):
            ev[0].record(stream)
            fn()
            ev[1].record(stream)
            torch.cuda.synchronize(dev)
            best = min(best, ev[0].elapsed_time(ev[1]))
        return best

    forms, results = {}, {}
    for form, tps in (("simplified", 32), ("simplified", 64), ("mixed", 32), ("plain", 0)):
        def run(form=form, tps=tps):
            t.zero_()
            AtmosphericChemistryE3SM.runDeviceBatch(d_tn, d_tt, None, d_tadv, d_state, d_photo, d_ext, t, dt, out, km,
                                                    form=form, threads_per_sample=tps, stream=stream)
        ms = timed(run)
        key = form if form != "simplified" else f"simplified_{tps}"
        forms[key] = {"value": B / (ms * 1e-3), "ms": ms}
        results[key] = out[:nc].cpu().numpy()
    best = max((k for k in forms if k.startswith("simplified")), key=lambda k: forms[k]["value"])
    omega = torch.empty(B, m, dtype=torch.float64, device=dev)
    ms_rates = timed(lambda: NetProductionRates.runDeviceBatch(d_state, d_photo, d_ext, omega, km, stream=stream))
    rate_bytes = B * 8 * (3 + km.nSpec + photo.shape[1] + 2 * m)  # state row, photolysis, sources in; omega out
    golden_rows = np.load(E3SM_GOLDEN)[nc:, 3:]
    golden = golden_rows[:, 3:3 + m]
    acc = {}
    for k, r in results.items():
        y = r[:, 3:3 + m]
        # the reference's file criterion (compareFilesValues) on the rows as written (%15.10e)
        written = np.vectorize(lambda v: float(f"{v:15.10e}"))(r)
        dw = np.abs(written - golden_rows)
        i = np.unravel_index(int(dw.argmax()), dw.shape)
        acc[k] = {"reference_file_criterion": float(dw[i] / abs(golden_rows[i])), "reference_file_bound": 1e-8,
                  "max_tolerance_units": float((np.abs(y - golden) / (ATOL + RTOL * np.abs(golden))).max())}
    # CPU restatement on the host cores (the E3SM leg's own CPU baseline), bounded sample
    o = E3smOracle(km, native=True)
    n = nc
    t0 = time.perf_counter()
    o.time_advance(tadv[:n], state[:n], photo[:n], ext[:n], TOL_NEWTON, tol_time)
    el = time.perf_counter() - t0
    n = int(min(B, max(nc, nc * round(cpu_seconds / max(el, 1e-6)))))
    t0 = time.perf_counter()
    o.time_advance(tadv[:n], state[:n], photo[:n], ext[:n], TOL_NEWTON, tol_time)
    el = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    return {"metric": METRIC, "value": forms[best]["value"], "unit": "samples/s", "form": best, "samples": B,
            "workload": "reference uci_col E3SM scenario (53 active species, 106 reactions, 22 photolysis rates, "
                        "external forcing), 80 columns tiled, 1800 s TR-BDF2",
            "forms": forms,
            "net_production_rates": {"value": B / (ms_rates * 1e-3), "unit": "samples/s", "ms": ms_rates,
                                     "achieved_gbs": rate_bytes / (ms_rates * 1e-3) / 1e9,
                                     "bytes_per_sample": rate_bytes // B, "bound": "fp64",
                                     "profile": "ncu of this kernel on 262,144 samples: FP64 pipe 86.6 % of "
                                                "peak, DRAM 0.2 %"},
            "accuracy_vs_reference_golden": acc,
            "cpu_baseline": {"value": n / el, "unit": "samples/s", "cores": cores, "kind": "port",
                             "sample": f"first {n} samples, E3SM CPU restatement built for the host CPU, OpenMP over "
                                       f"samples on {cores} threads ({el:.2f} s)"}}


# ---- gas-aerosol chemistry (SIMPOL.1) ---------------------------------------------------------

AERO_DIR = ROOT / "tests" / "golden" / "aerosol"
DRIVER_DIR = ROOT / "tests" / "golden" / "driver"


def aerosol_leg(B: int, cpu_seconds: float, dev, stream) -> dict:
    """The gas-aerosol TR-BDF2 advance (AerosolChemistry::runDeviceBatch, plain FP64) on the
    reference driver test's case: CB05CL_AE5 with four SIMPOL SOA transfers and one particle
    (83 ODEs), its state and number concentration perturbed per sample (seeded, x0.5..1.5), one
    30 s time step with its solver settings (tolerances 1e-12 / 1e-6, Newton 1e-6 / 1e-4, first
    step 1e-12); the first 16 end states against the oracle, sample 0 unperturbed against the
    driver test's output, and the oracle on the host cores."""
    import torch
    from oracle import AerosolOracle
    from tchem_gb import tadv_to_device, time_advance_array
    from tchem_gb.aerosol import AerosolChemistry, AerosolModel
    man = json.loads((ROOT / "tests" / "golden" / "manifest.json").read_text())["driver"]
    km = KineticModel.from_file(AERO_DIR / "cb05_soa_config_full_gas.yaml")
    am = AerosolModel.from_file(AERO_DIR / "cb05_soa_mechanism_aero.yaml", km)
    n = _capi.Numerics()
    _capi.check(_capi.lib().tchem_gb_numerics_read(str(DRIVER_DIR / "config_solver.yaml").encode(), C.byref(n)),
                "tchem_gb_numerics_read")
    st0 = np.zeros(am.state_dim)
    for k, v in man["state"].items():
        st0[int(k)] = v
    st0[3 + km.nSpec] = man["particles"]["first_species"]
    rng = np.random.default_rng(11)
    state = np.tile(st0, (B, 1))
    state[1:, 3:] *= rng.uniform(0.5, 1.5, (B - 1, am.state_dim - 3))
    nc = np.full((B, am.nParticles), man["particles"]["number_conc"])
    nc[1:] *= rng.uniform(0.5, 1.5, (B - 1, 1))
    del_t = man["del_t"]
    tadv = time_advance_array(B, tend=del_t, dt=n.dtmin, dtmin=n.dtmin, dtmax=del_t,
                              max_num_newton_iterations=n.max_newton_iterations,
                              num_time_iterations_per_interval=n.max_num_time_iterations)
    tol_newton = [n.atol_newton, n.rtol_newton]
    tol_time = np.tile([n.atol_time, n.rtol_time], (am.n_ode, 1))
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    d_state, d_nc, d_tadv = d(state), d(nc), tadv_to_device(tadv, dev)
    d_tn, d_tt = d(tol_newton), d(tol_time)
    out = torch.empty_like(d_state)
    t = torch.zeros(B, dtype=torch.float64, device=dev)
    dt = torch.zeros_like(t)
    stats = torch.zeros(B * 8, dtype=torch.int32, device=dev)
    ws = torch.zeros(AerosolChemistry.getWorkSpaceSize(km, am, B), dtype=torch.uint8, device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def run():
        t.zero_()
        return AerosolChemistry.runDeviceBatch(d_tn, d_tt, None, d_tadv, d_state, d_nc, t, dt, out, km, am,
                                               stats=stats, workspace=ws, stream=stream)
    run()
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(3):
        ev[0].record(stream)
        status = run()
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        best = min(best, ev[0].elapsed_time(ev[1]))
    res = out.cpu().numpy()
    st = np.frombuffer(stats.cpu().numpy().tobytes(), dtype=_capi.SAMPLE_STATS_DTYPE)
    K = min(16, B)
    ref, *_ = AerosolOracle(km, am).time_advance(tadv[:K], state[:K], nc[:K], tol_newton, tol_time)
    golden = np.loadtxt(DRIVER_DIR / "output_ref.txt")
    o = AerosolOracle(km, am, native=True)
    m = K
    t0 = time.perf_counter()
    o.time_advance(tadv[:m], state[:m], nc[:m], tol_newton, tol_time)
    el = time.perf_counter() - t0
    m = int(min(B, max(K, K * round(cpu_seconds / max(el, 1e-6)))))
    t0 = time.perf_counter()
    o.time_advance(tadv[:m], state[:m], nc[:m], tol_newton, tol_time)
    el = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    diff = res[:K, 3:] - ref[:, 3:]
    den = np.linalg.norm(ref[:, 3:], axis=0)
    col = np.where(den > 1e-23, np.linalg.norm(diff, axis=0) / np.where(den > 1e-23, den, 1.0), 0.0)
    return {"metric": "box-samples/s (gas-aerosol TR-BDF2, one 30 s driver step)", "value": B / (best * 1e-3),
            "unit": "samples/s", "samples": B, "ms": best, "form": "plain", "dtype": "f64",
            "workload": "reference driver test: CB05CL_AE5 + 4 SIMPOL SOA transfers, 1 particle, 83 ODEs, "
                        "state and number concentration perturbed x0.5..1.5 per sample (seed 11), 30 s",
            "status_ok": int((status.cpu().numpy() == 0).sum()),
            "steps_mean": float(st["n_steps"].mean()), "rhs_mean": float(st["n_rhs"].mean()),
            "accuracy": {"vs_oracle_norm_relative_max": float(col.max()), "oracle_samples": K,
                         "sample0_vs_driver_test_output_isclose": bool(np.all(np.isclose(res[0], golden)))},
            "cpu_baseline": {"value": m / el, "unit": "samples/s", "cores": cores, "kind": "port",
                             "sample": f"first {m} samples, aerosol CPU restatement built for the host CPU, OpenMP "
                                       f"over samples on {cores} threads ({el:.2f} s)"}}


# ---- 300-species mechanism: the tensor-core form ------------------------------------------------

LARGE_SPEC = dict(n_species=300, n_reactions=1000, seed=20251205)


def large_leg(B: int, horizon: float, dev, stream) -> dict:
    """The seeded 300-species / 1000-reaction mechanism (the large dense-LU configuration: same rate
    mix, at most 2 reactants and 4 products) in the tensor-core form (full Newton; FP32 Newton
    matrix, blocked LU with TF32 tcgen05 trailing updates, FP64 refinement), B samples over
    `horizon`; the first 4 end states against the FP64 oracle; and the plain FP64 form beside it on
    152 samples (one sample per SM) over 1e-4 s (49 steps; the plain form's FP64 LU in global memory
    is too slow for longer), with the tensor-core form on the same samples and horizon, for the rate
    ratio."""
    import torch
    from oracle import Oracle
    from tchem_gb import AtmosphericChemistry, tadv_to_device, time_advance_array
    km = KineticModel.from_string(mechanism_yaml(MechanismSpec(**LARGE_SPEC)))
    m = km.n_active
    state = sample_states(B, m, seed=SEED + 21)
    tol_time = np.tile([ATOL, RTOL], (m, 1))
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_tn, d_tt = torch.tensor(TOL_NEWTON, dtype=torch.float64, device=dev), d(tol_time)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def run(form, n, hz):
        tadv = time_advance_array(n, tend=hz, dt=1e-10, dtmin=1e-10, dtmax=hz, max_num_newton_iterations=20,
                                  num_time_iterations_per_interval=10**7)
        d_state = d(state[:n])
        out = torch.empty_like(d_state)
        t = torch.zeros(n, dtype=torch.float64, device=dev)
        dt = torch.zeros_like(t)
        stats = torch.zeros(n, 8, dtype=torch.int32, device=dev)
        ev[0].record(stream)
        st = AtmosphericChemistry.runDeviceBatch(d_tn, d_tt, None, tadv_to_device(tadv, dev), d_state, t, dt, out, km,
                                                 stats=stats, form=form, stream=stream)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        return (ev[0].elapsed_time(ev[1]), out.cpu().numpy(), int((st != 0).sum().item()),
                stats.cpu().numpy().astype(np.float64).mean(axis=0), tadv)

    run("mixed", min(B, 152), 1e-3)  # warm-up: module load, kernel attributes, workspace
    ms, res, bad, work, tadv = run("mixed", B, horizon)
    K = min(4, B)
    ref = Oracle([km], native=True).time_advance(tadv[:K], state[:K], TOL_NEWTON, tol_time)[0]
    err = rel_err(res[:K, 3:3 + m], ref[:, 3:3 + m])
    P = min(152, B)
    ms_tc, *_ = run("mixed", P, 1e-4)
    ms_pl, res_pl, bad_pl, *_ = run("plain", P, 1e-4)
    names = ["steps", "rejected", "newton_fail", "newton_iter", "factorizations", "solves", "rhs", "jacobians"]
    return {"samples": B, "species": m, "reactions": km.nReac, "horizon_s": horizon, "form": "tensor-core full Newton",
            "ms": ms, "value": B / (ms * 1e-3), "unit": "samples/s", "failed_samples": bad,
            "work_per_sample": {k: float(v) for k, v in zip(names, work)},
            "accuracy_vs_fp64_oracle": {"samples": K, "max": float(err.max()), "bound": 1e-6},
            "vs_plain_fp64": {"samples": P, "horizon_s": 1e-4, "tensor_core_ms": ms_tc, "plain_fp64_ms": ms_pl,
                              "speedup": ms_pl / ms_tc, "plain_failed_samples": bad_pl}}


# ---- tensor-core LU (300-species factorization) -----------------------------------------------

def tc_lu_leg(nb: int, dev, stream) -> dict:
    """Batched 300 x 300 FP32 LU with TF32 trailing updates on the tensor cores
    (tchem_gb_tc_lu_factor_tf32, one CTA per matrix), the factorization of the 300-species
    mechanism's Newton matrices: factorizations/s, the trailing-update TF32 flops per second
    (sum over panels of 2 (m - p1)^2 * 32) and the factors against the oracle's restatement on the
    first matrix."""
    import torch
    from oracle import lu_factor_blocked
    from tchem_gb.tensor_core import lu_factor_tf32
    n, lda = 300, 304
    rng = np.random.default_rng(5)
    a = (np.eye(n) - 0.05 * rng.standard_normal((nb, n, n))).astype(np.float32)
    A0 = np.zeros((nb, n, lda), np.float32)
    A0[:, :, :n] = a
    d0 = torch.from_numpy(A0).to(dev)
    dA = d0.clone()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    lu_factor_tf32(dA, stream=stream)
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(3):
        dA.copy_(d0)
        ev[0].record(stream)
        piv, info = lu_factor_tf32(dA, stream=stream)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        best = min(best, ev[0].elapsed_time(ev[1]))
    upd = sum(2.0 * (n - p1) ** 2 * 32 for p1 in range(32, n, 32))
    ref_lu, ref_piv = lu_factor_blocked(a[0], keep=10)
    lu0 = dA[0, :, :n].cpu().numpy()
    return {"matrices": nb, "m": n, "ms": best, "factorizations_per_s": nb / (best * 1e-3),
            "trailing_update_tflops": nb * upd / (best * 1e-3) / 1e12, "info_ok": int((info == 0).sum().item()),
            "vs_oracle": {"pivots_equal": bool(np.array_equal(piv[0].cpu().numpy(), ref_piv)),
                          "max_rel_factor_diff": float(np.abs(lu0 - ref_lu).max() / np.abs(ref_lu).max())}}


# ---- discrete adjoint -------------------------------------------------------------------------

def adjoint_leg(km, state, tol_time, n: int, dev, stream) -> dict:
    """Forward (plain FP64, trajectory recorded) and adjoint times on the first n samples over an
    1800 s horizon; the loss is the sum of squared log-ratios of 5 seeded target species."""
    import torch
    from tchem_gb import tadv_to_device
    from tchem_gb import adjoint as adj
    m = km.n_active
    n = min(n, state.shape[0])
    tadv = np.zeros(n, dtype=_capi.TIME_ADVANCE_DTYPE)
    tadv["tbeg"], tadv["tend"], tadv["dt"], tadv["dtmin"], tadv["dtmax"] = 0.0, 1800.0, 1e-10, 1e-10, 1800.0
    tadv["max_num_newton_iterations"] = 20
    tadv["num_time_iterations_per_interval"] = 1_000_000
    tadv["jacobian_interval"] = 1
    d_tadv = tadv_to_device(tadv, dev)
    d_state = torch.as_tensor(state[:n]).to(dev)
    d_tn = torch.tensor(TOL_NEWTON, dtype=torch.float64, device=dev)
    d_tt = torch.as_tensor(tol_time).to(dev)
    out = torch.empty_like(d_state)
    t = torch.zeros(n, dtype=torch.float64, device=dev)
    dt = torch.zeros_like(t)
    tape = adj.new_tape(n, m, 4096, dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    st = adj.record(km, d_tn, d_tt, d_tadv, d_state, t, dt, out, tape, stream=stream)
    ev[1].record(stream)
    y = out[:, 3:3 + m]
    rng = np.random.default_rng(20251203)
    tg = torch.as_tensor(rng.choice(m, 5, replace=False), device=dev)
    ref = y[:, tg] * torch.exp(torch.as_tensor(rng.normal(0.0, 0.1, size=(n, 5)), device=dev))
    lam = torch.zeros(n, m, dtype=torch.float64, device=dev)
    lam[:, tg] = 2 * torch.log(y[:, tg] / ref) / y[:, tg]
    ev[2].record(stream)
    gx, gk, ast = adj.adjoint(km, d_tn, d_tadv, d_state, tape, lam, stream=stream)
    ev[3].record(stream)
    torch.cuda.synchronize(dev)
    fwd = ev[0].elapsed_time(ev[1])
    bwd = ev[2].elapsed_time(ev[3])
    return {"samples": n, "horizon_s": 1800.0, "dtype": "f64", "checkpoint_every_steps": 32,
            "forward_ms": fwd, "adjoint_ms": bwd, "adjoint_over_forward": bwd / fwd,
            "failed_samples": int((st != 0).sum()) + int((ast != 0).sum()),
            "mean_steps": float(tape.nsteps.double().mean()),
            "gradients": "d loss / d ln A (156) and d loss / d ln x0 (51) per sample"}


# ---- engine arm -------------------------------------------------------------------------------

class HostLoop:
    """The reference's host time loop over one batch on the device: runDeviceBatch calls with the
    carry-over of t and dt between them, each call advancing every sample by the step budget that
    the previous carry-over wrote (caps_for). Arrays are private copies, so the caller's inputs stay
    untouched; the state advances in place (state_out = state), as in the reference's example."""

    def __init__(self, km, form, d_tn, d_tt, tadv: np.ndarray, d_state0, first_cap: int, stats: bool, dev):
        import torch
        from tchem_gb import AtmosphericChemistry, tadv_to_device
        self.AC = AtmosphericChemistry
        self.km, self.form, self.d_tn, self.d_tt = km, form, d_tn, d_tt
        t0 = tadv.copy()
        t0["num_time_iterations_per_interval"] = first_cap
        self.tadv = tadv_to_device(t0, dev)
        self.state = d_state0.clone()
        B = d_state0.shape[0]
        self.t = torch.zeros(B, dtype=torch.float64, device=dev)
        self.dt = torch.zeros_like(self.t)
        self.status = torch.empty(B, dtype=torch.int32, device=dev)
        self.stats = torch.zeros(B, 8, dtype=torch.int32, device=dev) if stats else None
        self.total = torch.zeros(B, 8, dtype=torch.int64, device=dev) if stats else None
        # zeroed: the device error word in the header persists until read, so it must start clear
        self.ws = torch.zeros(AtmosphericChemistry.getWorkSpaceSize(km, B, form=form), dtype=torch.uint8, device=dev)

    def advance(self, stream):
        """One runDeviceBatch call (the time-advance kernel)."""
        self.AC.runDeviceBatch(self.d_tn, self.d_tt, None, self.tadv, self.state, self.t, self.dt, self.state, self.km,
                               status=self.status, stats=self.stats, form=self.form, workspace=self.ws, stream=stream)

    def carry(self, stream, next_cap: int):
        """The carry-over of t and dt, with the next call's step budget."""
        if self.total is not None:
            self.total += self.stats
        self.AC.carry_over(self.tadv, self.t, self.dt, next_cap, stream=stream)


def fma_probe() -> C.CDLL:
    """The FMA-throughput probe library (built by tchem_gb.build beside the engine): FP64 and FP32
    FLOP/s of this GPU, the roofline denominators that the measured GPU peaks do not list."""
    from tchem_gb.build import PROBE_LIB_PATH
    lib = C.CDLL(str(PROBE_LIB_PATH))
    lib.tchem_gb_probe_fma_peak.restype = C.c_int
    lib.tchem_gb_probe_fma_peak.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    return lib


def caps_for(K: int, cap: int) -> list[int]:
    """Step budgets of the K calls: `cap` for calls 1..K-1, none for the last."""
    return [cap] * (K - 1) + [UNCAPPED]


def engine_arm(args, world: int, rank: int, local: int):
    import torch
    from tchem_gb import AtmosphericChemistry, kernel_launches, tadv_to_device

    assert torch.cuda.is_available(), "the engine arm needs a CUDA device"
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, K, W = args.samples, max(1, args.steps), max(0, args.warmup)
    km, state, tadv, tol_time = workload(B, rank)
    m = km.n_active
    stream = torch.cuda.current_stream(dev)
    L = _capi.lib()

    d_tn = torch.tensor(TOL_NEWTON, dtype=torch.float64, device=dev)
    d_tt = torch.as_tensor(tol_time).to(dev)
    d_tadv = tadv_to_device(tadv, dev)
    d_state = torch.as_tensor(state).to(dev)

    # probe: the autotuner picks the kernel shape (threads per sample) on the first 4096 samples over
    # the full horizon; one more probe run gives the mean step count that sizes the per-call budget
    P0 = min(4096, B)
    tuned = None
    if args.form != "plain":
        tps, times = AtmosphericChemistry.autotune(km, d_tn, d_tt, d_tadv[:P0], d_state[:P0].contiguous(),
                                                   form=args.form, stream=stream)
        tuned = {"threads_per_sample": tps, "probe_samples": P0,
                 "probe_ms": {str(a): round(b, 1) for a, b in times.items()}}
    p_out = torch.empty(P0, d_state.shape[1], dtype=torch.float64, device=dev)
    p_t = torch.zeros(P0, dtype=torch.float64, device=dev)
    p_dt = torch.zeros_like(p_t)
    p_stats = torch.zeros(P0, 8, dtype=torch.int32, device=dev)
    AtmosphericChemistry.runDeviceBatch(d_tn, d_tt, None, d_tadv[:P0], d_state[:P0].contiguous(), p_t, p_dt, p_out,
                                        km, stats=p_stats, form=args.form, stream=stream)
    ps = p_stats.cpu().numpy()
    probe_iters = float((ps[:, 0] + ps[:, 1] + ps[:, 2]).mean())
    cap = max(1, math.ceil(probe_iters / K))
    caps = caps_for(K, cap)

    # warm-up: W calls of the same loop (the first W budgets) on a separate copy of an eighth of the
    # batch (module loading, table staging, clocks; the timed calls start from a fresh copy)
    if W > 0:
        Bw = max(1, B // 8)
        warm = HostLoop(km, args.form, d_tn, d_tt, tadv[:Bw], d_state[:Bw], caps[0], False, dev)
        for k in range(W):
            warm.advance(stream)
            warm.carry(stream, caps[k + 1] if k + 1 < K else UNCAPPED)
        torch.cuda.synchronize(dev)
        assert AtmosphericChemistry.device_error(warm.ws, stream) == 0
        del warm
    loop = HostLoop(km, args.form, d_tn, d_tt, tadv, d_state, caps[0], True, dev)
    torch.cuda.synchronize(dev)

    # timed region: K calls + carry-overs, CUDA events on the launching stream, barrier + sync on
    # both sides; per-call events around the time-advance kernel alone give the roofline's launch time
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize(dev)
    n_launch0 = kernel_launches()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for k in range(K):
            ev[k][0].record(stream)
            loop.advance(stream)
            ev[k][1].record(stream)
            loop.carry(stream, caps[k + 1] if k + 1 < K else cap)
        e1.record(stream)
        torch.cuda.synchronize(dev)
    n_launch = kernel_launches() - n_launch0
    barrier(world)
    ms_local = e0.elapsed_time(e1)
    ms = max_over_ranks(ms_local, world, dev)
    value = B * world / (ms * 1e-3)
    call_ms = [a.elapsed_time(b) for a, b in ev]
    kernel_ms = sum(call_ms)
    status = loop.status.cpu().numpy()
    t_end = loop.t.cpu().numpy()
    stats = loop.total.cpu().numpy()
    out = loop.state.cpu().numpy()
    n_fail = int((status != 0).sum()) - int((status == 2).sum())  # skipped samples finished in an earlier call
    at_horizon = int((t_end >= HORIZON).sum())
    assert AtmosphericChemistry.device_error(loop.ws, stream) == 0

    # roofline of the time-advance kernel: algorithmic flops over all K launches / their summed time
    f32, f64 = work_flops(km, stats)
    peak64, peak32 = C.c_double(), C.c_double()
    probe = fma_probe()
    _capi.check(probe.tchem_gb_probe_fma_peak(1, 4, 4096, C.byref(peak64)), "FP64 FMA probe")
    _capi.check(probe.tchem_gb_probe_fma_peak(0, 4, 65536, C.byref(peak32)), "FP32 FMA probe")
    ach64 = f64 / (kernel_ms * 1e-3) / 1e12
    ach32 = f32 / (kernel_ms * 1e-3) / 1e12
    per_sample = NCU_DRAM_BYTES_PER_SAMPLE.get(args.form)
    traffic = None if per_sample is None else per_sample * B  # every launch reads each sample's row

    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": FORM_DTYPE[args.form], "data": "synthetic (seeded CB05-shaped mechanism and states)",
        "config": {**bench_config(B, args.form, world), "autotuned": tuned,
                   "host_loop": {"calls": K, "steps_per_call": cap, "last_call": "uncapped",
                                 "probe_mean_step_attempts": probe_iters,
                                 "pattern": "runDeviceBatch + carry-over of t and dt per call, in place "
                                            "(state_out = state), as the reference's box-model example"}},
        "samples_at_horizon": at_horizon,
        "failed_samples": n_fail,
        "ms_per_call": [round(x, 1) for x in call_ms],
        "work_per_sample": {k: float(stats[:, i].mean()) for i, k in enumerate(
            ["steps", "rejected", "newton_fail", "newton_iter", "factorizations", "solves", "rhs", "jacobians"])},
        "gpu_launches": n_launch,
        "clocks": clk.summary(),
        "roofline": {"bound": "fp64", "achieved": ach64, "peak": peak64.value / 1e12, "unit": "TFLOP/s",
                     "frac": ach64 / (peak64.value / 1e12), "traffic": traffic,
                     "kernel_ms": kernel_ms, "launches": K,
                     "peak_source": "FMA-chain probe measured in this run (libtchem_gb_probe.so); "
                                    "MEASURED_PEAKS.json has no FP64/FP32 figure",
                     "traffic_source": "DRAM bytes per sample from one ncu capture of a 4096-sample case of this "
                                       "kernel, times the samples of one launch",
                     "fp32": {"achieved": ach32, "peak": peak32.value / 1e12,
                              "frac": ach32 / (peak32.value / 1e12)},
                     "note": "algorithmic FP64 flops count the right-hand sides only (the work formula); "
                             "the FP32 side counts factorizations, solves and Jacobians"},
    }

    if not args.no_e2e:
        line["e2e"] = e2e_loop(km, state, tadv, tol_time, args.form, K, cap, world, dev, stream)

    if rank == 0:
        # plain FP64 form on a subsample (one uncapped call: its trajectory is that of the K calls, since
        # the plain form carries nothing between calls but t, dt and the state): its rate and the FP64
        # end states for the error figure
        P = min(args.plain_samples, B)
        pl_out = None
        if P > 0 and args.form != "plain":
            pl_out = torch.empty(P, d_state.shape[1], dtype=torch.float64, device=dev)
            pl_t = torch.zeros(P, dtype=torch.float64, device=dev)
            pl_dt = torch.zeros_like(pl_t)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            st_p = AtmosphericChemistry.runDeviceBatch(d_tn, d_tt, None, d_tadv[:P], d_state[:P].contiguous(), pl_t,
                                                       pl_dt, pl_out, km, form="plain", stream=stream)
            ev1.record(stream)
            torch.cuda.synchronize(dev)
            plain_rate = P / (ev0.elapsed_time(ev1) * 1e-3)
            pl = pl_out.cpu().numpy()
            e = rel_err(out[:P, 3:3 + m], pl[:, 3:3 + m])
            line["plain_fp64"] = {"value": plain_rate, "unit": "samples/s", "samples": P,
                                  "failed_samples": int((st_p != 0).sum()),
                                  "speedup_of_chosen_form": value / plain_rate,
                                  "note": "subsample of the same batch; samples are independent"}
            line["accuracy_vs_plain_fp64_gpu"] = {"samples": P, "max": float(e.max()),
                                                  "p99": float(np.percentile(e, 99)), "floor": ATOL,
                                                  "share_at_or_below_1e-6": float(np.mean(e <= 1e-6)),
                                                  "bound": 1e-6}
            # the other mixed form on a subsample, with its accuracy against the same FP64 results
            other = "mixed" if args.form == "simplified" else "simplified"
            Q = min(args.other_samples, B)
            if Q > 0:
                tps_o, _ = AtmosphericChemistry.autotune(km, d_tn, d_tt, d_tadv[:min(4096, Q)],
                                                         d_state[:min(4096, Q)].contiguous(), form=other,
                                                         stream=stream)
                q_out = torch.empty(Q, d_state.shape[1], dtype=torch.float64, device=dev)
                q_t = torch.zeros(Q, dtype=torch.float64, device=dev)
                q_dt = torch.zeros_like(q_t)
                ev0.record(stream)
                st_q = AtmosphericChemistry.runDeviceBatch(d_tn, d_tt, None, d_tadv[:Q], d_state[:Q].contiguous(), q_t,
                                                           q_dt, q_out, km, form=other, stream=stream)
                ev1.record(stream)
                torch.cuda.synchronize(dev)
                R = min(P, Q)
                eq = rel_err(q_out[:R].cpu().numpy()[:, 3:3 + m], pl[:R, 3:3 + m])
                line[f"form_{other}"] = {"value": Q / (ev0.elapsed_time(ev1) * 1e-3), "unit": "samples/s",
                                         "samples": Q, "dtype": FORM_DTYPE[other], "threads_per_sample": tps_o,
                                         "failed_samples": int((st_q != 0).sum()),
                                         "accuracy_vs_plain_fp64_gpu": {"samples": R, "max": float(eq.max()),
                                                                        "p99": float(np.percentile(eq, 99)),
                                                                        "floor": ATOL}}
        # CPU oracle: baseline rate and the accuracy reference
        n, _ = cpu_sample_size(km, state, tadv, tol_time, args.cpu_seconds)
        res, el = run_oracle(km, state, tadv, tol_time, n)
        e = rel_err(out[:n, 3:3 + m], res[0][:, 3:3 + m])
        cores = os.cpu_count() or 1
        line["cpu_baseline"] = {"value": n / el, "unit": "samples/s", "cores": cores, "kind": "port",
                                "sample": f"first {n} samples of the batch, 0 -> 3600 s, FP64 TR-BDF2 CPU restatement "
                                          f"built for the host CPU, OpenMP over samples on {cores} threads ({el:.1f} s)"}
        line["accuracy_vs_fp64_oracle"] = {"samples": n, "max": float(e.max()), "p99": float(np.percentile(e, 99)),
                                           "floor": ATOL}
        if pl_out is not None:
            eo = rel_err(pl[:min(n, P), 3:3 + m], res[0][:min(n, P), 3:3 + m])
            line["plain_fp64"]["accuracy_vs_fp64_oracle"] = {"samples": min(n, P), "max": float(eo.max()),
                                                             "bound": 1e-8}

    legs = [("e3sm", args.e3sm_samples, lambda n: e3sm_leg(n, min(args.cpu_seconds, 5.0), dev, stream)),
            ("large_mechanism", args.large_samples, lambda n: large_leg(n, args.large_horizon, dev, stream)),
            ("aerosol", args.aerosol_samples, lambda n: aerosol_leg(n, min(args.cpu_seconds, 5.0), dev, stream)),
            ("uneven_batch", args.uneven_samples, lambda n: uneven_leg(n, args.form, dev, stream)),
            ("adjoint", args.adjoint_samples, lambda n: adjoint_leg(km, state, tol_time, n, dev, stream)),
            ("tc_lu", args.tc_lu_matrices, lambda n: tc_lu_leg(n, dev, stream))]
    for key, n, fn in legs:
        if rank == 0 and n > 0:
            if time.perf_counter() - T_START > args.leg_budget_s:
                line[key] = {"skipped": f"the run passed {args.leg_budget_s:.0f} s before this leg started "
                                        f"(--leg-budget-s); run it alone with its own option"}
                continue
            t0 = time.perf_counter()
            line[key] = fn(n)
            line[key]["leg_wall_s"] = round(time.perf_counter() - t0, 1)
    if rank == 0:
        line["wall_s"] = round(time.perf_counter() - T_START, 1)
        print(json.dumps(line), flush=True)


def e2e_loop(km, state, tadv, tol_time, form: str, K: int, cap: int, world: int, dev, stream) -> dict:
    """The same K-call host loop end to end through the host-buffer C ABI
    (tchem_gb_time_advance_hostbuf, the runHostBatch face): pinned host arrays in, every call copies
    its inputs to the device and its results back, the carry-over of t and dt runs on the host
    between calls (as in the reference's loop over runHostBatch)."""
    import torch
    B, dim, m = state.shape[0], state.shape[1], km.n_active
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    h_state = pin(state.shape, torch.float64)
    h_state[:] = state
    h_tadv = pin((tadv.nbytes,), torch.uint8).view(tadv.dtype)
    h_tadv[:] = tadv
    h_t = pin((B,), torch.float64)
    h_t[:] = 0.0
    h_dt = pin((B,), torch.float64)
    h_st = pin((B,), torch.int32)
    tn = np.asarray(TOL_NEWTON, dtype=np.float64)
    o = _capi.AdvanceOpts()
    o.form = {"plain": 0, "mixed": 1, "simplified": 2}[form]
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    handles = (C.c_void_p * 1)(km.handle.value)
    caps = caps_for(K, cap)
    L = _capi.lib()
    h_tadv["num_time_iterations_per_interval"] = caps[0]
    barrier(world)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for k in range(K):
        rc = L.tchem_gb_time_advance_hostbuf(handles, 1, None, B, p(tn), p(tol_time), p(h_tadv), p(h_state),
                                             p(h_t), p(h_dt), p(h_state), p(h_st), None, C.byref(o),
                                             C.c_void_p(stream.cuda_stream))
        _capi.check(rc, "tchem_gb_time_advance_hostbuf")
        h_tadv["tbeg"] = h_t
        h_tadv["dt"] = h_dt
        h_tadv["num_time_iterations_per_interval"] = caps[k + 1] if k + 1 < K else cap
    el = time.perf_counter() - t0
    el = max_over_ranks(el, world, dev)
    h2d = 16 + 16 * m + tadv.itemsize * B + 8 * B * dim + 8 * B
    d2h = 8 * B * dim + 8 * B + 8 * B + 4 * B
    return {"value": B * world / el, "unit": "samples/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": K, "samples_at_horizon": int((h_t >= HORIZON).sum()),
            "failed_samples": int(((h_st != 0) & (h_st != 2)).sum()),
            "path": "tchem_gb_time_advance_hostbuf per call (C ABI, pinned host buffers, copies inside the timed "
                    "region), host-side carry-over of t and dt"}


def main():
    args = parse()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        engine_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
