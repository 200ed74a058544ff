#!/usr/bin/env python3
"""Benchmark of the flow timestep on GB300: cell-steps/s of the FP64 solver.

Workload (one "step" = one timestep, solve_hydro_2d + the conservation totals
the reference driver computes every iteration, main.c:82-91): a Sedov-type
blast on a 4096^2 uniform mesh, FP64, gamma 1.4, density 1, specific energy
1e-5 with a central 4x4-cell square at 1e4, zero velocity, reflective walls,
the params dt set to the CFL estimate of the initial state, 500 iterations.
Synthetic data.  The state (15 arrays of 4100^2 doubles, 2 GB) is larger than
L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line on rank 0.  Besides the timed FP64 line it reports:
  parity        per-field maxima of the fused step against the oracle (the C
                restatement of the reference omp3 set, strict IEEE) after the
                workload's full 500 steps;
  forms         the mixed-precision form (blast, 8192^2 Sod, a field in
                motion everywhere) and the batched forms at their stated
                lengths (200 and 1000 steps), with their errors;
  reference_cuda (in forms) the reference's own cuda kernel set built for
                sm_103a, timed on the same workload and GPU;
  cpu_baseline  the reference's own omp3 set built with its flags (where its
                sources were staged and built), else the oracle with the same
                flags, on the host cores.
With --impl reference the same workload runs on the host cores through that
same CPU build.  Under torchrun (N > 1) every rank advances its own replica
(the single-mesh decomposition, flow_gb300.decomp, exchanges halos through
host hooks and is not timed here).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s, % HBM peak: FP64 vs mixed/batched at stated L1 err"
UNIT = "cell-steps/s"
N_CELLS_SIDE = 4096
CONFIG_STEPS = 500   # the blast workload's stated length
B_ALG_FP64 = 64      # bytes/cell-step: rho, e, rho_u, rho_v read + written once
B_ALG_MIXED = 48     # rho, e (FP64) and rho_u, rho_v (FP32), each read + written

# Bytes per interior cell each fused kernel moves on a tile at rest through
# the step and the one before it (the blast's ambient mesh): the flags and
# skip marks only, so 0 -- the pressure phase, the CFL minimum, the first
# sweep's round-trip test and the velocity store take the previous step's
# results there.  Where the flow moves a kernel moves its full arrays; its
# bytes per cell on a whole workload are therefore measured (ncu, the
# committed figures below) rather than fixed here.
KERNEL_BYTES_PER_CELL = {
    "lag_pressure": 0, "lag_viscosity": 0, "lag_viscous_accel": 0, "lag_energy_dt": 0,
    "lag_fused": 8 * 6,          # one-kernel Lagrangian phase: rho, e, rho_u, rho_v in; u, v out
    "lag_apply": 0,
    "mass_sweep_x": 0, "mass_sweep_y": 0,
    "mom_uFx": 0, "mom_uFy": 0, "mom_vFx": 0, "mom_vFy": 0,
    "mesh_pow2": 0,
}

# ncu figures (DRAM bytes per cell of each kernel on the blast workload, FP64
# instructions per cell-step on a field in motion) with the fingerprint of the
# kernel sources they were measured on; used only while the sources match.
PROFILE_FIGURES = os.path.join(ROOT, "profiles", "ncu_figures_fused_fp64.json")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=CONFIG_STEPS)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=N_CELLS_SIDE)
    p.add_argument("--workload", default="sedov", choices=["sedov", "smooth"],
                   help="the FP64 line's problem: the blast (default) or a field in "
                        "motion everywhere")
    p.add_argument("--no-cpu-baseline", action="store_true",
                   help="skip the host-core legs (CPU baseline and oracle checks)")
    p.add_argument("--fp64-only", action="store_true", help="skip the mixed/batched forms")
    p.add_argument("--sod-size", type=int, default=8192,
                   help="side of the Sod tube of the mixed form (0 skips it)")
    p.add_argument("--parity-steps", type=int, default=CONFIG_STEPS,
                   help="steps of the per-cell oracle comparison (0 skips it)")
    p.add_argument("--batch-fp64-steps", type=int, default=200,
                   help="timed steps of the batched FP64 ensemble (its stated length)")
    p.add_argument("--batch-mixed-steps", type=int, default=1000,
                   help="timed steps of the batched mixed ensemble (its stated length)")
    return p.parse_args()


def dist_env():
    from flow_gb300.replicas import dist_env as env
    return env()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# The translation unit of the single-problem timestep kernels (fused.cu and
# everything it includes): the sources the committed ncu figures describe.
STEP_SOURCES = ("common.cuh", "fused.cu", "fused.h", "fused_math.cuh", "fused_tiles.cuh",
                "lag_fused.cuh", "precision.cuh", "profile.h", "stages.h")


def source_fingerprint() -> str:
    """sha256 (16 hex digits) of the timestep kernels' sources, in name order."""
    h = hashlib.sha256()
    csrc = os.path.join(ROOT, "flow_gb300", "csrc")
    for name in STEP_SOURCES:
        with open(os.path.join(csrc, name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def profile_figures():
    """The committed ncu figures when they were measured on these sources."""
    try:
        with open(PROFILE_FIGURES) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    return d if d.get("source_fingerprint") == source_fingerprint() else None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# Host-core leg: the oracle (C restatement of the reference omp3 set) as the
# timed CPU baseline and as the checker of the GPU results.  Nothing here is
# on the GPU path.

def _omp_env():
    ncpu = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncpu))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    return int(os.environ["OMP_NUM_THREADS"])


def main_problem(problems, workload: str, n: int):
    """The FP64 line's problem: the Sedov-type blast, or density and energy
    1 + a 16-mode smooth random field (seed 20261205)."""
    if workload == "smooth":
        import numpy as np
        return problems.smooth_random(n, np.random.default_rng(20261205))
    return problems.sedov(n)


def oracle_start(prob):
    """Host mesh and state of a problem, after the driver's initial
    set_timestep (main.c:64-66)."""
    from oracle import oracle as O
    hm = O.HostMesh(prob.gnx, prob.gny, width=prob.width, height=prob.height,
                    dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st)
    return hm, st


class quiet_stdout:
    """Sends file descriptor 1 to /dev/null (the reference's own code prints
    dt and totals every step; the benchmark prints one JSON line)."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)
        return self

    def __exit__(self, *exc):
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def cpu_kind() -> str:
    """The reference's own omp3 set built with its flags where it was built
    (oracle/_ref), else the oracle with the same flags."""
    from oracle import oracle as O
    ok = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libflow_ref_default.so"))
    return "reference_default" if ok else "fast"


def cpu_run(n: int, steps: int, warmup: int, budget_s: float, workload: str = "sedov"):
    """Times the reference's omp3 set (or, where it was not built, the oracle)
    built with the reference's flags (-O3 -march=native -fopenmp, Makefile:15)
    on the same workload, a step being solve_hydro_2d + print_conservation as
    the reference driver times it (main.c:80-93); returns (cell-steps/s,
    steps timed, threads, kind).  Times all `steps` steps unless that would
    take more than about budget_s seconds."""
    threads = _omp_env()
    from flow_gb300 import problems
    from oracle import oracle as O
    kind = cpu_kind()
    prob = main_problem(problems, workload, n)
    hm = O.HostMesh(n, n, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    L = O.lib(kind)
    with quiet_stdout():
        O.initial_timestep(hm, st, kind)

        def one(tt):
            O.step(hm, st, tt, kind)
            L.print_conservation(hm.nx, hm.ny, O.ptr(st["rho"]), O.ptr(st["e"]),
                                 O.ptr(st["reduce"]), O.ctypes.byref(hm.mesh))

        tt = 0
        for _ in range(max(1, warmup)):
            t0 = time.perf_counter()
            one(tt)
            tt += 1
            t_step = time.perf_counter() - t0
        timed = max(1, min(steps, int(budget_s / max(t_step, 1e-6))))
        t0 = time.perf_counter()
        for _ in range(timed):
            one(tt)
            tt += 1
        el = time.perf_counter() - t0
    return n * n * timed / el, timed, threads, kind


def oracle_compare(fields: dict, prob, steps: int, dt_pair=None):
    """Advances the oracle (strict IEEE build) `steps` steps from the problem's
    initial state and compares the given GPU fields (interior arrays by name)
    per cell: the largest |a-b| / max(|b|, 1e-3 max|b|) (the tests'
    tolerance measure), the L1 error sum|a-b| / sum|b| and the count of cells
    that differ at all."""
    import numpy as np
    from oracle import oracle as O
    _omp_env()
    hm, st = oracle_start(prob)
    O.run(hm, st, steps)
    out = {}
    for k, got in fields.items():
        want = st.interior(k)
        got = np.asarray(got, dtype=np.float64)
        scale = float(np.abs(want).max()) if want.size else 0.0
        d = np.abs(got - want)
        if scale == 0.0:
            out[k] = {"max_abs": float(d.max()), "cells_differing": int(np.count_nonzero(d))}
            continue
        rel = d / np.maximum(np.abs(want), 1e-3 * scale)
        out[k] = {"max_cell_rel": float(rel.max()),
                  "l1": float(d.sum() / np.abs(want).sum()),
                  "linf": float(d.max() / scale),
                  "cells_differing": int(np.count_nonzero(got != want))}
    if dt_pair is not None:
        out["dt"] = {"rel": abs(dt_pair[0] - hm.mesh.dt) / hm.mesh.dt,
                     "dt_h_rel": abs(dt_pair[1] - hm.mesh.dt_h) / hm.mesh.dt_h}
    return out


CPU_WHAT = {
    "reference_default": "the reference's own omp3/flow.c, main.c's step, built -O3 "
                         "-march=native -fopenmp as its Makefile:15 on the restated arch layer",
    "fast": "the oracle, a C restatement of the reference omp3 set that the tests hold "
            "bit-identical to it, built -O3 -march=native -fopenmp as the reference's Makefile:15",
}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    value, timed, threads, kind = cpu_run(args.size, args.steps, args.warmup, budget_s=150.0,
                                          workload=args.workload)
    sample = (f"{args.workload} {args.size}^2 FP64 timesteps + conservation totals on "
              f"{threads} host threads ({CPU_WHAT[kind]}): {timed} of {args.steps} requested "
              f"steps timed after {args.warmup} warm-up")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": args.size * args.size / value * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}_{args.size}_fp64", "nx": args.size, "ny": args.size,
                   "form": "fp64", "parallelism": "host OpenMP"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": "reference" if kind == "reference_default" else "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side.

def field_errors(fg, got, want, names=("rho", "e")):
    """L1 (sum|d| / sum|want|) and L-infinity (max|d| / max|want|) per field."""
    out = {}
    for k in names:
        a = got.interior(k)
        b = want.interior(k)
        if abs(b).max() == 0.0:
            # A field that stays zero in the FP64 path (rho_v of a tube split
            # along x): absolute errors instead.
            out[k] = {"l1_abs": float(abs(a - b).mean()), "linf_abs": float(abs(a - b).max())}
            continue
        out[k] = {"l1": float(abs(a - b).sum() / abs(b).sum()),
                  "linf": float(abs(a - b).max() / abs(b).max())}
    return out


def batch_problems(problems, kind: str):
    """The batched FP64 ensemble (kind "two_region"): 256 two-region instances
    with sides drawn from {128, 192, ..., 1024}; the batched mixed ensemble
    (kind "smooth"): 64 instances of 2048^2 smooth random fields.  Seeded."""
    import numpy as np
    if kind == "two_region":
        rng = np.random.default_rng(20261203)
        sides = rng.choice(np.arange(128, 1025, 64), size=256)
        return [problems.two_region(int(n), rng) for n in sides]
    rng = np.random.default_rng(20261204)
    return [problems.smooth_random(2048, rng) for _ in range(64)]


def run_batched_form(fg, problems, torch, device, kind, precision, steps, warmup, oracle_samples):
    """Times one batched ensemble (autotuned, graph-replayed) for `steps`
    steps and measures its error on sampled instances at the final step
    against the single-problem FP64 step on the GPU and, for the first
    `oracle_samples` of them, against the oracle on the host cores."""
    import numpy as np
    from flow_gb300.replicas import max_over_ranks, shard_instances, sum_over_ranks
    rank, world, _ = dist_env()
    probs = batch_problems(problems, kind)
    if world > 1:
        # Under torchrun the ensemble is split across the GPUs by instance.
        mine = shard_instances([p.gnx * p.gny for p in probs], rank, world)
        probs = [probs[i] for i in mine]
    b = fg.Batch(probs, precision=precision, device=device)
    tune = b.autotune(steps=2)
    b.step(warmup)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    b.step(steps, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    b.status()
    ms = max_over_ranks(e0.elapsed_time(e1), device)
    cells = int(sum_over_ranks(b.cells, device))
    value = cells * steps / (ms * 1e-3)
    total_steps = b.steps_done
    samples = [0, len(probs) // 2]
    errs, finals = {}, {}
    for i in samples:
        rho, e, dt, _ = b.state(i)
        ref = fg.DeviceSim(probs[i], device)
        ref.initial_timestep()
        ref.run(total_steps)
        rr, er = ref.interior("rho"), ref.interior("e")
        name = f"instance_{i}_{probs[i].gnx}x{probs[i].gny}"
        errs[name] = {
            "vs_fp64_gpu": {
                "rho_l1": float(np.abs(rho - rr).sum() / np.abs(rr).sum()),
                "e_l1": float(np.abs(e - er).sum() / np.abs(er).sum()),
                "rho_linf": float(np.abs(rho - rr).max() / np.abs(rr).max()),
                "max_abs_diff": float(max(np.abs(rho - rr).max(), np.abs(e - er).max()))}}
        finals[name] = (probs[i], {"rho": rho, "e": e})
        del ref
    del b
    torch.cuda.empty_cache()
    seq = run_sequential_ensemble(fg, torch, device, probs, precision, warmup=1, steps=2)
    b_alg = B_ALG_FP64 if precision == 0 else B_ALG_MIXED
    out = {"workload": f"batch_{kind}_{'fp64' if precision == 0 else 'mixed'}",
           "instances": len(probs), "cells": cells, "value": value, "unit": UNIT,
           "ms_per_step": ms / steps, "steps_timed": steps, "steps_total": total_steps,
           "graph": True, "tuning": tune,
           "hbm_fraction_of_step": value * b_alg / (measured_peaks()[0] * 1e9),
           "errors": errs,
           "sequential_same_ensemble": seq,
           "speedup_vs_sequential": value / seq["value"]}
    # The first sampled instances against the oracle (host cores).
    oracle_todo = list(finals.items())[:oracle_samples]
    return out, total_steps, oracle_todo


def run_sequential_ensemble(fg, torch, device, probs, precision, warmup, steps):
    """The same ensemble advanced one problem at a time through the
    single-problem path of the same precision (solve_hydro_2d per instance, or
    gb300_mixed_solve), each instance its own arrays: what a caller without
    the batched form would run."""
    sims = [(fg.DeviceSim if precision == 0 else fg.MixedSim)(p, device) for p in probs]
    if precision == 0:
        for s in sims:
            s.initial_timestep()
    for _ in range(warmup):
        for s in sims:
            s.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for s in sims:
            s.step()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    cells = sum(p.gnx * p.gny for p in probs)
    del sims
    torch.cuda.empty_cache()
    return {"value": cells * steps / el, "unit": UNIT, "steps_timed": steps,
            "ms_per_step": el * 1e3 / steps,
            "what": "per-instance single-problem steps, host-timed (each step reads dt back)"}


def timed_run(torch, sim, steps, warmup):
    for _ in range(warmup):
        sim.step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        sim.step()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def smooth_problem(problems, n):
    import numpy as np
    return problems.smooth_random(n, np.random.default_rng(20261205))


def run_fp64_smooth(fg, problems, torch, device, n, steps, warmup, figures, fma_rate):
    """The FP64 step on a field with structure everywhere (density and energy
    1 + a 16-mode smooth random field, seed 20261205): no flat regions, so
    every slope and limiter is live -- the general-case rate next to the
    blast problem, most of whose mesh is still at rest.  Bound by the FP64
    pipe: its fraction is the FP64 instructions per cell-step (ncu) times the
    cell-steps/s over the measured FP64 issue rate."""
    sim = fg.DeviceSim(smooth_problem(problems, n), device)
    sim.initial_timestep()
    ms = timed_run(torch, sim, steps, warmup)
    del sim
    torch.cuda.empty_cache()
    value = n * n * steps / (ms * 1e-3)
    out = {"workload": f"smooth_{n}_fp64", "value": value, "unit": UNIT,
           "ms_per_step": ms / steps, "steps": steps, "warmup": warmup,
           "hbm_fraction_of_step": value * B_ALG_FP64 / (measured_peaks()[0] * 1e9)}
    per_cell = (figures or {}).get("fp64_inst_per_cell_step_moving")
    if per_cell and fma_rate > 0:
        out["fp64_pipe"] = {"fp64_inst_per_cell_step": per_cell,
                            "fraction_of_measured_fp64_rate": per_cell * value / fma_rate}
    return out


def run_reference_cuda(fg, problems, torch, device, n, steps, warmup, workload, fused_value):
    """A second GPU baseline: the reference's own cuda kernel set (cuda/flow.cu
    and cuda/flow.k, its flow_interface.h entry points) built for sm_103a on
    the restated arch CUDA layer, timed on the same workload and GPU -- a step
    is its solve_hydro_2d (22 kernels and 19 ghost fills, each followed by a
    device synchronisation, and the dt read back) -- with its errors against
    the fused step after the same steps."""
    import ctypes
    from oracle import oracle as O
    if not O.have_reference_cuda():
        return {"unavailable": "the reference's cuda set was not built here (its sources "
                               "were not staged to this machine)"}
    Lr = O.lib("reference_cuda")
    sim = fg.DeviceSim(main_problem(problems, workload, n), device)
    m = sim.mesh
    mp = ctypes.cast(ctypes.addressof(m), ctypes.POINTER(O.Mesh))
    args = sim.args()
    with quiet_stdout():
        Lr.set_timestep(sim.nx, sim.ny, args[8], args[9], args[1], args[3], mp, args[16], 0,
                        m.celldx, m.celldy)
        for tt in range(warmup):
            Lr.solve_hydro_2d(mp, tt, *args)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for tt in range(warmup, warmup + steps):
            Lr.solve_hydro_2d(mp, tt, *args)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
    value = n * n * steps / el
    ref = fg.DeviceSim(main_problem(problems, workload, n), device)
    ref.initial_timestep()
    ref.run(warmup + steps)
    errs = field_errors(fg, sim, ref, names=STATE)
    del sim, ref
    torch.cuda.empty_cache()
    return {"workload": f"{workload}_{n}_fp64", "value": value, "unit": UNIT,
            "ms_per_step": el * 1e3 / steps, "steps": steps, "warmup": warmup,
            "what": "the reference's cuda set (cuda/flow.cu, cuda/flow.k) for sm_103a, host-timed",
            "fused_fp64_over_reference_cuda": fused_value / value,
            "errors_vs_fused_fp64": errs}


def mixed_problem(problems, workload, n):
    if workload == "sedov":
        return problems.sedov(n)
    if workload == "sod":
        return problems.sod(n)
    return smooth_problem(problems, n)


def run_mixed_form(fg, problems, torch, device, workload, n, steps, warmup):
    """Times the mixed form on a workload and measures it against the FP64
    path after the same steps from the same initial state (the FP64 path is
    held to the oracle per cell): L1/Linf per field and the mass/energy
    drift.  Also times the FP64 path on that workload for the speed-up."""
    sim = fg.MixedSim(mixed_problem(problems, workload, n), device)
    ms = timed_run(torch, sim, steps, warmup)
    value = n * n * steps / (ms * 1e-3)
    ref = fg.DeviceSim(mixed_problem(problems, workload, n), device)
    ref.initial_timestep()
    ms_ref = timed_run(torch, ref, steps, warmup)
    fp64_value = n * n * steps / (ms_ref * 1e-3)
    out = {"workload": f"{workload}_{n}_mixed", "value": value, "unit": UNIT,
           "ms_per_step": ms / steps, "steps": steps, "warmup": warmup,
           "hbm_fraction_of_step_48B": value * B_ALG_MIXED / (measured_peaks()[0] * 1e9),
           "errors_vs_fp64": field_errors(fg, sim, ref,
                                          names=("rho", "e", "u", "v", "rho_u", "rho_v"))}
    cm, cr = sim.conservation(), ref.conservation()
    out["mass_drift"] = abs(cm[0] - cr[0]) / cr[0]
    out["energy_drift"] = abs(cm[1] - cr[1]) / cr[1]
    out["fp64_value_same_workload"] = fp64_value
    out["speedup_vs_fp64"] = value / fp64_value
    del sim, ref
    torch.cuda.empty_cache()
    return out


STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = f"cuda:{local}"
    torch.cuda.set_device(device)
    import flow_gb300 as fg
    from flow_gb300 import build, problems
    if not os.path.exists(fg.LIB_PATH):
        build.build()
    L = fg.lib()
    fg.set_stream(torch.cuda.current_stream())
    fg.set_mode(fg.MODE_FUSED)
    n = args.size
    figures = profile_figures()

    from flow_gb300.replicas import barrier, job_throughput, max_over_ranks

    prob = main_problem(problems, args.workload, n)
    sim = fg.DeviceSim(prob, device)
    sim.initial_timestep()
    out2 = (fg.ctypes.c_double * 2)()
    out2p = fg.ctypes.cast(out2, fg.ctypes.POINTER(fg.ctypes.c_double))
    nx, ny = sim.nx, sim.ny

    def step():
        sim.step()
        # The pointers of the totals' arrays, formed once per sim (kept on it).
        ca = getattr(sim, "_totals_args", None)
        if ca is None:
            ca = sim._totals_args = (fg.dptr(sim.a["rho"]), fg.dptr(sim.a["e"]),
                                     fg.dptr(sim.a["reduce"]))
        if L.gb300_conservation(nx, ny, 2, *ca, out2p, 1) != 0:
            fg.check()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    # No per-kernel events here: an event between two kernels serialises the
    # programmatic launch of the second (which otherwise fills the SMs the
    # first one's last wave leaves idle).  The per-kernel durations come from
    # the profiled pass below, the same steps of the same workload.
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        launches0 = L.gb300_launch_count()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        launches = L.gb300_launch_count() - launches0
        barrier()
    # The job's time is its slowest replica's.
    ms = max_over_ranks(e0.elapsed_time(e1), device)
    ms_per_step = ms / args.steps
    value = job_throughput(n * n * args.steps, world, ms * 1e-3)
    mass, energy = out2[0], out2[1]

    # ---- profiled pass: the same steps from the same initial state, with a
    # CUDA event on the launch stream before every kernel ----
    del sim
    torch.cuda.empty_cache()
    sim = fg.DeviceSim(main_problem(problems, args.workload, n), device)
    sim.initial_timestep()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    L.gb300_profile_reset()
    L.gb300_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    L.gb300_profile_enable(0)

    kernels = []
    buf = fg.ctypes.create_string_buffer(64)
    nlaunch = fg.ctypes.c_longlong()
    tot = fg.ctypes.c_double()
    for i in range(L.gb300_profile_count()):
        L.gb300_profile_entry(i, buf, 64, fg.ctypes.byref(nlaunch), fg.ctypes.byref(tot))
        kernels.append((buf.value.decode(), nlaunch.value, tot.value))
    kernels.sort(key=lambda k: -k[2])

    # ---- end to end through the C ABI with host buffers ----
    fields = ("rho", "e", "rho_u", "rho_v", "u", "v")
    prob2 = main_problem(problems, args.workload, n)
    sim2 = fg.DeviceSim(prob2, device)
    host_in = {f: sim2.a[f].cpu().pin_memory() for f in fields}
    host_out = {f: torch.empty_like(host_in[f]).pin_memory() for f in fields}
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for f in fields:
        sim2.a[f].copy_(host_in[f], non_blocking=True)
    sim2.initial_timestep()
    ca2 = (fg.dptr(sim2.a["rho"]), fg.dptr(sim2.a["e"]), fg.dptr(sim2.a["reduce"]))
    for _ in range(args.steps):
        sim2.step()
        if L.gb300_conservation(nx, ny, 2, *ca2, out2p, 1) != 0:
            fg.check()
    for f in fields:
        host_out[f].copy_(sim2.a[f], non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, device)
    barrier()
    h2d = sum(host_in[f].numel() * 8 for f in fields)
    d2h = sum(host_out[f].numel() * 8 for f in fields)
    e2e_value = job_throughput(n * n * args.steps, world, e2e_s)
    del host_in, host_out, sim, sim2
    torch.cuda.empty_cache()

    # ---- parity of the timed path on the full workload (rank 0) ----
    parity = None
    host_legs = rank == 0 and not args.no_cpu_baseline
    if host_legs and args.parity_steps > 0:
        psim = fg.DeviceSim(main_problem(problems, args.workload, n), device)
        psim.initial_timestep()
        psim.run(args.parity_steps)
        got = {k: psim.interior(k) for k in STATE}
        pair = (psim.mesh.dt, psim.mesh.dt_h)
        del psim
        torch.cuda.empty_cache()
        parity = {"steps": args.parity_steps,
                  "against": "oracle: C restatement of the reference omp3 set, strict IEEE "
                             "(bit-identical to the reference compiled from its sources)",
                  "measure": "max_cell_rel = max |a-b| / max(|b|, 1e-3 max|b|)",
                  "tolerance": 1e-12,
                  "fields": oracle_compare(got, main_problem(problems, args.workload, n),
                                           args.parity_steps, pair)}
        parity["within_tolerance"] = all(
            v.get("max_cell_rel", 0.0) <= 1e-12 for k, v in parity["fields"].items() if k != "dt")

    fma_rate = fg.ctypes.c_double()
    L.gb300_measure_fp64_fma_rate(fg.ctypes.byref(fma_rate))

    # ---- the mixed-precision and batched forms ----
    forms = {}
    oracle_checks = []
    if not args.fp64_only:
        forms["reference_cuda"] = run_reference_cuda(fg, problems, torch, device, n,
                                                     min(args.steps, 50), 2, args.workload,
                                                     value / world)
        if args.workload != "smooth":
            forms["fp64_smooth"] = run_fp64_smooth(fg, problems, torch, device, n,
                                                   min(args.steps, 100), args.warmup, figures,
                                                   fma_rate.value)
        for workload, size in (("sedov", n), ("sod", args.sod_size), ("smooth", n)):
            if size <= 0:
                continue
            name = {"sedov": "mixed", "sod": f"mixed_sod_{size}", "smooth": "mixed_smooth"}[workload]
            forms[name] = run_mixed_form(fg, problems, torch, device, workload, size,
                                         args.steps if workload != "smooth" else min(args.steps, 100),
                                         args.warmup)
        for key, kind, prec, steps, nsamp in (
                ("batched_fp64", "two_region", 0, args.batch_fp64_steps, 2),
                ("batched_mixed", "smooth", 1, args.batch_mixed_steps, 1)):
            if steps <= 0:
                continue
            res, total, todo = run_batched_form(fg, problems, torch, device, kind, prec, steps,
                                                args.warmup, nsamp)
            forms[key] = res
            oracle_checks += [(key, name, p, f, total) for name, (p, f) in todo]

    if rank != 0:
        return

    # Batched instances against the oracle at their final step (host cores).
    if host_legs:
        for key, name, p, f, total in oracle_checks:
            res = oracle_compare(f, p, total)
            forms[key]["errors"][name]["vs_oracle"] = {
                k: {m: v[m] for m in ("l1", "linf", "max_cell_rel") if m in v}
                for k, v in res.items()}

    # ---- roofline of the whole step and of the dominant kernel ----
    peak, peak_kind = measured_peaks()
    name, nl, total = kernels[0] if kernels else ("none", 1, float("nan"))
    cells = (nx - 4) * (ny - 4)
    measured_bpc = (figures or {}).get("dram_bytes_per_cell") or {}

    def kernel_bpc(k):
        """DRAM bytes per cell kernel k moves on this workload (ncu, when the
        figures describe these sources), else its bytes on a tile at rest."""
        return measured_bpc.get(k, KERNEL_BYTES_PER_CELL.get(k, B_ALG_FP64))

    achieved = kernel_bpc(name) * cells / (total / nl * 1e-3) / 1e9
    tb = measured_bpc.get(name)
    traffic = tb * cells if tb is not None else None
    step_gbs = value / world * B_ALG_FP64 / 1e9
    step_bpc = (figures or {}).get("dram_bytes_per_cell_step")

    cpu = None
    if host_legs:
        cv, timed, threads, kind = cpu_run(n, args.steps, 1, budget_s=60.0,
                                           workload=args.workload)
        cpu = {"value": cv, "unit": UNIT, "cores": threads,
               "kind": "reference" if kind == "reference_default" else "port",
               "sample": f"{args.workload} {n}^2 FP64 timesteps + conservation totals, {timed} "
                         f"of the GPU arm's {args.steps} steps, on {threads} host threads "
                         f"({CPU_WHAT[kind]})"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}_{n}_fp64", "nx": n, "ny": n, "form": "fp64",
                   "iterations_timed": args.steps, "l2": "inputs larger than L2 (2.3 GB state), no flush; a step re-reads only the "
                         "tiles that move (0.9 DRAM B/cell-step, ncu), whose data and the "
                         "flags may stay in L2 from one step to the next as in any run",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "hbm_fraction_of_step": value / world * B_ALG_FP64 / (peak * 1e9)},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps + 32,
                "what": "initial state H2D from pinned host, K timesteps + conservation readback "
                        "through the C ABI, final state D2H"},
        # The step as the unit (its 64 algorithmic bytes per cell-step: rho,
        # e, rho_u, rho_v read and written once), timed live with CUDA
        # events; traffic: the DRAM bytes ncu measured per step on this
        # workload.  kernel: the dominant kernel, on the DRAM bytes per cell
        # ncu measured for it on this workload over its live duration.
        "roofline": {"bound": "hbm", "kernel": "timestep", "achieved": step_gbs, "peak": peak,
                     "unit": "GB/s", "frac": step_gbs / peak,
                     "traffic": step_bpc * cells if step_bpc is not None else None,
                     "peak_kind": peak_kind,
                     "what": "cell-steps/s x 64 B (rho, e, rho_u, rho_v read and written once "
                             "per step) over the measured copy bandwidth",
                     "dram_bytes_per_cell_step": step_bpc,
                     "dominant_kernel": {"name": name, "achieved": achieved,
                                         "frac": achieved / peak, "traffic": traffic,
                                         "bytes_per_cell": kernel_bpc(name)}},
        "fp64_pipe": {"fma_per_s_peak": fma_rate.value,
                      "note": "FP64 issue rate measured on this GPU; bounds the FP64 step on "
                              "fields in motion (forms.fp64_smooth.fp64_pipe)"},
        # Per kernel: launches, total ms, share of the step, and the GB/s of
        # the DRAM bytes per cell it moves on this workload (kernel_bpc) over
        # its live duration, with the fraction of the measured copy bandwidth.
        "kernels": [{"name": k, "launches": c, "ms": t, "share": t / sum(x[2] for x in kernels),
                     "bytes_per_cell": kernel_bpc(k),
                     "gbs": kernel_bpc(k) * cells / (t / c * 1e-3) / 1e9,
                     "frac": kernel_bpc(k) * cells / (t / c * 1e-3) / 1e9 / peak}
                    for k, c, t in kernels],
        "parity": parity,
        "forms": forms,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "mass": mass, "energy": energy,
        "kernel_sources": source_fingerprint(),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
