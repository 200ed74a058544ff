#!/usr/bin/env python3
"""Benchmark of the flow timestep on GB300: cell-steps/s of the FP64 solver.

Workload (one "step" = one timestep, solve_hydro_2d + the conservation totals
the reference driver computes every iteration, main.c:82-91): a Sedov-type
blast on a 4096^2 uniform mesh, FP64, gamma 1.4, density 1, specific energy
1e-5 with a central 4x4-cell square at 1e4, zero velocity, reflective walls,
the params dt set to the CFL estimate of the initial state.  Synthetic data.
The state (17 arrays of 4100^2 doubles, 2.3 GB) is larger than L2, so no L2
flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line on rank 0.  With --impl reference the same workload runs
on the host cores through the CPU oracle (a C restatement of the reference
omp3 kernel set, bit-exact with it), since the reference has no GPU path that
builds here.  Under torchrun (N > 1) every rank advances its own independent
replica (the single-mesh timestep does not shard without a halo exchange).
"""
from __future__ import annotations

import argparse
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
B_ALG_FP64 = 64  # bytes/cell-step: rho, e, rho_u, rho_v read + written once

# Algorithmic bytes per interior cell of each fused kernel: the arrays it must
# read and write once (8 bytes each) on every cell.  Arrays that change only
# where the flow moves (momenta, energy) are counted as read; their writes on
# moving cells come on top.  Used for the per-kernel HBM roofline.
KERNEL_BYTES_PER_CELL = {
    "lag_pressure": 8 * 8,       # rho, e, rho_u, rho_v in; P, rho_old, u, v out
    "lag_viscosity": 8 * 5,      # u, v, rho in; Qxx, Qyy out
    "lag_viscous_accel": 8 * 2,  # Qxx, Qyy in (momenta, densities, velocities where a stress gradient acts)
    "lag_energy_dt": 8 * 6,      # rho, e, Qxx, Qyy, u, v in (P in, e out where the cell is compressed)
    "mass_sweep_x": 8 * 6,       # rho, e, u in; rho, e, F_x out
    "mass_sweep_y": 8 * 6,
    # Momentum pairs (flux fused with its update), one launch per step each;
    # the velocity is recomputed (rho, the momentum in, the velocity out:
    # 24 B) in every other step's launch, so half of it counts per launch.
    "mom_uFx": 8 + 12,           # F_x in (u where mass moves)
    "mom_uFy": 16 + 12,          # F_y, u in
    "mom_vFx": 16 + 12,          # F_x, u in (v where mass moves)
    "mom_vFy": 16 + 12,          # F_y, v in
    "mesh_pow2": 0,              # the step's one-block mesh test (spacings only)
}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per interior cell of
# one launch, from an ncu capture (one pass) of the FP64 fused kernels on the
# Sedov blast at the benchmark size, 4096^2, after five timesteps; scaled to a
# launch by its cell count.
NCU_TRAFFIC_BYTES_PER_CELL = {
    "lag_pressure": 62.2,
    "lag_viscosity": 38.7,
    "lag_viscous_accel": 16.0,
    "lag_energy_dt": 48.2,
    "mass_sweep_x": 53.0,
    "mass_sweep_y": 45.4,
    "mom_uFx": 30.6,             # the launch that recomputes u
    "mom_uFy": 16.0,
    "mom_vFx": 39.1,             # the launch that recomputes v
    "mom_vFy": 16.0,
}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=N_CELLS_SIDE)
    p.add_argument("--workload", default="sedov", choices=["sedov", "smooth"],
                   help="the FP64 line's problem: the blast (default) or a field in "
                        "motion everywhere")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--fp64-only", action="store_true", help="skip the mixed/batched forms")
    p.add_argument("--sod-size", type=int, default=8192,
                   help="side of the Sod tube of the mixed form (0 skips it)")
    p.add_argument("--batch-steps", type=int, default=20,
                   help="timed steps of each batched form (a sample of its 200/1000)")
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
# CPU side: the oracle (C restatement of the reference omp3 set).

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


def cpu_run(n: int, steps: int, warmup: int, budget_s: float, workload: str = "sedov"):
    """Times the oracle on the same workload; returns (cell-steps/s, steps
    timed, threads).  Times at most ~budget_s seconds of steps."""
    threads = _omp_env()
    from flow_gb300 import problems
    from oracle import oracle as O
    prob = main_problem(problems, workload, n)
    hm = O.HostMesh(n, n, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st, "fast")
    L = O.lib("fast")
    out = (O.ctypes.c_double * 2)()

    def one(tt):
        O.step(hm, st, tt, "fast")
        L.flow_oracle_conservation(hm.nx, hm.ny, O.PAD, O.ptr(st["rho"]), O.ptr(st["e"]),
                                   O.ctypes.cast(out, O.ctypes.POINTER(O.ctypes.c_double)))

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
    return n * n * timed / el, timed, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    value, timed, threads = cpu_run(args.size, args.steps, args.warmup, budget_s=150.0,
                                    workload=args.workload)
    sample = (f"{args.workload} {args.size}^2 FP64 timesteps on {threads} host threads: "
              f"{timed} of {args.steps} requested steps timed after {args.warmup} warm-up")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": args.size * args.size / value * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}_{args.size}_fp64", "nx": args.size, "ny": args.size,
                   "form": "fp64", "parallelism": "host OpenMP"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side.

B_ALG_MIXED = 48  # rho, e (FP64) and rho_u, rho_v (FP32), each read + written


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
    """Config 3 (kind "two_region"): 256 two-region instances with sides drawn
    from {128, 192, ..., 1024}; config 4 (kind "smooth"): 64 instances of
    2048^2 smooth random fields.  Seeded."""
    import numpy as np
    if kind == "two_region":
        rng = np.random.default_rng(20261203)
        sides = rng.choice(np.arange(128, 1025, 64), size=256)
        return [problems.two_region(int(n), rng) for n in sides]
    rng = np.random.default_rng(20261204)
    return [problems.smooth_random(2048, rng) for _ in range(64)]


def run_batched_form(fg, problems, torch, device, kind, precision, steps, warmup):
    """Times one batched ensemble (autotuned, graph-replayed) and measures its
    error on two sampled instances against the single-problem FP64 step."""
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
    errs = {}
    for i in samples:
        rho, e, dt, _ = b.state(i)
        ref = fg.DeviceSim(probs[i], device)
        ref.initial_timestep()
        ref.run(total_steps)
        rr, er = ref.interior("rho"), ref.interior("e")
        errs[f"instance_{i}_{probs[i].gnx}x{probs[i].gny}"] = {
            "rho_l1": float(np.abs(rho - rr).sum() / np.abs(rr).sum()),
            "e_l1": float(np.abs(e - er).sum() / np.abs(er).sum()),
            "rho_linf": float(np.abs(rho - rr).max() / np.abs(rr).max()),
            "max_abs_diff": float(max(np.abs(rho - rr).max(), np.abs(e - er).max()))}
        del ref
    del b
    torch.cuda.empty_cache()
    seq = run_sequential_ensemble(fg, torch, device, probs, precision, warmup=1, steps=2)
    b_alg = B_ALG_FP64 if precision == 0 else B_ALG_MIXED
    return {"workload": f"batch_{kind}_{'fp64' if precision == 0 else 'mixed'}",
            "instances": len(probs), "cells": cells, "value": value, "unit": UNIT,
            "ms_per_step": ms / steps, "steps_timed": steps, "steps_total": total_steps,
            "graph": True, "tuning": tune,
            "hbm_fraction_of_step": value * b_alg / (measured_peaks()[0] * 1e9),
            "errors_vs_fp64_single_problem": errs,
            "sequential_same_ensemble": seq,
            "speedup_vs_sequential": value / seq["value"]}


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


def run_fp64_smooth(fg, problems, torch, device, n, steps, warmup):
    """The FP64 step on a field with structure everywhere (density and energy
    1 + a 16-mode smooth random field, seed 20261205): no flat regions, so
    every slope and limiter is live -- the general-case rate next to the
    blast problem, most of whose mesh is still at rest."""
    import numpy as np
    sim = fg.DeviceSim(problems.smooth_random(n, np.random.default_rng(20261205)), device)
    sim.initial_timestep()
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
    ms = e0.elapsed_time(e1)
    del sim
    torch.cuda.empty_cache()
    return {"workload": f"smooth_{n}_fp64", "value": n * n * steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup}


def run_mixed_form(fg, problems, torch, device, n, steps, warmup, ref_state=None, workload="sedov"):
    """Times the mixed form on the same workload; returns its result dict and
    the final simulation object."""
    prob = problems.sedov(n) if workload == "sedov" else problems.sod(n)
    sim = fg.MixedSim(prob, device)
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
    ms = e0.elapsed_time(e1)
    value = n * n * steps / (ms * 1e-3)
    return {"workload": f"{workload}_{n}_mixed", "value": value, "unit": UNIT,
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup,
            "hbm_fraction_of_step_48B": value * B_ALG_MIXED / (measured_peaks()[0] * 1e9)}, sim

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
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
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
    launches = fg.ctypes.c_longlong()
    tot = fg.ctypes.c_double()
    for i in range(L.gb300_profile_count()):
        L.gb300_profile_entry(i, buf, 64, fg.ctypes.byref(launches), fg.ctypes.byref(tot))
        kernels.append((buf.value.decode(), launches.value, tot.value))
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
    del host_in, host_out

    # ---- the mixed-precision form on the same workload ----
    forms = {}
    if not args.fp64_only:
        del sim, sim2
        torch.cuda.empty_cache()
        if args.workload != "smooth":
            forms["fp64_smooth"] = run_fp64_smooth(fg, problems, torch, device, n,
                                                   min(args.steps, 100), args.warmup)
        # The mixed form on the FP64 workload, then on the 8192^2 Sod tube.
        for workload, size in (("sedov", n), ("sod", args.sod_size)):
            if size <= 0:
                continue
            mixed, msim = run_mixed_form(fg, problems, torch, device, size, args.steps,
                                         args.warmup, workload=workload)
            # Error against the FP64 path after the same number of steps from
            # the same initial state (the FP64 path itself matches the CPU
            # oracle to ~1e-13 per cell).
            prob_ref = problems.sedov(size) if workload == "sedov" else problems.sod(size)
            ref = fg.DeviceSim(prob_ref, device)
            ref.initial_timestep()
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record()
            ref.run(args.steps + args.warmup)
            t1.record()
            torch.cuda.synchronize()
            fp64_value = size * size * (args.steps + args.warmup) / (t0.elapsed_time(t1) * 1e-3)
            mixed["errors_vs_fp64"] = field_errors(fg, msim, ref,
                                                   names=("rho", "e", "u", "v", "rho_u", "rho_v"))
            cm, cr = msim.conservation(), ref.conservation()
            mixed["mass_drift"] = abs(cm[0] - cr[0]) / cr[0]
            mixed["energy_drift"] = abs(cm[1] - cr[1]) / cr[1]
            mixed["fp64_value_same_workload"] = fp64_value
            mixed["speedup_vs_fp64"] = mixed["value"] / fp64_value
            forms["mixed" if workload == "sedov" else f"mixed_sod_{size}"] = mixed
            del msim, ref
            torch.cuda.empty_cache()
        bsteps = min(args.steps, args.batch_steps)
        forms["batched_fp64"] = run_batched_form(fg, problems, torch, device, "two_region", 0,
                                                 bsteps, args.warmup)
        forms["batched_mixed"] = run_batched_form(fg, problems, torch, device, "smooth", 1,
                                                  bsteps, args.warmup)

    if rank != 0:
        return

    # ---- roofline of the dominant kernel and of the FP64 pipe ----
    peak, peak_kind = measured_peaks()
    name, nl, total = kernels[0] if kernels else ("none", 1, float("nan"))
    cells = (nx - 4) * (ny - 4)
    bytes_launch = KERNEL_BYTES_PER_CELL.get(name, B_ALG_FP64) * cells
    achieved = bytes_launch / (total / nl * 1e-3) / 1e9
    tb = NCU_TRAFFIC_BYTES_PER_CELL.get(name)
    traffic = tb * cells if tb is not None else None
    fma_rate = fg.ctypes.c_double()
    L.gb300_measure_fp64_fma_rate(fg.ctypes.byref(fma_rate))

    cpu = None
    if not args.no_cpu_baseline:
        cv, timed, threads = cpu_run(n, 64, 1, budget_s=20.0, workload=args.workload)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.workload} {n}^2 FP64, {timed} timesteps on {threads} host threads "
                         "(C restatement of the reference omp3 set, OpenMP)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}_{n}_fp64", "nx": n, "ny": n, "form": "fp64",
                   "iterations_timed": args.steps, "l2": "inputs larger than L2 (2.3 GB state)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "hbm_fraction_of_step": value / world * B_ALG_FP64 / (peak * 1e9)},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps + 32,
                "what": "initial state H2D from pinned host, K timesteps + conservation readback "
                        "through the C ABI, final state D2H"},
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind},
        "fp64_pipe": {"fma_per_s_peak": fma_rate.value,
                      "note": "FP64 issue rate measured on this GPU; the FP64 timestep is bound here"},
        # Per kernel: launches, total ms, share of the step, and its achieved
        # GB/s on its algorithmic bytes (KERNEL_BYTES_PER_CELL) with the
        # fraction of the measured HBM copy bandwidth.
        "kernels": [{"name": k, "launches": c, "ms": t, "share": t / sum(x[2] for x in kernels),
                     "alg_gbs": KERNEL_BYTES_PER_CELL.get(k, B_ALG_FP64) * cells / (t / c * 1e-3) / 1e9,
                     "alg_frac": KERNEL_BYTES_PER_CELL.get(k, B_ALG_FP64) * cells
                                 / (t / c * 1e-3) / 1e9 / peak}
                    for k, c, t in kernels],
        "forms": forms,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": 12 * args.steps,  # mesh test + 10 timestep kernels + the conservation totals
        "mass": mass, "energy": energy,
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
