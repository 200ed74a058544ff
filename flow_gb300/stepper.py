"""Runs the fused timestep of one problem on the GPU and reports its speed.

    python -m flow_gb300.stepper --size 4096 --workload sedov --form fp64 \
        --steps 500 --warmup 5 [--no-profile]

Prints one JSON line (milliseconds per step and cell-steps/s over the timed
steps, CUDA events on the current stream) and, unless --no-profile, the time
of each kernel of the step from the library's per-kernel event profile.
Workloads: "sedov" (the blast of the benchmark), "sod" (a tube split at
x = 0.5), "smooth" (density and energy 1 + a 16-mode smooth random field,
seed 20261205).  Forms: "fp64" (solve_hydro_2d in the fused mode),
"fp64lag" (the same with the one-kernel Lagrangian phase) and "mixed"
(gb300_mixed_solve).  Small runs of this module are what the ncu
captures of the kernels profile.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def make_problem(problems, workload: str, n: int):
    if workload == "sedov":
        return problems.sedov(n)
    if workload == "sod":
        return problems.sod(n)
    return problems.smooth_random(n, np.random.default_rng(20261205))


def main(argv=None) -> None:
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--size", type=int, default=4096)
    p.add_argument("--workload", choices=["sedov", "sod", "smooth"], default="sedov")
    p.add_argument("--form", choices=["fp64", "fp64lag", "mixed"], default="fp64")
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--no-profile", action="store_true")
    args = p.parse_args(argv)

    import torch

    import flow_gb300 as fg
    from flow_gb300 import problems

    L = fg.lib()
    fg.set_stream(torch.cuda.current_stream())
    fg.set_mode(fg.MODE_FUSED_LAG if args.form == "fp64lag" else fg.MODE_FUSED)
    prob = make_problem(problems, args.workload, args.size)
    if args.form == "mixed":
        sim = fg.MixedSim(prob, "cuda:0")
    else:
        sim = fg.DeviceSim(prob, "cuda:0")
        sim.initial_timestep()
    for _ in range(args.warmup):
        sim.step()
    torch.cuda.synchronize()
    if not args.no_profile:
        L.gb300_profile_reset()
        L.gb300_profile_enable(1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        sim.step()
    e1.record()
    torch.cuda.synchronize()
    L.gb300_profile_enable(0)
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    print(json.dumps({"size": args.size, "workload": args.workload, "form": args.form,
                      "steps": args.steps, "ms_per_step": ms,
                      "cell_steps_per_s": args.size * args.size / (ms * 1e-3)}))
    if args.no_profile:
        return
    buf = fg.ctypes.create_string_buffer(64)
    n = fg.ctypes.c_longlong()
    t = fg.ctypes.c_double()
    rows = []
    for i in range(L.gb300_profile_count()):
        L.gb300_profile_entry(i, buf, 64, fg.ctypes.byref(n), fg.ctypes.byref(t))
        rows.append((buf.value.decode(), n.value, t.value))
    total = sum(r[2] for r in rows) or 1.0
    for name, count, tms in sorted(rows, key=lambda r: -r[2]):
        print(f"  {name:20s} {count:6d} {tms / max(1, args.steps) * 1e3:9.1f} us/step "
              f"{100 * tms / total:5.1f}%")


if __name__ == "__main__":
    main()
