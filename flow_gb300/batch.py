"""Batched ensembles of independent flow problems (C ABI Part 4).

A Batch owns one device pool (a PyTorch byte tensor) into which the library
lays out every instance's arrays; instances of different sizes advance
together, each with its own dt: one launch per phase of the timestep over
every instance's tiles, or one persistent kernel launch per timestep
(set_schedule), captured two steps at a time as a CUDA graph.
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import GB300_OK, FlowError, check, lib
from .problems import Problem

BATCH_PHASES = 0      # include/flow_gb300.h GB300_BATCH_PHASES
BATCH_PERSISTENT = 1  # GB300_BATCH_PERSISTENT

_TUNE_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tuning_cache.json")


class Batch:
    def __init__(self, problems: list[Problem], precision: int = 0, device: str = "cuda:0"):
        import torch
        if not torch.cuda.is_available():
            raise FlowError("flow_gb300 needs a CUDA device (no CPU fallback)")
        self.torch = torch
        self.problems = problems
        self.precision = precision
        n = len(problems)
        L = lib()
        gnx = (ctypes.c_int * n)(*[p.gnx for p in problems])
        gny = (ctypes.c_int * n)(*[p.gny for p in problems])
        w = (ctypes.c_double * n)(*[p.width for p in problems])
        h = (ctypes.c_double * n)(*[p.height for p in problems])
        handle = ctypes.c_void_p()
        if L.gb300_batch_create(n, gnx, gny, w, h, precision, ctypes.byref(handle)) != GB300_OK:
            check()
        self.handle = handle
        self.bytes = int(L.gb300_batch_pool_bytes(handle))
        self.pool = torch.empty(self.bytes, dtype=torch.uint8, device=device)
        if L.gb300_batch_bind(handle, ctypes.c_void_p(self.pool.data_ptr()), self.bytes) != GB300_OK:
            check()
        from . import boxes_array
        for i, p in enumerate(problems):
            if p.box_list is not None:
                # Problem boxes are rasterised on the device: no host fields.
                st = L.gb300_batch_fill_boxes(handle, i, boxes_array(p.box_list),
                                              len(p.box_list), p.dt_param)
            else:
                rho = np.ascontiguousarray(p.interior(p.rho), dtype=np.float64)
                e = np.ascontiguousarray(p.interior(p.e), dtype=np.float64)
                st = L.gb300_batch_set_state(handle, i,
                                             rho.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             p.dt_param)
            if st != GB300_OK:
                check()
        torch.cuda.synchronize()
        self.steps_done = 0

    @property
    def cells(self) -> int:
        return int(lib().gb300_batch_cells(self.handle))

    def tuning(self) -> dict:
        r, c, o, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().gb300_batch_get_tuning(self.handle, ctypes.byref(r), ctypes.byref(c), ctypes.byref(o),
                                     ctypes.byref(g))
        return {"rows": r.value, "ctas_per_sm": c.value, "order": o.value, "grid": g.value}

    def set_tuning(self, rows: int, ctas_per_sm: int, order: int) -> None:
        if lib().gb300_batch_set_tuning(self.handle, rows, ctas_per_sm, order) != GB300_OK:
            check()

    def set_schedule(self, schedule: int) -> None:
        """BATCH_PHASES (one launch per phase over every instance's tiles) or
        BATCH_PERSISTENT (one cooperative launch per step)."""
        if lib().gb300_batch_set_schedule(self.handle, schedule) != GB300_OK:
            check()

    @property
    def schedule(self) -> int:
        return int(lib().gb300_batch_get_schedule(self.handle))

    def step(self, steps: int = 1, use_graph: bool = True) -> None:
        if lib().gb300_batch_step(self.handle, steps, int(use_graph)) != GB300_OK:
            check()
        self.steps_done += steps

    def set_spin_limit(self, spins: int) -> None:
        """Bound of each grid-barrier wait, in 64 ns naps (default 2**25)."""
        if lib().gb300_batch_set_spin_limit(self.handle, spins) != GB300_OK:
            check()

    def status_code(self) -> int:
        """The status word after the steps so far (synchronises): GB300_OK,
        or GB300_ERR_TIMEOUT when a grid barrier ran out (the barrier state is
        then cleared, so the batch can be stepped again)."""
        return int(lib().gb300_batch_status(self.handle))

    def status(self) -> None:
        if lib().gb300_batch_status(self.handle) != GB300_OK:
            check()

    def state(self, i: int):
        p = self.problems[i]
        rho = np.empty((p.gny, p.gnx))
        e = np.empty((p.gny, p.gnx))
        dt = (ctypes.c_double * 2)()
        tot = (ctypes.c_double * 2)()
        dp = ctypes.POINTER(ctypes.c_double)
        if lib().gb300_batch_get_state(self.handle, i, rho.ctypes.data_as(dp), e.ctypes.data_as(dp),
                                       ctypes.cast(dt, dp), ctypes.cast(tot, dp)) != GB300_OK:
            check()
        return rho, e, (dt[0], dt[1]), (tot[0], tot[1])

    def autotune(self, candidates=None, steps: int = 2, cache: bool = True) -> dict:
        """Times each (schedule, rows, ctas_per_sm, order) candidate for
        `steps` timesteps (these steps advance the ensemble, like warm-up
        steps) and keeps the fastest; the choice is cached per GPU and batch
        signature.  ctas_per_sm only applies to the persistent schedule."""
        torch = self.torch
        key = self._signature()
        if cache and os.path.exists(_TUNE_CACHE):
            try:
                with open(_TUNE_CACHE) as f:
                    got = json.load(f).get(key)
                if got and "schedule" in got:
                    self.set_schedule(got["schedule"])
                    self.set_tuning(got["rows"], got["ctas_per_sm"], got["order"])
                    return {"cached": True, **got}
            except (OSError, ValueError):
                pass
        candidates = candidates or (
            [(BATCH_PHASES, r, 0, o) for r in (8, 16, 32) for o in (0, 1)]
            + [(BATCH_PERSISTENT, r, c, o) for r in (8, 16, 32) for c in (0, 2) for o in (0, 1)])
        results = []
        for (sc, r, c, o) in candidates:
            self.set_schedule(sc)
            self.set_tuning(r, c, o)
            self.step(2, use_graph=False)  # warm the variant
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            self.step(steps, use_graph=False)
            torch.cuda.synchronize()
            results.append((time.perf_counter() - t0, sc, r, c, o))
        results.sort()
        _, sc, r, c, o = results[0]
        self.set_schedule(sc)
        self.set_tuning(r, c, o)
        best = {"schedule": sc, "rows": r, "ctas_per_sm": c, "order": o,
                "ms_per_step": results[0][0] / steps * 1e3,
                "tried": [{"schedule": ss, "rows": rr, "ctas_per_sm": cc, "order": oo,
                           "ms_per_step": t / steps * 1e3}
                          for (t, ss, rr, cc, oo) in results]}
        if cache:
            data = {}
            if os.path.exists(_TUNE_CACHE):
                try:
                    with open(_TUNE_CACHE) as f:
                        data = json.load(f)
                except (OSError, ValueError):
                    data = {}
            data[key] = {"rows": r, "ctas_per_sm": c, "order": o}
            with open(_TUNE_CACHE, "w") as f:
                json.dump(data, f, indent=1)
        return {"cached": False, **best}

    def _signature(self) -> str:
        name = self.torch.cuda.get_device_name()
        sizes = sorted((p.gnx, p.gny) for p in self.problems)
        return f"{name}|p{self.precision}|n{len(sizes)}|cells{sum(a * b for a, b in sizes)}|max{sizes[-1]}"

    def __del__(self):
        try:
            lib().gb300_batch_destroy(self.handle)
        except Exception:
            pass
