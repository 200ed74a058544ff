"""Single-mesh domain decomposition of the flow timestep over ranks.

The reference decomposes one mesh over MPI ranks through its arch layer
(Makefile:47-59, DECOMP=ROWS|COLS|TILES): every rank holds a band of the mesh
with pad ghost layers, exchanges those layers with its neighbours inside each
handle_boundary_2d(..., PACK) (19 per step, e.g. omp3/flow.c:156-157), and
reduces the CFL minimum with reduce_all_min (omp3/flow.c:100).  Here the mesh
is split into bands of rows (DECOMP=ROWS); a rank's Mesh names its
neighbours (FLOW_SOUTH = the band below, FLOW_NORTH = the band above), and the
kernel set calls two hooks this module provides (gb300_set_halo_exchange,
gb300_set_reduce_min) with one of two transports:

* DistTransport  -- torch.distributed point-to-point and all-reduce: one
  process per rank (gloo on host arrays, NCCL on device arrays);
* ThreadTransport -- ranks as threads of one process sharing one GPU; the
  threads meet on the host between kernel launches (no kernel waits on
  another), which tests the decomposed GPU path on a single GPU.

A ghost layer is filled with the single-rank step's value at the same place of
the mesh, so a decomposed run matches the single-rank run bit for bit.  For a
cell or x-face array (h = local_ny rows) the ghost rows below a rank are the
last pad interior rows of the band below, the ghost rows above it the first
pad interior rows of the band above.  A y-face array has h = local_ny + 1
rows and the face between two bands is interior to both (each computes it
from the same values), so its ghost rows are shifted by one: the rows below
take the band below's rows ny' - 2 pad .. ny' - pad - 1 and the rows above
take the band above's rows pad + 1 .. 2 pad.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from .problems import PAD, Problem

FLOW_EDGE = -1
FLOW_NORTH, FLOW_EAST, FLOW_SOUTH, FLOW_WEST = 0, 1, 2, 3

HALO_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_int, ctypes.c_int, ctypes.c_int)
MIN_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double))


def row_bands(gny: int, nranks: int) -> list[tuple[int, int]]:
    """(first interior row, rows) of each rank's band, as even as possible."""
    if nranks < 1:
        raise ValueError("need at least one rank")
    base, extra = divmod(gny, nranks)
    if base < 2 * PAD:
        raise ValueError(f"{gny} rows over {nranks} ranks leaves a band under {2 * PAD} rows")
    out, off = [], 0
    for r in range(nranks):
        n = base + (1 if r < extra else 0)
        out.append((off, n))
        off += n
    return out


def neighbours(rank: int, nranks: int) -> list[int]:
    """Mesh.neighbours of a rank of a row decomposition (N, E, S, W)."""
    nb = [FLOW_EDGE] * 4
    if rank > 0:
        nb[FLOW_SOUTH] = rank - 1
    if rank < nranks - 1:
        nb[FLOW_NORTH] = rank + 1
    return nb


class BandProblem(Problem):
    """The band of a global problem that one rank holds: its interior rows,
    with the global mesh's spacings and face positions (so that the
    arithmetic sees the same numbers as the single-rank run)."""

    def __init__(self, prob: Problem, y_off: int, rows: int):
        super().__init__(prob.gnx, rows, width=prob.width, height=prob.height,
                         dt_param=prob.dt_param, max_dt=prob.max_dt, sim_end=prob.sim_end)
        self.global_problem = prob
        self.y_off = y_off
        g = prob.interior
        self.fields(g(prob.rho)[y_off:y_off + rows], g(prob.e)[y_off:y_off + rows])

    @property
    def edgey(self):
        g = self.global_problem
        return g.height * (np.arange(self.ny + 1, dtype=np.float64) + self.y_off - PAD) / g.gny

    @property
    def edgedy(self):
        g = self.global_problem
        return np.full(self.ny + 1, g.height / g.gny)

    @property
    def celldy(self):
        return self.edgedy


def halo_rows(h: int, local_ny: int, side: int) -> tuple[slice, slice]:
    """(rows sent to the neighbour on `side`, rows received from it) of an
    array of h rows on a rank whose cell arrays have local_ny rows."""
    yface = 1 if h == local_ny + 1 else 0
    if side == FLOW_SOUTH:
        return slice(PAD + yface, 2 * PAD + yface), slice(0, PAD)
    if side == FLOW_NORTH:
        return slice(h - 2 * PAD - yface, h - PAD - yface), slice(h - PAD, h)
    raise ValueError("row decomposition: only north and south neighbours")


class DistTransport:
    """Halo and minimum exchange over torch.distributed (the default process
    group): isend/irecv of the boundary rows, all_reduce(MIN) of the CFL
    minimum.  Host arrays go through CPU tensors (gloo), device tensors stay
    on the device (NCCL)."""

    def exchange(self, rank, sends: dict, recv_like: dict) -> dict:
        import torch
        import torch.distributed as dist
        reqs, got = [], {}
        for nb, buf in sends.items():
            t = buf if isinstance(buf, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(buf))
            reqs.append(dist.isend(t.contiguous(), nb))
        for nb, like in recv_like.items():
            t = torch.empty_like(like) if isinstance(like, torch.Tensor) else \
                torch.empty(like.shape, dtype=torch.float64)
            got[nb] = t
            reqs.append(dist.irecv(t, nb))
        for r in reqs:
            r.wait()
        return got

    def min(self, rank, value: float) -> float:
        import torch
        import torch.distributed as dist
        t = torch.tensor([value], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MIN)
        return float(t.item())


class ThreadTransport:
    """Ranks as threads of one process: each exchange posts the rank's rows
    in a mailbox and waits (on the host, with a time limit) for its
    neighbours'; the minimum is reduced through a barrier."""

    def __init__(self, nranks: int, timeout: float = 60.0):
        self.n = nranks
        self.timeout = timeout
        self.cv = threading.Condition()
        self.box = {}
        self.seq = [0] * nranks
        self.mins = {}
        self.min_seq = [0] * nranks

    def exchange(self, rank, sends: dict, recv_like: dict) -> dict:
        with self.cv:
            k = self.seq[rank]
            self.seq[rank] += 1
            for nb, buf in sends.items():
                self.box[(k, rank, nb)] = buf.clone() if hasattr(buf, "clone") else buf.copy()
            self.cv.notify_all()
            keys = [(k, nb, rank) for nb in recv_like]
            if not self.cv.wait_for(lambda: all(key in self.box for key in keys), self.timeout):
                raise TimeoutError(f"rank {rank}: halo exchange {k} timed out")
            return {key[1]: self.box.pop(key) for key in keys}

    def min(self, rank, value: float) -> float:
        with self.cv:
            k = self.min_seq[rank]
            self.min_seq[rank] += 1
            self.mins.setdefault(k, {})[rank] = value
            self.cv.notify_all()
            if not self.cv.wait_for(lambda: len(self.mins[k]) == self.n, self.timeout):
                raise TimeoutError(f"rank {rank}: minimum {k} timed out")
            return min(self.mins[k].values())


class RankContext:
    """What the hooks need to know about the calling rank: its number, its
    Mesh (for neighbours and local_ny), how to find the array behind a
    pointer, and the transport."""

    def __init__(self, rank: int, nranks: int, transport, resolve):
        self.rank = rank
        self.nranks = nranks
        self.transport = transport
        self.resolve = resolve  # (address, w, h) -> 2-D array view (h, w)


class Hooks:
    """ctypes callbacks for a library's halo and minimum hooks.  The calling
    rank is found per thread (ThreadTransport) or is the process's only rank
    (DistTransport): register it with bind()."""

    def __init__(self, mesh_type):
        self.mesh_type = mesh_type
        self.local = threading.local()
        self.halo = HALO_FN(self._halo)
        self.min = MIN_FN(self._min)
        self.errors = []

    def bind(self, ctx: RankContext) -> None:
        self.local.ctx = ctx

    def _halo(self, _user, mesh_p, arr_p, w, h, invert):
        try:
            ctx = self.local.ctx
            mesh = ctypes.cast(mesh_p, ctypes.POINTER(self.mesh_type)).contents
            arr = ctx.resolve(arr_p, w, h)
            sends, likes, recv_rows = {}, {}, {}
            for side in (FLOW_SOUTH, FLOW_NORTH):
                nb = mesh.neighbours[side]
                if nb == FLOW_EDGE:
                    continue
                send, recv = halo_rows(h, mesh.local_ny, side)
                sends[nb] = arr[send]
                likes[nb] = arr[recv]
                recv_rows[nb] = recv
            got = ctx.transport.exchange(ctx.rank, sends, likes)
            for nb, rows in recv_rows.items():
                src = got[nb]
                if hasattr(arr, "copy_"):
                    import torch
                    src = src if isinstance(src, torch.Tensor) else torch.from_numpy(src)
                    arr[rows].copy_(src.to(arr.device))
                else:
                    arr[rows] = np.asarray(src)
            return 0
        except Exception as exc:  # reported through the library's status
            self.errors.append(repr(exc))
            return 1

    def _min(self, _user, value_p):
        try:
            ctx = self.local.ctx
            value_p[0] = ctx.transport.min(ctx.rank, float(value_p[0]))
            return 0
        except Exception as exc:
            self.errors.append(repr(exc))
            return 1


def numpy_resolver(arrays: dict):
    """Address -> (h, w) view of the host arrays (numpy) of one rank."""
    by_addr = {a.ctypes.data: a for a in arrays.values()}

    def resolve(addr, w, h):
        a = by_addr[addr]
        return a[: w * h].reshape(h, w)
    return resolve


def torch_resolver(arrays: dict):
    """Address -> (h, w) view of the device tensors of one rank."""
    by_addr = {t.data_ptr(): t for t in arrays.values()}

    def resolve(addr, w, h):
        t = by_addr[addr]
        return t[: w * h].view(h, w)
    return resolve


def set_rank_mesh(mesh, rank: int, nranks: int, y_off: int) -> None:
    """Marks a Mesh (ctypes) as one band of a row decomposition."""
    mesh.rank, mesh.nranks, mesh.y_off = rank, nranks, y_off
    for k, v in enumerate(neighbours(rank, nranks)):
        mesh.neighbours[k] = v


class DecomposedSim:
    """One rank's band of a global problem on the GPU, stepped by the kernel
    set's exact mode with its ghost layers exchanged through `hooks`.  The
    initial ghost fill (main.c:56-59) and the driver's first set_timestep
    (main.c:64-66) are the decomposed ones, so every rank of a job must
    construct its DecomposedSim (they exchange halos) and step together."""

    def __init__(self, prob: Problem, rank: int, nranks: int, transport, hooks: Hooks,
                 device: str = "cuda:0"):
        from . import check, dptr, lib, sim
        y_off, rows = row_bands(prob.gny, nranks)[rank]
        self.band = BandProblem(prob, y_off, rows)
        self.y_off, self.rows = y_off, rows
        self.sim = sim.DeviceSim(self.band, device)
        set_rank_mesh(self.sim.mesh, rank, nranks, y_off)
        hooks.bind(RankContext(rank, nranks, transport, torch_resolver(self.sim.a)))
        L = lib()
        for f in ("rho", "e"):
            L.handle_boundary_2d(self.sim.nx, self.sim.ny, ctypes.byref(self.sim.mesh),
                                 dptr(self.sim.a[f]), 0, 1)
        check()

    def initial_timestep(self) -> None:
        self.sim.initial_timestep()

    def step(self) -> None:
        self.sim.step()

    def interior(self, name: str) -> np.ndarray:
        """The band's interior rows of a field (a y-face field also gets the
        face above the band only on the last rank, as in the global layout)."""
        a = self.sim.interior(name)
        if name in ("v", "rho_v", "F_y") and self.sim.mesh.neighbours[FLOW_NORTH] != FLOW_EDGE:
            return a[:-1]
        return a


def _declare(lib) -> None:
    for name in ("gb300_set_halo_exchange", "gb300_set_reduce_min"):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        fn.restype = ctypes.c_int


def install(lib, hooks: Hooks) -> None:
    """Registers the hooks with the kernel set (keep `hooks` alive)."""
    _declare(lib)
    if lib.gb300_set_halo_exchange(ctypes.cast(hooks.halo, ctypes.c_void_p), None) != 0 or \
            lib.gb300_set_reduce_min(ctypes.cast(hooks.min, ctypes.c_void_p), None) != 0:
        raise RuntimeError("could not register the decomposition hooks")


def uninstall(lib) -> None:
    """Clears the hooks (decomposed meshes are then rejected)."""
    _declare(lib)
    lib.gb300_set_halo_exchange(None, None)
    lib.gb300_set_reduce_min(None, None)
