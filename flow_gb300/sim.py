"""Device-resident state of one problem, driven through the C ABI.

Mirrors the reference host (main.c:17-115): the same arrays, the same
initial ghost fill (main.c:56-59), the same initial ``set_timestep`` with
``first_step = 0`` (main.c:64-66) and one ``solve_hydro_2d`` per iteration
(main.c:82-88).  Device memory comes from PyTorch; all compute is the kernel
set's.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import GB300_OK, FlowError, Mesh, check, dptr, lib
from .problems import C_T, PAD, Problem

CELL_FIELDS = ("P", "rho", "rho_old", "e", "Qxx", "Qyy", "reduce")
FACE_FIELDS = ("u", "v", "rho_u", "rho_v", "F_x", "F_y", "uF_x", "uF_y", "vF_x", "vF_y")
# Argument order of solve_hydro_2d after (mesh, tt), flow_interface.h:16-20.
SOLVE_ORDER = ("P", "rho", "rho_old", "e", "u", "v", "rho_u", "rho_v", "Qxx", "Qyy",
               "F_x", "F_y", "uF_x", "uF_y", "vF_x", "vF_y", "reduce")


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise FlowError("flow_gb300 needs a CUDA device (no CPU fallback)")
    return torch


class DeviceSim:
    """All arrays of one problem on one GPU plus its ``Mesh``."""

    def __init__(self, prob: Problem, device: str = "cuda:0"):
        torch = _torch()
        self.torch = torch
        self.prob = prob
        self.device = torch.device(device)
        nx, ny = prob.nx, prob.ny
        self.nx, self.ny = nx, ny
        f64 = dict(dtype=torch.float64, device=self.device)
        self.a = {}
        for f in CELL_FIELDS:
            self.a[f] = torch.zeros(nx * ny, **f64)
        for f in FACE_FIELDS:
            self.a[f] = torch.zeros((nx + 1) * (ny + 1), **f64)
        self.mesh_arrays = {k: torch.from_numpy(np.ascontiguousarray(getattr(prob, k))).to(self.device)
                            for k in ("edgex", "edgey", "edgedx", "edgedy", "celldx", "celldy")}
        m = Mesh()
        m.global_nx, m.global_ny = prob.gnx, prob.gny
        m.local_nx, m.local_ny = nx, ny
        m.pad, m.x_off, m.y_off, m.rank, m.nranks = PAD, 0, 0, 0, 1
        for i in range(4):
            m.neighbours[i] = -1
        m.width, m.height = prob.width, prob.height
        m.max_dt, m.sim_end = prob.max_dt, prob.sim_end
        m.dt = C_T * prob.dt_param
        m.dt_h = m.dt
        for k, t in self.mesh_arrays.items():
            setattr(m, k, dptr(t))
        self.mesh = m
        self._mesh_ref = ctypes.byref(m)
        self._solve = lib().gb300_solve_hydro_2d
        self._args = None
        self.tt = 0
        if prob.box_list is not None:
            self.fill_boxes(prob.box_list)
        else:
            self.upload(prob.rho, prob.e)

    # -- state transfer -----------------------------------------------------
    def upload(self, rho: np.ndarray, e: np.ndarray) -> None:
        """Copies padded density/energy to the device and fills their ghosts
        (main.c:56-59)."""
        torch = self.torch
        n = self.nx * self.ny
        self.a["rho"].copy_(torch.from_numpy(np.ascontiguousarray(rho, dtype=np.float64).reshape(n)))
        self.a["e"].copy_(torch.from_numpy(np.ascontiguousarray(e, dtype=np.float64).reshape(n)))
        L = lib()
        for f in ("rho", "e"):
            L.handle_boundary_2d(self.nx, self.ny, ctypes.byref(self.mesh), dptr(self.a[f]), 0, 1)
        check()

    def fill_boxes(self, boxes) -> None:
        """Rasterises problem boxes on the device (gb300_fill_boxes) and fills
        the ghosts (main.c:52-59)."""
        from . import boxes_array
        L = lib()
        if L.gb300_fill_boxes(self.nx, self.ny, self.mesh.edgex, self.mesh.edgey,
                              boxes_array(boxes), len(boxes), dptr(self.a["rho"]),
                              dptr(self.a["e"])) != GB300_OK:
            check()
        for f in ("rho", "e"):
            L.handle_boundary_2d(self.nx, self.ny, ctypes.byref(self.mesh), dptr(self.a[f]), 0, 1)
        check()

    def host(self, name: str) -> np.ndarray:
        return self.a[name].cpu().numpy()

    def interior(self, name: str) -> np.ndarray:
        """Interior view of a state field in its own grid (cells, x- or y-faces)."""
        nx, ny, p = self.nx, self.ny, PAD
        a = self.host(name)
        if name in ("u", "rho_u", "F_x"):
            return a[: ny * (nx + 1)].reshape(ny, nx + 1)[p:ny - p, p:nx + 1 - p]
        if name in ("v", "rho_v", "F_y"):
            return a[: (ny + 1) * nx].reshape(ny + 1, nx)[p:ny + 1 - p, p:nx - p]
        return a[: nx * ny].reshape(ny, nx)[p:ny - p, p:nx - p]

    # -- the reference call sequence ----------------------------------------
    def initial_timestep(self) -> None:
        """set_timestep(first_step = 0) before the loop (main.c:64-66)."""
        L = lib()
        L.set_timestep(self.nx, self.ny, dptr(self.a["Qxx"]), dptr(self.a["Qyy"]),
                       dptr(self.a["rho"]), dptr(self.a["e"]), ctypes.byref(self.mesh),
                       dptr(self.a["reduce"]), 0, self.mesh.celldx, self.mesh.celldy)
        check()

    def args(self):
        # The arrays are allocated once, in __init__, and written in place
        # afterwards, so their pointers are formed once: a ctypes cast per
        # array per step would keep the GPU waiting on the host after every
        # step whose totals are read back.
        if self._args is None:
            self._args = tuple(dptr(self.a[f]) for f in SOLVE_ORDER)
        return self._args

    def step(self) -> None:
        st = self._solve(self._mesh_ref, self.tt, *self.args())
        if st != GB300_OK:
            check()
        self.tt += 1

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()

    def conservation(self) -> tuple[float, float]:
        out = (ctypes.c_double * 2)()
        st = lib().gb300_conservation(self.nx, self.ny, PAD, dptr(self.a["rho"]), dptr(self.a["e"]),
                                      dptr(self.a["reduce"]), ctypes.cast(out, ctypes.POINTER(ctypes.c_double)), 1)
        if st != GB300_OK:
            check()
        return float(out[0]), float(out[1])


class MixedSim:
    """One problem in the mixed-precision form: FP64 density and specific
    energy, FP32 momenta, every other array in a device workspace."""

    def __init__(self, prob: Problem, device: str = "cuda:0"):
        torch = _torch()
        self.torch = torch
        self.prob = prob
        self.device = torch.device(device)
        nx, ny = prob.nx, prob.ny
        self.nx, self.ny = nx, ny
        f64 = dict(dtype=torch.float64, device=self.device)
        f32 = dict(dtype=torch.float32, device=self.device)
        self.rho = torch.from_numpy(np.ascontiguousarray(prob.rho, dtype=np.float64).reshape(-1)).to(self.device)
        self.e = torch.from_numpy(np.ascontiguousarray(prob.e, dtype=np.float64).reshape(-1)).to(self.device)
        self.rho_u = torch.zeros((nx + 1) * (ny + 1), **f32)
        self.rho_v = torch.zeros((nx + 1) * (ny + 1), **f32)
        self.reduce = torch.zeros(nx * ny, **f64)
        L = lib()
        self.work_bytes = int(L.gb300_mixed_workspace_bytes(nx, ny))
        self.work = torch.zeros(self.work_bytes, dtype=torch.uint8, device=self.device)
        self.mesh_arrays = {k: torch.from_numpy(np.ascontiguousarray(getattr(prob, k))).to(self.device)
                            for k in ("edgex", "edgey", "edgedx", "edgedy", "celldx", "celldy")}
        m = Mesh()
        m.global_nx, m.global_ny = prob.gnx, prob.gny
        m.local_nx, m.local_ny = nx, ny
        m.pad, m.x_off, m.y_off, m.rank, m.nranks = PAD, 0, 0, 0, 1
        for i in range(4):
            m.neighbours[i] = -1
        m.width, m.height = prob.width, prob.height
        m.max_dt, m.sim_end = prob.max_dt, prob.sim_end
        m.dt = C_T * prob.dt_param
        m.dt_h = m.dt
        for k, t in self.mesh_arrays.items():
            setattr(m, k, dptr(t))
        self.mesh = m
        self.tt = 0
        for f in (self.rho, self.e):
            L.handle_boundary_2d(nx, ny, ctypes.byref(m), dptr(f), 0, 1)
        check()
        from . import vptr
        self.vptr = vptr
        if L.gb300_mixed_prepare(ctypes.byref(m), dptr(self.rho), dptr(self.e), vptr(self.work),
                                 self.work_bytes, dptr(self.reduce), 1) != GB300_OK:
            check()

    def step(self) -> None:
        L = lib()
        st = L.gb300_mixed_solve(ctypes.byref(self.mesh), self.tt, dptr(self.rho), dptr(self.e),
                                 self.vptr(self.rho_u), self.vptr(self.rho_v), self.vptr(self.work),
                                 self.work_bytes, dptr(self.reduce))
        if st != GB300_OK:
            check()
        self.tt += 1

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()

    def interior(self, name: str) -> np.ndarray:
        nx, ny, p = self.nx, self.ny, PAD
        if name in ("u", "v"):
            # FP32 velocities inside the workspace (gb300_mixed_workspace_offset).
            off = int(lib().gb300_mixed_workspace_offset(nx, ny, 0 if name == "u" else 1))
            n = (nx + 1) * (ny + 1)
            a = self.work[off:off + 4 * n].view(self.torch.float32).cpu().numpy().astype(np.float64)
            if name == "u":
                return a[: ny * (nx + 1)].reshape(ny, nx + 1)[p:ny - p, p:nx + 1 - p]
            return a[: (ny + 1) * nx].reshape(ny + 1, nx)[p:ny + 1 - p, p:nx - p]
        a = getattr(self, name).cpu().numpy().astype(np.float64)
        if name == "rho_u":
            return a[: ny * (nx + 1)].reshape(ny, nx + 1)[p:ny - p, p:nx + 1 - p]
        if name == "rho_v":
            return a[: (ny + 1) * nx].reshape(ny + 1, nx)[p:ny + 1 - p, p:nx - p]
        return a[: nx * ny].reshape(ny, nx)[p:ny - p, p:nx - p]

    def conservation(self) -> tuple[float, float]:
        out = (ctypes.c_double * 2)()
        st = lib().gb300_conservation(self.nx, self.ny, PAD, dptr(self.rho), dptr(self.e),
                                      dptr(self.reduce), ctypes.cast(out, ctypes.POINTER(ctypes.c_double)), 1)
        if st != GB300_OK:
            check()
        return float(out[0]), float(out[1])
