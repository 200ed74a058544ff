"""ORACLE TEST INFRASTRUCTURE -- ctypes access to the CPU checkers.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module.  It loads

* ``oracle/libflow_oracle.so``      -- the C restatement of the reference omp3
  kernel set (flow_oracle.c), strict IEEE evaluation;
* ``oracle/libflow_oracle_fast.so`` -- the same source with the reference's
  timed compiler flags (CPU baseline);
* ``oracle/_ref/libflow_ref.so``    -- the reference's own omp3/flow.c compiled
  against the arch shim (only where the reference sources were available).

All three export the flow_interface.h / omp3/flow.h entry points with the same
``Mesh`` layout as ``include/flow_mesh.h``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PAD = 2
GAM = 1.4
C_T = 0.3

_dp = ctypes.POINTER(ctypes.c_double)


class Mesh(ctypes.Structure):
    """Mirror of ``Mesh`` in include/flow_mesh.h."""

    _fields_ = [
        ("global_nx", ctypes.c_int), ("global_ny", ctypes.c_int),
        ("local_nx", ctypes.c_int), ("local_ny", ctypes.c_int),
        ("pad", ctypes.c_int), ("x_off", ctypes.c_int), ("y_off", ctypes.c_int),
        ("rank", ctypes.c_int), ("nranks", ctypes.c_int), ("niters", ctypes.c_int),
        ("neighbours", ctypes.c_int * 4),
        ("width", ctypes.c_double), ("height", ctypes.c_double),
        ("max_dt", ctypes.c_double), ("sim_end", ctypes.c_double),
        ("dt", ctypes.c_double), ("dt_h", ctypes.c_double),
        ("edgex", _dp), ("edgey", _dp), ("edgedx", _dp), ("edgedy", _dp),
        ("celldx", _dp), ("celldy", _dp),
    ]


_lock = threading.Lock()
_libs: dict[str, ctypes.CDLL] = {}


# The reference's source tree, where present (FLOW_REF_DIR overrides).
REF_DIR = os.environ.get("FLOW_REF_DIR", "/root/reference")


def build() -> None:
    """Compiles the C restatement (and the reference, where its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if os.path.isdir(REF_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_DIR}"], check=True)


def _load(name: str) -> ctypes.CDLL:
    with _lock:
        if name in _libs:
            return _libs[name]
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
        lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL)
        _declare(lib)
        _libs[name] = lib
        return lib


def have_reference() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libflow_ref.so"))


def have_reference_cuda() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libflow_ref_cuda.so"))


def lib(kind: str = "port") -> ctypes.CDLL:
    """``port`` (strict restatement), ``fast`` (timed flags), ``reference``
    (omp3/flow.c, strict IEEE evaluation), ``reference_default`` (omp3/flow.c
    with the reference's default -O3 -march=native flags) or
    ``reference_cuda`` (the reference's cuda set for sm_103a: the same entry
    points over device arrays)."""
    return _load({"port": "libflow_oracle.so", "fast": "libflow_oracle_fast.so",
                  "reference": os.path.join("_ref", "libflow_ref.so"),
                  "reference_default": os.path.join("_ref", "libflow_ref_default.so"),
                  "reference_cuda": os.path.join("_ref", "libflow_ref_cuda.so")}[kind])


def _declare(lib: ctypes.CDLL) -> None:
    I, D, P, M = ctypes.c_int, ctypes.c_double, _dp, ctypes.POINTER(Mesh)
    sig = {
        "solve_hydro_2d": [M, I] + [P] * 17,
        "equation_of_state": [I, I, P, P, P],
        "set_timestep": [I, I, P, P, P, P, M, P, I, P, P],
        "pressure_acceleration": [I, I, M, D, P, P, P, P, P, P, P, P, P, P],
        "artificial_viscosity": [I, I, M, D, P, P, P, P, P, P, P, P, P, P, P],
        "shock_heating_and_work": [I, I, M, D, P, P, P, P, P, P, P, P, P],
        "advect_mass_and_energy": [I, I, M, I, D, D] + [P] * 13,
        "x_mass_and_energy_flux": [I, I, I, M, D, D] + [P] * 10,
        "y_mass_and_energy_flux": [I, I, I, M, D, D] + [P] * 10,
        "advect_momentum": [I, I, I, M, D, D] + [P] * 15,
        "momentum_x_flux_in_x": [I, I, M, D, P, P, P, P, P, P],
        "momentum_x_flux_in_y": [I, I, M, D, P, P, P, P, P, P, P],
        "momentum_y_flux_in_x": [I, I, M, D, P, P, P, P, P, P, P],
        "momentum_y_flux_in_y": [I, I, M, D, P, P, P, P, P, P],
        "print_conservation": [I, I, P, P, P, M],
        "handle_boundary_2d": [I, I, M, P, I, I],
    }
    for name, args in sig.items():
        if not hasattr(lib, name):  # the cuda set has no host stage functions
            continue
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = None
    if hasattr(lib, "flow_oracle_conservation"):
        lib.flow_oracle_conservation.argtypes = [I, I, I, P, P, P]
        lib.flow_oracle_conservation.restype = None


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


# --------------------------------------------------------------------------
# Problem set-up (arch initialise_mesh_2d / initialise_shared_data_2d, as
# restated in oracle/arch/arch_shim.c).


class HostMesh:
    """Uniform mesh of ``gnx x gny`` interior cells with its spacing arrays."""

    def __init__(self, gnx: int, gny: int, width: float = 1.0, height: float = 1.0,
                 dt: float = 1e-3, max_dt: float = 10.0, sim_end: float = 10.0):
        self.gnx, self.gny = gnx, gny
        self.nx, self.ny = gnx + 2 * PAD, gny + 2 * PAD
        k = np.arange(self.nx + 1, dtype=np.float64) - PAD
        self.edgex = width * k / gnx
        k = np.arange(self.ny + 1, dtype=np.float64) - PAD
        self.edgey = height * k / gny
        self.edgedx = np.full(self.nx + 1, width / gnx)
        self.celldx = self.edgedx.copy()
        self.edgedy = np.full(self.ny + 1, height / gny)
        self.celldy = self.edgedy.copy()
        m = Mesh()
        m.global_nx, m.global_ny = gnx, gny
        m.local_nx, m.local_ny = self.nx, self.ny
        m.pad, m.x_off, m.y_off, m.rank, m.nranks = PAD, 0, 0, 0, 1
        for i in range(4):
            m.neighbours[i] = -1
        m.width, m.height, m.max_dt, m.sim_end = width, height, max_dt, sim_end
        m.dt = C_T * dt
        m.dt_h = m.dt
        m.edgex, m.edgey = ptr(self.edgex), ptr(self.edgey)
        m.edgedx, m.edgedy = ptr(self.edgedx), ptr(self.edgedy)
        m.celldx, m.celldy = ptr(self.celldx), ptr(self.celldy)
        self.mesh = m

    @property
    def cshape(self):
        return (self.ny, self.nx)


FIELDS = ("P", "rho", "rho_old", "e", "u", "v", "rho_u", "rho_v", "Qxx", "Qyy",
          "F_x", "F_y", "uF_x", "uF_y", "vF_x", "vF_y", "reduce")


class HostState:
    """All arrays of one problem, allocated as the reference host does
    (cell arrays nx*ny; face/flux arrays (nx+1)*(ny+1), main.c:52-62)."""

    def __init__(self, hm: HostMesh):
        nc = hm.nx * hm.ny
        nf = (hm.nx + 1) * (hm.ny + 1)
        self.hm = hm
        self.a = {}
        for f in FIELDS:
            n = nf if f in ("u", "v", "rho_u", "rho_v", "F_x", "F_y", "uF_x",
                            "uF_y", "vF_x", "vF_y") else nc
            self.a[f] = np.zeros(n, dtype=np.float64)

    def __getitem__(self, k):
        return self.a[k]

    def copy(self) -> "HostState":
        out = HostState.__new__(HostState)
        out.hm = self.hm
        out.a = {k: v.copy() for k, v in self.a.items()}
        return out

    def args(self):
        return [ptr(self.a[f]) for f in FIELDS]

    def cell(self, name):
        return self.a[name][: self.hm.nx * self.hm.ny].reshape(self.hm.cshape)

    def interior(self, name):
        """Interior view of a state field in its own grid layout."""
        hm, p = self.hm, PAD
        a = self.a[name]
        if name in ("u", "rho_u", "F_x"):        # x faces: ny rows, nx+1 cols
            return a[: hm.ny * (hm.nx + 1)].reshape(hm.ny, hm.nx + 1)[p:hm.ny - p, p:hm.nx + 1 - p]
        if name in ("v", "rho_v", "F_y"):        # y faces: ny+1 rows, stride nx
            return a[: (hm.ny + 1) * hm.nx].reshape(hm.ny + 1, hm.nx)[p:hm.ny + 1 - p, p:hm.nx - p]
        return self.cell(name)[p:hm.ny - p, p:hm.nx - p]


def fill_boxes(hm: HostMesh, st: HostState, boxes) -> None:
    """Rasterises (density, energy, xpos, ypos, width, height) boxes with the
    left/bottom-edge rule of arch_shim.c set_problem_2d, then applies the
    initial reflective ghost fill of main.c:56-59."""
    rho, e = st.cell("rho"), st.cell("e")
    ex, ey = hm.edgex[: hm.nx], hm.edgey[: hm.ny]
    for (d, en, x0, y0, w, h) in boxes:
        mx = (ex >= x0) & (ex < x0 + w)
        my = (ey >= y0) & (ey < y0 + h)
        sel = my[:, None] & mx[None, :]
        rho[sel] = d
        e[sel] = en
    L = lib("port")
    L.handle_boundary_2d(hm.nx, hm.ny, ctypes.byref(hm.mesh), ptr(st["rho"]), 0, 1)
    L.handle_boundary_2d(hm.nx, hm.ny, ctypes.byref(hm.mesh), ptr(st["e"]), 0, 1)


def fill_fields(hm: HostMesh, st: HostState, rho_int: np.ndarray, e_int: np.ndarray) -> None:
    """Sets interior density/energy from arrays and applies the ghost fill."""
    p = PAD
    st.cell("rho")[p:hm.ny - p, p:hm.nx - p] = rho_int
    st.cell("e")[p:hm.ny - p, p:hm.nx - p] = e_int
    L = lib("port")
    L.handle_boundary_2d(hm.nx, hm.ny, ctypes.byref(hm.mesh), ptr(st["rho"]), 0, 1)
    L.handle_boundary_2d(hm.nx, hm.ny, ctypes.byref(hm.mesh), ptr(st["e"]), 0, 1)


def sod_boxes():
    """Sod shock tube (the 512x512 CPU-runnable case): right state everywhere,
    left half high."""
    return [(0.125, 2.0, 0.0, 0.0, 1.0, 1.0), (1.0, 2.5, 0.0, 0.0, 0.5, 1.0)]


def sedov_boxes(n: int):
    """Sedov-type blast: rho 1, e 1e-5, central 4x4 cells with e 1e4."""
    c = (n // 2 - 2) / n
    return [(1.0, 1e-5, 0.0, 0.0, 1.0, 1.0), (1.0, 1e4, c, c, 4.0 / n, 4.0 / n)]


def flow_params_boxes():
    """The reference's own problem (flow.params:1-2)."""
    return [(0.125, 2.0, 0.0, 0.0, 1.0, 1.0), (1.0, 2.5, 0.4, 0.4, 0.2, 0.2)]


def initial_timestep(hm: HostMesh, st: HostState, kind: str = "port") -> None:
    """The driver's set_timestep(first_step = 0) before the loop, main.c:64-66."""
    L = lib(kind)
    L.set_timestep(hm.nx, hm.ny, ptr(st["Qxx"]), ptr(st["Qyy"]), ptr(st["rho"]),
                   ptr(st["e"]), ctypes.byref(hm.mesh), ptr(st["reduce"]), 0,
                   hm.mesh.celldx, hm.mesh.celldy)


def step(hm: HostMesh, st: HostState, tt: int, kind: str = "port") -> None:
    L = lib(kind)
    L.solve_hydro_2d(ctypes.byref(hm.mesh), tt, *st.args())


def run(hm: HostMesh, st: HostState, steps: int, kind: str = "port", t0: int = 0) -> None:
    for tt in range(t0, t0 + steps):
        step(hm, st, tt, kind)


def conservation(hm: HostMesh, st: HostState) -> tuple[float, float]:
    out = np.zeros(2)
    lib("port").flow_oracle_conservation(hm.nx, hm.ny, PAD, ptr(st["rho"]), ptr(st["e"]), ptr(out))
    return float(out[0]), float(out[1])
