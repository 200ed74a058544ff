"""Host-side problem set-up for the flow kernel set.

Restates, for the single-rank case, what the reference host gets from the
arch layer before its timestep loop (main.c:17-66):

* the uniform mesh: face jj of the padded mesh sits at
  ``width*(jj - pad)/global_nx``, and every edge and cell spacing is
  ``width/global_nx`` (arch ``initialise_mesh_2d``, used at main.c:40);
* the problem boxes of a params file (``problem_N density= energy= xpos= ypos=
  width= height=``, flow.params:1-2): a cell takes a box's state when its
  left/bottom edge coordinate lies in ``[pos, pos+extent)``; later boxes win
  (arch ``initialise_shared_data_2d``, main.c:52-54).  This is the rule the
  reference's golden totals (flow.tests:1) require: the 0.2-wide box of
  flow.params must cover exactly 819 x 819 cells at 4096^2;
* the initial timestep pair ``dt = dt_h = C_T * params dt`` (main.c:30-31).

It also generates the synthetic workloads of the benchmark (Sod tube,
Sedov-type blast, two-region ensembles, smooth random fields).
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

PAD = 2
GAM = 1.4
C_T = 0.3


@dataclass
class Problem:
    """A uniform single-rank mesh of ``gnx x gny`` interior cells and its
    initial density/energy (padded cell arrays, ghosts filled later)."""

    gnx: int
    gny: int
    width: float = 1.0
    height: float = 1.0
    dt_param: float = 1e-3      # the params-file dt (main.c:30)
    max_dt: float = 10.0        # start value of the CFL minimum (arch.params)
    sim_end: float = 10.0
    rho: np.ndarray = field(default=None, repr=False)
    e: np.ndarray = field(default=None, repr=False)
    # The boxes the fields were built from, when they were built from boxes
    # alone (None once fields() sets them): the device can rasterise those
    # itself (gb300_fill_boxes) instead of receiving host arrays.
    box_list: list = field(default=None, repr=False)

    def __post_init__(self):
        if self.gnx < 2 or self.gny < 2:
            raise ValueError("need at least 2 interior cells per axis")
        self.nx, self.ny = self.gnx + 2 * PAD, self.gny + 2 * PAD
        if self.rho is None:
            self.rho = np.zeros((self.ny, self.nx))
            self.e = np.zeros((self.ny, self.nx))
            self.box_list = []

    # -- mesh arrays (local_n + 1 entries each) ------------------------------
    @property
    def edgex(self):
        return self.width * (np.arange(self.nx + 1, dtype=np.float64) - PAD) / self.gnx

    @property
    def edgey(self):
        return self.height * (np.arange(self.ny + 1, dtype=np.float64) - PAD) / self.gny

    @property
    def edgedx(self):
        return np.full(self.nx + 1, self.width / self.gnx)

    @property
    def edgedy(self):
        return np.full(self.ny + 1, self.height / self.gny)

    celldx = edgedx
    celldy = edgedy

    @property
    def cells(self) -> int:
        return self.gnx * self.gny

    # -- initial state --------------------------------------------------------
    def boxes(self, boxes) -> "Problem":
        """Rasterises (density, energy, xpos, ypos, width, height) boxes."""
        ex, ey = self.edgex[: self.nx], self.edgey[: self.ny]
        for (d, en, x0, y0, w, h) in boxes:
            sel = ((ey >= y0) & (ey < y0 + h))[:, None] & ((ex >= x0) & (ex < x0 + w))[None, :]
            self.rho[sel] = d
            self.e[sel] = en
        if self.box_list is not None:
            self.box_list = self.box_list + [tuple(float(v) for v in b) for b in boxes]
        return self

    def fields(self, rho_int: np.ndarray, e_int: np.ndarray) -> "Problem":
        """Sets the interior density and specific energy from arrays."""
        p = PAD
        self.rho[p:self.ny - p, p:self.nx - p] = rho_int
        self.e[p:self.ny - p, p:self.nx - p] = e_int
        self.box_list = None
        return self

    def interior(self, a: np.ndarray) -> np.ndarray:
        return a[PAD:self.ny - PAD, PAD:self.nx - PAD]

    def cfl_dt(self) -> float:
        """Smallest celldx / c_s over the interior of the initial state, the
        params dt the benchmark workloads use, so that the first step
        starts at the C_T safety factor (a larger params dt makes the first
        Lagrangian step run at up to C_T*params dt, main.c:30 and
        omp3/flow.c:103-105)."""
        e = self.interior(self.e)
        cs = np.sqrt(GAM * (GAM - 1.0) * np.maximum(e, 0.0))
        h = min(self.width / self.gnx, self.height / self.gny)
        return float(h / cs.max())

    def with_cfl_dt(self) -> "Problem":
        self.dt_param = self.cfl_dt()
        return self


def parse_params(text: str) -> dict:
    """Reads the reference params format (flow.params:1-7): ``key value``
    lines and ``problem_N k=v ...`` lines."""
    out: dict = {"problems": []}
    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if re.fullmatch(r"problem_\d+", tok[0]):
            kv = dict(t.split("=", 1) for t in tok[1:] if "=" in t)
            out["problems"].append((int(tok[0].split("_")[1]), {k: float(v) for k, v in kv.items()}))
        elif len(tok) >= 2:
            out[tok[0]] = tok[1]
    out["problems"].sort()
    return out


def from_params(text: str, width: float = 1.0, height: float = 1.0) -> tuple[Problem, int]:
    """Problem and iteration count of a params file's text."""
    p = parse_params(text)
    prob = Problem(int(p["nx"]), int(p["ny"]), width, height, dt_param=float(p["dt"]))
    prob.boxes([(b["density"], b["energy"], b["xpos"], b["ypos"], b["width"], b["height"])
                for _, b in p["problems"]])
    return prob, int(p.get("iterations", 1))


# ---------------------------------------------------------------------------
# Benchmark workloads (synthetic, seeded).

def sod(n: int, ny: int | None = None) -> Problem:
    """2-D Sod tube: density 0.125 / energy 2.0 everywhere, density 1.0 /
    energy 2.5 for x < 0.5."""
    return Problem(n, ny or n).boxes([(0.125, 2.0, 0.0, 0.0, 1.0, 1.0),
                                      (1.0, 2.5, 0.0, 0.0, 0.5, 1.0)]).with_cfl_dt()


def sedov(n: int) -> Problem:
    """Sedov-type blast: density 1, energy 1e-5, central 4x4 cells at 1e4."""
    c = (n // 2 - 2) / n
    return Problem(n, n).boxes([(1.0, 1e-5, 0.0, 0.0, 1.0, 1.0),
                                (1.0, 1e4, c, c, 4.0 / n, 4.0 / n)]).with_cfl_dt()


def reference_problem(n: int = 4096) -> Problem:
    """The reference's own flow.params problem (flow.params:1-5)."""
    return Problem(n, n, dt_param=1e-3).boxes([(0.125, 2.0, 0.0, 0.0, 1.0, 1.0),
                                               (1.0, 2.5, 0.4, 0.4, 0.2, 0.2)])


def two_region(n: int, rng: np.random.Generator) -> Problem:
    """One instance of the two-region ensemble: split at the midpoint along a
    random axis; density ratio log-uniform in [1, 100] with the high side at
    1.0; specific energies uniform in [0.5, 5] per side."""
    ratio = math.exp(rng.uniform(0.0, math.log(100.0)))
    e_hi, e_lo = rng.uniform(0.5, 5.0, size=2)
    axis = int(rng.integers(0, 2))
    high_first = bool(rng.integers(0, 2))
    # As boxes: the low side everywhere, then the high half (cells 0..n/2-1
    # or n/2..n-1 along the axis; the left/bottom-edge rule at k/n is exact).
    half = n // 2
    lo, extent = (0.0, half / n) if high_first else (half / n, 1.0)
    high = (lo, 0.0, extent, 1.0) if axis == 0 else (0.0, lo, 1.0, extent)
    return Problem(n, n).boxes([(1.0 / ratio, e_lo, 0.0, 0.0, 1.0, 1.0),
                                (1.0, e_hi) + high]).with_cfl_dt()


def fourier_field(n: int, rng: np.random.Generator, modes: int = 16,
                  kmax: int = 8, amplitude: float = 0.1) -> np.ndarray:
    """Sum of `modes` random Fourier modes with integer wavenumbers 1..kmax in
    each direction, random phases, amplitudes scaled so sum |a_k| = amplitude.
    Evaluated separably: cos(a + b) = cos a cos b - sin a sin b."""
    x = (np.arange(n) + 0.5) / n
    kx = rng.integers(1, kmax + 1, size=modes)
    ky = rng.integers(1, kmax + 1, size=modes)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=modes)
    amp = rng.uniform(0.0, 1.0, size=modes)
    amp *= amplitude / amp.sum()
    ax = 2 * math.pi * kx[:, None] * x[None, :] + ph[:, None]      # modes x n
    ay = 2 * math.pi * ky[:, None] * x[None, :]
    cx, sx = np.cos(ax) * amp[:, None], np.sin(ax) * amp[:, None]
    cy, sy = np.cos(ay), np.sin(ay)
    # f[i, j] = sum_k amp_k (cos(ay_k[i]) cos(ax_k[j]) - sin(ay_k[i]) sin(ax_k[j]))
    return cy.T @ cx - sy.T @ sx


def smooth_random(n: int, rng: np.random.Generator) -> Problem:
    """One instance of the smooth ensemble: density 1 + f1, energy 1 + f2."""
    f1 = fourier_field(n, rng)
    f2 = fourier_field(n, rng)
    return Problem(n, n).fields(1.0 + f1, 1.0 + f2).with_cfl_dt()
