"""Generates the golden fixtures of tests/golden/ from the REFERENCE itself.

Run in a container that has the reference sources (it builds
oracle/_ref/libflow_ref.so from omp3/flow.c with the arch shim):

    python tests/golden/make_golden.py

Each case stores its initial interior density/energy, the params dt, the
step count, and every array of the reference host state after the run
(main.c:52-62 layout), plus the dt/dt_h history; the state fields are also
stored as the reference's default build (-march=native, FMA contraction)
computes them, which measures the reference's own rounding variation.  The reference's own
known-answer vector (flow.tests:1) is checked separately by
tests/test_oracle.py.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

STATE_FIELDS = ("rho", "e", "u", "v", "rho_u", "rho_v")


def _smooth(n_x, n_y, rng, modes=16, kmax=8, amp=0.1):
    x = (np.arange(n_x) + 0.5) / n_x
    y = (np.arange(n_y) + 0.5) / n_y
    f = np.zeros((n_y, n_x))
    a = rng.uniform(0, 1, modes)
    a *= amp / a.sum()
    for k in range(modes):
        kx, ky = rng.integers(1, kmax + 1, 2)
        ph = rng.uniform(0, 2 * np.pi)
        f += a[k] * np.cos(2 * np.pi * (kx * x[None, :] + ky * y[:, None]) + ph)
    return f


def _boxes_state(gnx, gny, boxes):
    hm = O.HostMesh(gnx, gny)
    st = O.HostState(hm)
    O.fill_boxes(hm, st, boxes)
    return O.PAD, st.interior("rho").copy(), st.interior("e").copy()


def _cfl(gnx, gny, e):
    cs = np.sqrt(O.GAM * (O.GAM - 1.0) * e.max())
    return min(1.0 / gnx, 1.0 / gny) / cs


def cases():
    rng = np.random.default_rng(20261203)
    out = {}
    _, r, e = _boxes_state(24, 20, O.sod_boxes())
    out["sod_24x20"] = dict(rho=r, e=e, dt=_cfl(24, 20, e), steps=30)
    _, r, e = _boxes_state(32, 32, O.sedov_boxes(32))
    out["blast_32"] = dict(rho=r, e=e, dt=_cfl(32, 32, e), steps=40)
    _, r, e = _boxes_state(40, 40, O.flow_params_boxes())
    out["refproblem_40"] = dict(rho=r, e=e, dt=1e-3, steps=25)
    r = 1.0 + _smooth(20, 28, rng)
    e = 1.0 + _smooth(20, 28, rng)
    out["smooth_20x28"] = dict(rho=r, e=e, dt=_cfl(20, 28, e), steps=21)
    _, r, e = _boxes_state(151, 93, O.flow_params_boxes())
    out["refproblem_151x93"] = dict(rho=r, e=e, dt=1e-3, steps=41)
    # The known-answer problem with its params dt scaled to 64^2 (the same
    # ratio to the cell width as dt 1e-3 at 4096^2): the first step runs at
    # Courant ~0.9 and shock heating drives 52 cells to negative energy, whose
    # CFL candidates are NaN in the reference.
    _, r, e = _boxes_state(64, 64, O.flow_params_boxes())
    out["courant_64"] = dict(rho=r, e=e, dt=0.064, steps=30)
    r = np.array([[1.0, 0.5], [0.25, 0.75], [0.6, 0.9]])
    e = np.array([[2.0, 1.0], [1.5, 3.0], [2.5, 0.8]])
    out["tiny_2x3"] = dict(rho=r, e=e, dt=_cfl(2, 3, e), steps=9)
    return out


def run_case(kind, c):
    gny, gnx = c["rho"].shape
    hm = O.HostMesh(gnx, gny, dt=c["dt"])
    st = O.HostState(hm)
    O.fill_fields(hm, st, c["rho"], c["e"])
    O.initial_timestep(hm, st, kind)
    hist = [(hm.mesh.dt, hm.mesh.dt_h)]
    for tt in range(c["steps"]):
        O.step(hm, st, tt, kind)
        hist.append((hm.mesh.dt, hm.mesh.dt_h))
    return hm, st, np.array(hist)


def write_reference_case():
    """The reference's known-answer case in the reference params format,
    restated from its problem (flow.params:1-6), and its golden totals
    (flow.tests:1), for the C-driver test."""
    lines = ["problem_0 density=0.125 energy=2.0 xpos=0.0 ypos=0.0 width=1.0 height=1.0",
             "problem_1 density=1.0 energy=2.5 xpos=0.4 ypos=0.4 width=0.2 height=0.2",
             "dt            1.0e-3", "nx            4096", "ny            4096",
             "iterations    100", "visit_dump    0"]
    with open(os.path.join(HERE, "flow.params"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(O.REF_DIR, "flow.tests")) as f:
        golden = f.read().strip()
    with open(os.path.join(HERE, "flow.tests"), "w") as f:
        f.write(golden + "\n")


def main(names=None):
    """Writes every case, or only the named ones."""
    write_reference_case()
    if not O.have_reference():
        O.build()
    assert O.have_reference(), "needs the reference sources to build oracle/_ref"
    for name, c in cases().items():
        if names and name not in names:
            continue
        hm, st, hist = run_case("reference", c)
        # The reference built with its default flags: how far its own builds
        # differ per cell (rounding only), stored for the state fields.
        _, st_d, _ = run_case("reference_default", c)
        arrays = {f"out_{k}": v for k, v in st.a.items() if k != "reduce"}
        arrays.update({f"default_out_{k}": st_d.a[k] for k in STATE_FIELDS})
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), rho0=c["rho"], e0=c["e"],
                            dt_param=c["dt"], steps=c["steps"], dt_hist=hist, **arrays)
        print(name, hm.gnx, hm.gny, c["steps"], "dt", hist[-1])


if __name__ == "__main__":
    main(sys.argv[1:])
