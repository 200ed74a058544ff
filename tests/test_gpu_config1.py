"""Per-cell parity on the benchmark workload at its full size and length:
the Sedov-type blast on a 4096^2 mesh, FP64, 500 iterations (the problem the
cell-steps/s headline is measured on).

The fused FP64 step (the default solve_hydro_2d mode) is compared with the
oracle -- the C restatement of the reference's omp3 set, compiled with strict
IEEE evaluation -- after every one of the 500 steps for dt, and per cell at
steps 250 and 500 for density, specific energy, both velocities and both
momenta, each within 1e-12 relative (tests/tolerance.py: |a-b| <= 1e-12 *
max(|b|, 1e-3 max|b|)).  Total mass is conserved to round-off.  The exact
mode runs beside it and must equal the oracle bit for bit on every cell.

The fused form's still-field paths (warp-uniform skips of arithmetic whose
result an exact zero fixes) run on most of this mesh, which is at rest
outside the blast wave; smaller blasts exercise them far less, so this case
is the one that pins the headline's numbers.  Runtime: about a minute (the
oracle steps on every host core).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tolerance import FP64_TOL, cell_rel_err

pytestmark = pytest.mark.gpu

STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")
N = 4096
STEPS = 500


def test_sedov_4096_500_steps_fused_and_exact_vs_oracle():
    import flow_gb300 as fg
    from flow_gb300 import problems
    fg.lib()
    prob = problems.sedov(N)
    fg.set_mode(fg.MODE_FUSED)
    fused = fg.DeviceSim(prob)
    fused.initial_timestep()
    fg.set_mode(fg.MODE_EXACT)
    exact = fg.DeviceSim(prob)
    exact.initial_timestep()
    hm = O.HostMesh(N, N, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st)
    worst = {}
    try:
        for tt in range(STEPS):
            fg.set_mode(fg.MODE_FUSED)
            fused.step()
            fg.set_mode(fg.MODE_EXACT)
            exact.step()
            O.step(hm, st, tt)
            assert abs(fused.mesh.dt - hm.mesh.dt) <= FP64_TOL * hm.mesh.dt, tt
            assert abs(fused.mesh.dt_h - hm.mesh.dt_h) <= FP64_TOL * hm.mesh.dt_h, tt
            assert exact.mesh.dt == hm.mesh.dt and exact.mesh.dt_h == hm.mesh.dt_h, tt
            if (tt + 1) % 250 == 0:
                for k in STATE:
                    want = st.interior(k)
                    err = cell_rel_err(fused.interior(k), want)
                    worst[k] = max(worst.get(k, 0.0), err)
                    assert err <= FP64_TOL, (tt + 1, k, err)
                    diff = int(np.count_nonzero(exact.interior(k) != want))
                    assert diff == 0, (tt + 1, k, "exact mode differs on", diff, "cells")
    finally:
        fg.set_mode(fg.MODE_FUSED)
    mass0 = float(prob.interior(prob.rho).sum())
    mass, _ = fused.conservation()
    assert abs(mass - mass0) <= 1e-13 * mass0, (mass, mass0)
    print("sedov 4096^2 x 500: max per-cell rel err of the fused step", worst)
