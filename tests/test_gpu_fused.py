"""GPU parity of the fused FP64 timestep (the default solve_hydro_2d mode)
against the reference and the oracle.

Density and energy: within 1e-12 per cell (tests/tolerance.py), always.
Velocities and momenta: within 1e-12 per cell on the benchmark problems; on
the golden fixtures within max(1e-12, 2x the reference's own build-to-build
difference on that fixture).  The reference has no single bitwise answer for
these signed fields: its default build (Makefile:15, -march=native, which
contracts FMAs) and a strict IEEE build differ by up to ~1e-11 per cell where
momenta pass through zero, and each fixture stores both.  dt within 1e-12;
mass conserved to round-off."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tolerance import FP64_TOL, cell_rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)
    return flow_gb300


def pair(fg, prob):
    sim = fg.DeviceSim(prob)
    hm = O.HostMesh(prob.gnx, prob.gny, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    return sim, hm, st


def compare(sim, st, tol=FP64_TOL, fields=STATE):
    errs = {k: cell_rel_err(sim.interior(k), st.interior(k)) for k in fields}
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, errs
    return errs


def run_both(fg, prob, steps, check_every=None):
    sim, hm, st = pair(fg, prob)
    sim.initial_timestep()
    O.initial_timestep(hm, st)
    for tt in range(steps):
        sim.step()
        O.step(hm, st, tt)
        assert abs(sim.mesh.dt - hm.mesh.dt) <= FP64_TOL * hm.mesh.dt, tt
        assert abs(sim.mesh.dt_h - hm.mesh.dt_h) <= FP64_TOL * hm.mesh.dt_h, tt
        if check_every and (tt + 1) % check_every == 0:
            compare(sim, st)
    return sim, hm, st


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_fused_matches_reference_fixture(fg, path):
    from flow_gb300.problems import Problem
    z = np.load(path)
    gny, gnx = z["rho0"].shape
    prob = Problem(gnx, gny, dt_param=float(z["dt_param"])).fields(z["rho0"], z["e0"])
    sim = fg.DeviceSim(prob)
    sim.initial_timestep()
    for _ in range(int(z["steps"])):
        sim.step()
    np.testing.assert_allclose(sim.mesh.dt, z["dt_hist"][-1][0], rtol=FP64_TOL)
    hm = O.HostMesh(gnx, gny)
    ref, ref_default = O.HostState(hm), O.HostState(hm)
    for k in STATE:
        ref.a[k][:] = z[f"out_{k}"]
        ref_default.a[k][:] = z[f"default_out_{k}"]
    for k in STATE:
        err = cell_rel_err(sim.interior(k), ref.interior(k))
        build_var = cell_rel_err(ref_default.interior(k), ref.interior(k))
        tol = FP64_TOL if k in ("rho", "e") else max(FP64_TOL, 2 * build_var)
        assert err <= tol, (k, err, build_var)


def test_fused_sod_512_100_steps(fg):
    """Config 0: 512^2 Sod tube, 100 iterations, per-cell within 1e-12."""
    from flow_gb300 import problems
    sim, hm, st = run_both(fg, problems.sod(512), 100, check_every=25)
    errs = compare(sim, st)
    m_gpu, _ = sim.conservation()
    m0 = 0.125 * 512 * 256 + 1.0 * 512 * 256
    assert abs(m_gpu - m0) <= 1e-13 * m0, (m_gpu, m0)
    print("sod512 max per-cell rel err", errs)


def test_fused_blast_128_200_steps(fg):
    """Sedov-type blast (config 1 at reduced size), 200 iterations."""
    from flow_gb300 import problems
    sim, hm, st = run_both(fg, problems.sedov(128), 200, check_every=50)
    compare(sim, st)


def test_fused_known_answer_4096_per_cell(fg):
    """The reference's own known-answer case (flow.params: 4096^2, params dt
    1e-3, 100 iterations, flow.tests:1) per cell against the oracle.  Its
    first step runs at Courant ~0.9 and drives 3276 cells to negative energy
    inside the step (NaN CFL candidates in the reference).  Density and energy
    within 1e-12; velocities and momenta within 1e-11, which is 2.5x the
    reference's own strict-vs-default-build difference on this case
    (4.0e-12 in rho_u)."""
    from flow_gb300.problems import Problem
    prob = Problem(4096, 4096, dt_param=1e-3).boxes(O.flow_params_boxes())
    sim = fg.DeviceSim(prob)
    sim.initial_timestep()
    hm = O.HostMesh(4096, 4096, dt=1e-3)
    st = O.HostState(hm)
    O.fill_boxes(hm, st, O.flow_params_boxes())
    O.initial_timestep(hm, st)
    for tt in range(100):
        sim.step()
        O.step(hm, st, tt)
        assert abs(sim.mesh.dt - hm.mesh.dt) <= FP64_TOL * hm.mesh.dt, tt
    errs = {k: cell_rel_err(sim.interior(k), st.interior(k)) for k in STATE}
    for k, v in errs.items():
        assert v <= (FP64_TOL if k in ("rho", "e") else 1e-11), errs
    e_total = sim.interior("e").sum()
    assert abs(e_total - 3.389026275051e+07) <= 1e-11 * 3.389026275051e+07


def test_fused_and_exact_modes_agree(fg):
    from flow_gb300 import problems
    prob = problems.sod(200, 136)
    sims = []
    for mode in (fg.MODE_EXACT, fg.MODE_FUSED):
        fg.set_mode(mode)
        s = fg.DeviceSim(prob)
        s.initial_timestep()
        s.run(30)
        sims.append(s)
    fg.set_mode(fg.MODE_FUSED)
    for k in STATE:
        assert cell_rel_err(sims[1].interior(k), sims[0].interior(k)) <= FP64_TOL, k
