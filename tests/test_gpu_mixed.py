"""The mixed-precision form (gb300_mixed_solve) against the FP64 oracle.

The scheme is unchanged; FP32 arithmetic perturbs the solution, so the test
bounds the L1 error per field (sum|got-want| / sum|want|) after the stated
step count, the L-infinity error, and the drift of total mass (conserved to
FP64 round-off by the FP64 conservative update).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tolerance import l1_rel, linf_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    return flow_gb300


def run_pair(fg, prob, steps):
    sim = fg.MixedSim(prob)
    hm = O.HostMesh(prob.gnx, prob.gny, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st)
    assert abs(sim.mesh.dt - hm.mesh.dt) <= 1e-6 * hm.mesh.dt
    m0 = sim.conservation()[0]
    for tt in range(steps):
        sim.step()
        O.step(hm, st, tt)
    return sim, hm, st, m0


def errors(sim, st):
    out = {}
    for k in ("rho", "e", "u", "v", "rho_u", "rho_v"):
        out[k] = (l1_rel(sim.interior(k), st.interior(k)), linf_rel(sim.interior(k), st.interior(k)))
    return out


def test_mixed_sod_256_100_steps(fg):
    from flow_gb300 import problems
    sim, hm, st, m0 = run_pair(fg, problems.sod(256), 100)
    err = errors(sim, st)
    print("mixed sod256 L1/Linf", err)
    assert err["rho"][0] <= 1e-5 and err["e"][0] <= 1e-5
    assert err["rho_u"][0] <= 1e-4 and err["u"][0] <= 1e-4
    m1 = sim.conservation()[0]
    assert abs(m1 - m0) <= 1e-12 * m0
    assert abs(sim.mesh.dt - hm.mesh.dt) <= 1e-4 * hm.mesh.dt


def test_mixed_blast_128_200_steps(fg):
    from flow_gb300 import problems
    sim, hm, st, m0 = run_pair(fg, problems.sedov(128), 200)
    err = errors(sim, st)
    print("mixed blast128 L1/Linf", err)
    assert err["rho"][0] <= 1e-5 and err["e"][0] <= 1e-4
    assert err["u"][0] <= 1e-4 and err["v"][0] <= 1e-4
    assert np.isfinite(sim.interior("e")).all() and sim.interior("e").min() > 0
    assert abs(sim.conservation()[0] - m0) <= 1e-12 * m0


def test_mixed_ragged_reference_problem(fg):
    from flow_gb300.problems import Problem
    prob = Problem(203, 157, dt_param=1e-3).boxes(O.flow_params_boxes())
    sim, hm, st, m0 = run_pair(fg, prob, 33)
    err = errors(sim, st)
    assert err["rho"][0] <= 1e-5 and err["e"][0] <= 1e-5, err


def test_mixed_rejects_small_workspace(fg):
    from flow_gb300 import problems
    import ctypes
    sim = fg.MixedSim(problems.sod(32))
    st = fg.lib().gb300_mixed_solve(ctypes.byref(sim.mesh), 0, fg.dptr(sim.rho), fg.dptr(sim.e),
                                    fg.vptr(sim.rho_u), fg.vptr(sim.rho_v), fg.vptr(sim.work),
                                    sim.work_bytes - 1, fg.dptr(sim.reduce))
    assert st == 2
    with pytest.raises(fg.FlowError):
        fg.check()
