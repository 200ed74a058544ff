"""The reference's own cuda kernel set (cuda/flow.cu, cuda/flow.k), built for
sm_103a on the restated arch CUDA layer (oracle/arch/cuda), as a second GPU
baseline: it must run through its flow_interface.h entry points on device
arrays and agree with the oracle.  It is the reference's GPU code, compiled
with nvcc's default FMA contraction, so it matches the strict oracle to
round-off rather than bit for bit.  Skipped where the reference's sources
(or their staged copy) were not available to build it."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tolerance import cell_rel_err

pytestmark = pytest.mark.gpu

STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


def run_reference_cuda(fg, prob, steps):
    Lr = O.lib("reference_cuda")
    sim = fg.DeviceSim(prob)  # device arrays, ghost-filled initial state
    m = sim.mesh
    mp = ctypes.cast(ctypes.addressof(m), ctypes.POINTER(O.Mesh))  # same layout
    args = sim.args()
    Lr.set_timestep(sim.nx, sim.ny, args[8], args[9], args[1], args[3], mp, args[16], 0,
                    m.celldx, m.celldy)
    for tt in range(steps):
        Lr.solve_hydro_2d(mp, tt, *args)
    return sim


@pytest.mark.skipif(not O.have_reference_cuda(), reason="the reference's cuda set was not built")
def test_reference_cuda_set_runs_and_matches_the_oracle():
    import flow_gb300 as fg
    from flow_gb300 import problems
    fg.lib()
    prob = problems.sod(96, 80)
    steps = 20
    sim = run_reference_cuda(fg, prob, steps)
    hm = O.HostMesh(prob.gnx, prob.gny, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st)
    O.run(hm, st, steps)
    assert abs(sim.mesh.dt - hm.mesh.dt) <= 1e-10 * hm.mesh.dt
    for k in STATE:
        assert cell_rel_err(sim.interior(k), st.interior(k)) <= 1e-9, k
    mass = sim.interior("rho").sum()
    assert abs(mass - prob.interior(prob.rho).sum()) <= 1e-12 * mass
