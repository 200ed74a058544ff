"""The fused single-problem step keeps flags for the work that happens only
where the flow moves (viscous-stress flags, mass-flux flags in the caller's
reduce_array); the batched kernels keep none.  On meshes large enough to hold
the flags, the single-problem step must therefore equal a one-instance batch
bit for bit, step after step -- here on problems chosen to put moving cells
where the flag logic has its edge cases: a blast in a corner (ghost images of
flagged rows and columns), a blast straddling a 127-column x-sweep tile, a
128-column tile and a 16-row tile boundary, a shock tube whose mesh width is
no multiple of any tile width, and a field in motion everywhere (every flag
set), in both precision forms."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 20


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)
    return flow_gb300


def problems_with_flags():
    from flow_gb300 import problems
    P = problems.Problem
    return {
        "corner_blast": P(130, 70).boxes([(1.0, 1e-5, 0.0, 0.0, 1.0, 1.0),
                                          (1.0, 1e3, 0.0, 0.0, 6 / 130, 6 / 70)]).with_cfl_dt(),
        "tile_boundary_blast": P(300, 90).boxes(
            [(1.0, 1e-5, 0.0, 0.0, 1.0, 1.0),
             (1.0, 1e3, 124 / 300, 13 / 90, 8 / 300, 7 / 90)]).with_cfl_dt(),
        "sod_257x33": problems.sod(257, 33),
        "smooth_96": problems.smooth_random(96, np.random.default_rng(11)),
    }


def flags_active(p):
    # The flags fit in reduce_array (nx*ny doubles) after the 2056 header and
    # partial slots: four word arrays of at most (ny + 1) x 4 ceil((nx + 1) / 127).
    words = 4 * (p.ny + 1) * 4 * ((p.nx + 1 + 126) // 127 + (p.nx + 127) // 128)
    return 8 * p.nx * p.ny >= 8 * 2056 + 4 * words


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["corner_blast", "tile_boundary_blast", "sod_257x33",
                                  "smooth_96"])
def test_flagged_step_equals_unflagged_batch(fg, name, precision):
    p = problems_with_flags()[name]
    assert flags_active(p)
    sim = fg.DeviceSim(p) if precision == 0 else fg.MixedSim(p)
    if precision == 0:
        sim.initial_timestep()
    b = fg.Batch([p], precision=precision)
    for tt in range(STEPS):
        sim.step()
        b.step(1, use_graph=False)
        b.status()
        rho, e, dt, _ = b.state(0)
        assert np.array_equal(rho, sim.interior("rho")), (tt, "rho",
                                                          int(np.count_nonzero(rho != sim.interior("rho"))))
        assert np.array_equal(e, sim.interior("e")), (tt, "e")
        assert dt[0] == sim.mesh.dt and dt[1] == sim.mesh.dt_h, tt
