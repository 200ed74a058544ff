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
        # Tiles away from every wall, most of them at rest from one step to
        # the next while the blast grows into them (the previous step's
        # marks: pressures, velocities, CFL minima and round trips reused).
        "wide_blast": P(700, 300).boxes(
            [(1.0, 1e-5, 0.0, 0.0, 1.0, 1.0),
             (1.0, 1e3, 300 / 700, 140 / 300, 10 / 700, 10 / 300)]).with_cfl_dt(),
        # A pressure jump at rest: the first step changes momenta where the
        # velocities it stores may still be +0.
        "sod_700x64": problems.sod(700, 64),
    }


def flags_active(p):
    # The flags fit in reduce_array (nx*ny doubles) after the 2057 header and
    # partial slots: four word arrays of at most (ny + 1) x 4 ceil((nx + 1) / 127).
    words = 4 * (p.ny + 1) * 4 * ((p.nx + 1 + 126) // 127 + (p.nx + 127) // 128)
    return 8 * p.nx * p.ny >= 8 * 2057 + 4 * words


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["corner_blast", "tile_boundary_blast", "sod_257x33",
                                  "smooth_96", "wide_blast", "sod_700x64"])
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


STATE = ("rho", "e", "rho_u", "rho_v", "u", "v")


def test_state_written_between_steps(fg):
    """A caller that writes the state between two steps announces it
    (gb300_state_changed): the next step then recomputes every tile, and the
    run equals a fresh one started from the written state."""
    import torch
    p = problems_with_flags()["wide_blast"]
    a = fg.DeviceSim(p)
    a.initial_timestep()
    for _ in range(6):
        a.step()
    # A second blast, written by the caller into cells at rest.
    e2 = a.a["e"][: a.nx * a.ny].view(a.ny, a.nx)
    e2[150:160, 100:110] = 1e3
    assert fg.lib().gb300_state_changed() == 0
    b = fg.DeviceSim(p)
    for f in STATE:
        b.a[f].copy_(a.a[f])
    b.mesh.dt, b.mesh.dt_h, b.tt = a.mesh.dt, a.mesh.dt_h, a.tt
    torch.cuda.synchronize()
    for _ in range(8):
        a.step()
    for _ in range(8):
        b.step()
    for f in STATE:
        assert torch.equal(a.a[f], b.a[f]), f
    assert a.mesh.dt == b.mesh.dt and a.mesh.dt_h == b.mesh.dt_h


def test_conservation_kept_tiles_equal_fresh_sums(fg):
    """The conservation totals after each step keep the partial sums of tiles
    at rest through that step; they must equal, bit for bit, the totals summed
    afresh from the same cells (a copy of the state in other arrays)."""
    import ctypes
    import torch
    p = problems_with_flags()["wide_blast"]
    a = fg.DeviceSim(p)
    a.initial_timestep()
    kept, states = [], []
    for _ in range(12):
        a.step()
        kept.append(a.conservation())
        states.append((a.a["rho"].clone(), a.a["e"].clone()))
    L = fg.lib()
    ra = torch.zeros_like(a.a["reduce"])
    out = (ctypes.c_double * 2)()
    for k, (rho, e) in enumerate(states):
        assert L.gb300_conservation(a.nx, a.ny, 2, fg.dptr(rho), fg.dptr(e), fg.dptr(ra),
                                    ctypes.cast(out, ctypes.POINTER(ctypes.c_double)), 1) == 0
        assert (out[0], out[1]) == kept[k], k
