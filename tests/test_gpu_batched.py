"""The batched form (many instances of different sizes, each with its own dt,
advanced by one launch per phase over every instance's tiles or by one
persistent cooperative launch per timestep) against the single-problem fused
step: every instance must match it bit for bit, in both precision forms, both
schedules, with or without the captured CUDA graph and for every tile shape;
the FP64 instances must also match the oracle (1e-12 per cell for density and
energy)."""
import numpy as np
import pytest

from oracle import oracle as O
from tolerance import FP64_TOL, cell_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    flow_gb300.lib()
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)
    return flow_gb300


def ensemble():
    from flow_gb300 import problems
    rng = np.random.default_rng(7)
    return [problems.sod(40, 36), problems.sedov(64), problems.two_region(48, rng),
            problems.two_region(24, rng), problems.smooth_random(33, rng)]


def single(fg, prob, steps, precision):
    sim = fg.DeviceSim(prob) if precision == 0 else fg.MixedSim(prob)
    if precision == 0:
        sim.initial_timestep()
    sim.run(steps)
    return sim


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("schedule", [0, 1], ids=["phases", "persistent"])
def test_batch_matches_single_problem_step(fg, precision, use_graph, schedule):
    probs = ensemble()
    steps = 9
    b = fg.Batch(probs, precision=precision)
    b.set_schedule(schedule)
    b.step(steps, use_graph=use_graph)
    b.status()
    for i, p in enumerate(probs):
        rho, e, dt, _ = b.state(i)
        sim = single(fg, p, steps, precision)
        assert np.array_equal(rho, sim.interior("rho")), (i, "rho")
        assert np.array_equal(e, sim.interior("e")), (i, "e")
        assert dt[0] == sim.mesh.dt and dt[1] == sim.mesh.dt_h, i


@pytest.mark.parametrize("tuning", [(0, 8, 0, 0), (0, 32, 0, 1), (1, 8, 0, 0), (1, 32, 1, 1),
                                    (1, 16, 2, 0)])
def test_batch_tile_shapes_give_identical_results(fg, tuning):
    probs = ensemble()[:3]
    ref = fg.Batch(probs, precision=0)
    ref.step(6)
    b = fg.Batch(probs, precision=0)
    b.set_schedule(tuning[0])
    b.set_tuning(*tuning[1:])
    b.step(6)
    b.status()
    for i in range(len(probs)):
        assert np.array_equal(b.state(i)[0], ref.state(i)[0])
        assert np.array_equal(b.state(i)[1], ref.state(i)[1])


def test_batch_fp64_matches_oracle(fg):
    probs = ensemble()[:3]
    steps = 20
    b = fg.Batch(probs, precision=0)
    b.step(steps)
    for i, p in enumerate(probs):
        hm = O.HostMesh(p.gnx, p.gny, dt=p.dt_param)
        st = O.HostState(hm)
        O.fill_fields(hm, st, p.interior(p.rho), p.interior(p.e))
        O.initial_timestep(hm, st)
        O.run(hm, st, steps)
        rho, e, dt, tot = b.state(i)
        assert cell_rel_err(rho, st.interior("rho")) <= FP64_TOL
        assert cell_rel_err(e, st.interior("e")) <= FP64_TOL
        assert abs(dt[0] - hm.mesh.dt) <= FP64_TOL * hm.mesh.dt
        m0 = float(p.interior(p.rho).sum())
        assert abs(tot[0] - m0) <= 1e-13 * m0


def test_batch_rejects_bad_arguments(fg):
    import ctypes
    L = fg.lib()
    h = ctypes.c_void_p()
    one = (ctypes.c_int * 1)(1)
    assert L.gb300_batch_create(1, one, one, None, None, 0, ctypes.byref(h)) == 2
    L.gb300_batch_clear = None
    fg.lib().gb300_clear_error()


@pytest.mark.parametrize("use_graph", [False, True])
def test_bounded_barrier_runs_out_and_recovers(fg, use_graph):
    """A grid barrier of the persistent kernel whose wait bound is zero naps
    runs out in every block that is not the last to arrive: the kernel records
    GB300_ERR_TIMEOUT in its status word and every block returns (no hang, no
    fault), the status call reports the timeout and re-arms the barrier, and
    with the default bound restored the same batch steps again and reports
    GB300_OK; a fresh batch from the same problems then still matches the
    single-problem step."""
    probs = ensemble()
    b = fg.Batch(probs, precision=0)
    b.set_schedule(1)  # the persistent schedule (the one with grid barriers)
    b.set_spin_limit(0)
    b.step(2, use_graph=use_graph)
    assert b.status_code() == fg.GB300_ERR_TIMEOUT
    assert "timed out" in fg.lib().gb300_last_error_message().decode()
    fg.lib().gb300_clear_error()
    b.set_spin_limit(1 << 25)
    b.step(2, use_graph=use_graph)
    assert b.status_code() == fg.GB300_OK
    # The context is usable: a new batch advances exactly like the
    # single-problem step.
    b2 = fg.Batch(probs, precision=0)
    b2.step(3, use_graph=use_graph)
    b2.status()
    for i, p in enumerate(probs):
        rho, e, _, _ = b2.state(i)
        ref = single(fg, p, 3, 0)
        assert np.array_equal(rho, ref.interior("rho")) and np.array_equal(e, ref.interior("e"))
