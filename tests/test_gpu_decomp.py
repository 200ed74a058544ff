"""The decomposed GPU timestep: one mesh split into bands of rows, each band a
rank running the kernel set's exact mode with its ghost layers exchanged
through the library's halo and minimum hooks (flow_gb300.decomp).  The ranks
are threads of this process sharing one GPU (ThreadTransport): they meet on
the host between kernel launches, so no kernel waits on another.  Every field
and dt must equal the single-rank exact step bit for bit (which the other
tests hold equal to the oracle); the same hooks drive one process per GPU
over torch.distributed (DistTransport)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


@pytest.fixture(scope="module")
def fg():
    import flow_gb300
    from flow_gb300 import decomp
    L = flow_gb300.lib()
    hooks = decomp.Hooks(flow_gb300.Mesh)
    decomp.install(L, hooks)
    yield flow_gb300, hooks
    decomp.uninstall(L)
    flow_gb300.set_mode(flow_gb300.MODE_FUSED)


def run_ranks(fg, hooks, prob, nranks, steps):
    from flow_gb300 import decomp
    transport = decomp.ThreadTransport(nranks, timeout=120.0)
    results, errors = {}, []

    def rank_main(rank):
        try:
            fg.set_mode(fg.MODE_EXACT)  # the mode is per host thread
            sim = decomp.DecomposedSim(prob, rank, nranks, transport, hooks)
            sim.initial_timestep()
            dts = []
            for _ in range(steps):
                sim.step()
                dts.append((sim.sim.mesh.dt, sim.sim.mesh.dt_h))
            results[rank] = ({k: sim.interior(k) for k in STATE}, dts)
        except Exception as exc:  # surfaced below
            errors.append((rank, repr(exc), fg.lib().gb300_last_error_message()))

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(nranks)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors and not hooks.errors, (errors, hooks.errors)
    return results


def single_rank(fg, prob, steps):
    fg.set_mode(fg.MODE_EXACT)
    sim = fg.DeviceSim(prob)
    sim.initial_timestep()
    dts = []
    for _ in range(steps):
        sim.step()
        dts.append((sim.mesh.dt, sim.mesh.dt_h))
    return sim, dts


@pytest.mark.parametrize("nranks,case", [(2, "sedov"), (3, "two_region"), (4, "sod")])
def test_decomposed_step_matches_single_rank(fg, nranks, case):
    fgm, hooks = fg
    from flow_gb300 import problems
    prob = {"sedov": lambda: problems.sedov(64),
            "two_region": lambda: problems.two_region(70, np.random.default_rng(5)),
            "sod": lambda: problems.sod(60, 66)}[case]()
    steps = 15
    parts = run_ranks(fgm, hooks, prob, nranks, steps)
    ref, dts = single_rank(fgm, prob, steps)
    for r in range(nranks):
        assert parts[r][1] == dts, r
    for k in STATE:
        got = np.concatenate([parts[r][0][k] for r in range(nranks)], axis=0)
        want = ref.interior(k)
        assert got.shape == want.shape, k
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), \
            (k, int(np.count_nonzero(got != want)))


def test_fused_mode_rejects_a_decomposed_mesh(fg):
    fgm, hooks = fg
    from flow_gb300 import decomp, problems
    fgm.set_mode(fgm.MODE_FUSED)
    sim = fgm.DeviceSim(problems.sod(32, 32))
    decomp.set_rank_mesh(sim.mesh, 0, 2, 0)
    L = fgm.lib()
    L.gb300_clear_error()
    args = sim.args()
    rc = L.gb300_solve_hydro_2d(sim._mesh_ref, 0, *args)
    assert rc == fgm.GB300_ERR_ARG
    assert b"GB300_MODE_EXACT" in L.gb300_last_error_message()
    L.gb300_clear_error()
