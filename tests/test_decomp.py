"""Single-mesh domain decomposition on CPU: the oracle's timestep (the C
restatement of omp3/flow.c) run as world_size-2 and -3 gloo process groups,
each rank holding a band of rows and exchanging its ghost layers through the
transport of flow_gb300.decomp (the hooks the kernel set calls), must equal
the single-rank oracle bit for bit in every field after every step tested.
This pins the decomposition itself -- the bands, the neighbours, which rows
of cell, x-face and y-face arrays go where, the order of wall fills and
exchange, the all-reduced CFL minimum -- independently of the GPU."""
import os
import socket

import numpy as np
import pytest

from flow_gb300 import decomp

STATE = ("rho", "e", "u", "v", "rho_u", "rho_v")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def band_oracle(prob, rank, world, hooks, transport):
    """One rank's oracle state for its band, ghosts filled by the exchange."""
    from oracle import oracle as O
    y_off, rows = decomp.row_bands(prob.gny, world)[rank]
    band = decomp.BandProblem(prob, y_off, rows)
    hm = O.HostMesh(prob.gnx, rows, width=prob.width, height=prob.height, dt=prob.dt_param)
    hm.edgey[:] = band.edgey
    hm.edgedy[:] = band.edgedy
    hm.celldy[:] = band.celldy
    decomp.set_rank_mesh(hm.mesh, rank, world, y_off)
    st = O.HostState(hm)
    hooks.bind(decomp.RankContext(rank, world, transport, decomp.numpy_resolver(st.a)))
    O.fill_fields(hm, st, band.interior(band.rho), band.interior(band.e))
    return hm, st


def _rank_main(rank: int, world: int, port: int, out_dir: str, case: str, steps: int) -> None:
    import torch.distributed as dist

    from oracle import oracle as O
    from flow_gb300 import problems

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prob = {"sedov": lambda: problems.sedov(48),
                "two_region": lambda: problems.two_region(50, np.random.default_rng(3))}[case]()
        hooks = decomp.Hooks(O.Mesh)
        L = O.lib("port")
        L.flow_shim_set_halo(hooks.halo, None)
        L.flow_shim_set_reduce_min(hooks.min, None)
        hm, st = band_oracle(prob, rank, world, hooks, decomp.DistTransport())
        O.initial_timestep(hm, st)
        out = {}
        for tt in range(steps):
            O.step(hm, st, tt)
            out[f"dt{tt}"] = np.array([hm.mesh.dt, hm.mesh.dt_h])
        for k in STATE:
            a = st.interior(k)
            if k in ("v", "rho_v") and rank < world - 1:
                a = a[:-1]  # the face above the band is the next band's first
            out[k] = a
        assert not hooks.errors, hooks.errors
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), **out)
    finally:
        dist.destroy_process_group()


def single_rank(case, steps):
    from oracle import oracle as O
    from flow_gb300 import problems
    prob = {"sedov": lambda: problems.sedov(48),
            "two_region": lambda: problems.two_region(50, np.random.default_rng(3))}[case]()
    hm = O.HostMesh(prob.gnx, prob.gny, dt=prob.dt_param)
    st = O.HostState(hm)
    O.fill_fields(hm, st, prob.interior(prob.rho), prob.interior(prob.e))
    O.initial_timestep(hm, st)
    dts = []
    for tt in range(steps):
        O.step(hm, st, tt)
        dts.append((hm.mesh.dt, hm.mesh.dt_h))
    return st, dts


@pytest.mark.timeout(300)
@pytest.mark.parametrize("world,case", [(2, "sedov"), (3, "two_region")])
def test_decomposed_oracle_matches_single_rank(tmp_path, world, case):
    import torch.multiprocessing as mp
    steps = 12
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path), case, steps), nprocs=world,
             join=True)
    parts = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    st, dts = single_rank(case, steps)
    for tt in range(steps):
        for p in parts:
            assert tuple(p[f"dt{tt}"]) == dts[tt], tt
    for k in STATE:
        got = np.concatenate([p[k] for p in parts], axis=0)
        want = st.interior(k)
        assert got.shape == want.shape, k
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), \
            (k, int(np.count_nonzero(got != want)))


def test_bands_and_halo_rows():
    assert decomp.row_bands(10, 2) == [(0, 5), (5, 5)]
    assert decomp.row_bands(13, 3) == [(0, 5), (5, 4), (9, 4)]
    with pytest.raises(ValueError):
        decomp.row_bands(7, 2)
    assert decomp.neighbours(0, 3) == [1, -1, -1, -1]
    assert decomp.neighbours(1, 3) == [2, -1, 0, -1]
    # cell arrays (h = local_ny = 9): first/last two interior rows
    assert decomp.halo_rows(9, 9, decomp.FLOW_SOUTH) == (slice(2, 4), slice(0, 2))
    assert decomp.halo_rows(9, 9, decomp.FLOW_NORTH) == (slice(5, 7), slice(7, 9))
    # y-face arrays (h = local_ny + 1): shifted past the shared face
    assert decomp.halo_rows(10, 9, decomp.FLOW_SOUTH) == (slice(3, 5), slice(0, 2))
    assert decomp.halo_rows(10, 9, decomp.FLOW_NORTH) == (slice(5, 7), slice(8, 10))
