"""The multi-GPU path on CPU: replicas of the single-mesh step and instance
shards of an ensemble, as world_size-2 gloo process groups.

Each rank advances its own replica (the oracle's timestep stands in for the
GPU step, which needs a device), the ranks agree on the slowest rank's time,
and the job throughput counts every rank's cells over that time -- the
aggregation bench.py uses under torchrun.  No collective touches the data.
"""
import os
import socket

import numpy as np
import pytest

from flow_gb300.replicas import job_throughput, max_over_ranks, shard_instances


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import time

    import torch.distributed as dist

    from oracle import oracle as O
    from flow_gb300.replicas import barrier, sum_over_ranks

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # A replica per rank: the same problem, independent state.
        hm = O.HostMesh(48, 40, dt=1e-3)
        st = O.HostState(hm)
        O.fill_boxes(hm, st, O.sod_boxes())
        O.initial_timestep(hm, st)
        barrier()
        t0 = time.perf_counter()
        O.run(hm, st, 5 + 5 * rank)  # uneven work: rank 1 is the slow one
        local = time.perf_counter() - t0
        slowest = max_over_ranks(local)
        shards_total = sum_over_ranks(rank + 1)  # 1 + 2
        barrier()
        mass = O.conservation(hm, st)[0]
        np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                np.array([local, slowest, mass, shards_total]))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_two_gloo_ranks_agree_on_the_slowest_replica(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    # Both ranks hold the same max, and it is the larger local time.
    assert r0[1] == r1[1] == max(r0[0], r1[0])
    # The replicas ran independently: each conserved its own mass.
    assert abs(r0[2] - r1[2]) <= 1e-13 * r0[2]
    assert r0[3] == r1[3] == 3.0
    cells = 48 * 40
    assert job_throughput(cells * 10, 2, r0[1]) == pytest.approx(2 * cells * 10 / r0[1])


def test_max_over_ranks_without_a_group_is_the_local_value():
    assert max_over_ranks(3.5) == 3.5


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_instance_shards_partition_and_balance(world):
    rng = np.random.default_rng(20261203)
    sides = rng.choice(np.arange(128, 1025, 64), size=256)
    cells = [int(n) * int(n) for n in sides]
    shards = [shard_instances(cells, r, world) for r in range(world)]
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(cells)))
    loads = [sum(cells[i] for i in s) for s in shards]
    # Greedy largest-first: no rank exceeds the mean by more than one instance.
    assert max(loads) - sum(loads) / world <= max(cells)
    assert shards == [shard_instances(cells, r, world) for r in range(world)]


def test_instance_shards_reject_bad_ranks():
    with pytest.raises(ValueError):
        shard_instances([1, 2], 2, 2)
