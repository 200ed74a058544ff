"""Running the timestep on several GPUs of one node.

A single mesh does not shard without the reference's MPI halo exchange (the
arch layer's domain decomposition, out of scope here), so N GPUs run N
independent replicas of the single-mesh step: no collective touches the data
path.  Batched ensembles shard by instance.  The only collectives are the
barriers around the timed region and the max-over-ranks reduction of its
duration, which turns per-rank times into one whole-job throughput.

Launch one process per GPU (torchrun); RANK / WORLD_SIZE / LOCAL_RANK come
from the environment, and the process group (NCCL on GPUs, gloo on CPU) is
created by the caller.
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def _group_ready() -> bool:
    import torch.distributed as dist
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def barrier() -> None:
    """Barrier over all ranks (no-op for a single process)."""
    if _group_ready():
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """The largest of every rank's value (all ranks get it); the job's time is
    its slowest rank's."""
    if not _group_ready():
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device: str = "cpu") -> float:
    """The sum of every rank's value (all ranks get it)."""
    if not _group_ready():
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard_instances(cells: list[int], rank: int, world: int) -> list[int]:
    """Indices of the instances rank `rank` of `world` advances: largest
    first, each to the rank with the fewest cells so far (ties to the lower
    rank), so every rank gets a near-equal share of the ensemble's cells.
    Deterministic; the shards partition range(len(cells))."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    load = [0] * world
    owner = [0] * len(cells)
    for i in sorted(range(len(cells)), key=lambda k: (-cells[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += cells[i]
    return [i for i in range(len(cells)) if owner[i] == rank]


def job_throughput(units_per_rank: list[float] | float, world: int, seconds: float) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    total = sum(units_per_rank) if isinstance(units_per_rank, list) else units_per_rank * world
    return total / seconds
