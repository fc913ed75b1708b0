"""Replicas across GPUs.

Within one simulation the step does not shard: the spherical-harmonic step
needs every l at each r (and every r for each l) once per step, and the
cylindrical ADI step a z <-> rho transpose.  Simulations are independent, so
several GPUs run replicas: each rank (one process per GPU) advances its own
share of the simulations with no collective on the data path.  The only
cross-rank operations are a barrier around timed regions and the maximum of
the per-rank elapsed times.

* ``sweep_seed``: weak scaling — every rank runs its own seeded sweep of the
  same size (seed + rank);
* ``shard``: a fixed set of simulations or requests split round-robin, for a
  run that should cover the set exactly once across the ranks.
"""

import os
from typing import List, Sequence, TypeVar

T = TypeVar("T")


def rank_world():
    """(rank, world size, local rank) from the launcher's environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def sweep_seed(base_seed: int, rank: int) -> int:
    return int(base_seed) + int(rank)


def shard(items: Sequence[T], rank: int, world: int) -> List[T]:
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(items[rank::world])


def max_over_ranks(value: float) -> float:
    """The maximum of ``value`` over the ranks of the default process group
    (the value itself without one).  Uses the group's backend: NCCL on GPUs,
    gloo on CPU."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()
