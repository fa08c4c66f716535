"""Multi-GPU layout of the PBF step: replicas and independent scenes, no data exchange.

A PBF scene steps on one GPU; nothing in the step exchanges data between scenes.  N GPUs therefore
run N replicas (one scene each) or split a set of independent scenes between them, and the only
collectives are host-side bookkeeping: a barrier around the timed region and the maximum of the
ranks' elapsed times.  One process per GPU; rank, world size and rendezvous come from the
environment torchrun sets (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR, MASTER_PORT).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class DistEnv:
    world: int
    rank: int
    local_rank: int


def dist_env() -> DistEnv:
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad RANK/WORLD_SIZE: %d/%d" % (rank, world))
    return DistEnv(world, rank, local)


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of rank `rank`'s replica: every rank steps its own jittered copy of the workload."""
    return base_seed + 1000003 * rank


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over all ranks (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, elapsed_s: float, world: int) -> float:
    """Whole-job throughput: units all ranks processed over the slowest rank's time."""
    if elapsed_s <= 0:
        raise ValueError("elapsed time must be positive")
    return units_per_rank * world / elapsed_s


def shard_scenes(particle_counts, world: int) -> list[list[int]]:
    """Splits independent scenes between `world` ranks, balancing particles: scenes are taken
    largest first and each goes to the rank with the fewest particles so far (ties to the lower
    rank).  Deterministic; returns each rank's scene indices in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    order = sorted(range(len(particle_counts)), key=lambda s: (-int(particle_counts[s]), s))
    for s in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(s)
        load[r] += int(particle_counts[s])
    return [sorted(v) for v in out]
