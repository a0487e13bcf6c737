"""Ensembles of disks spread over the GPUs of one node.

The disks of an ensemble are independent, so they shard with no exchange on
the data path: each rank (one process per GPU) advances a disjoint subset
of the disks, and the ranks only gather their metrics on the host at the
end.  This replaces, for ensembles, the reference's MPI radial-ring split of
one disk (src_main/split.c, commbound.c, mpiTasks.c), which is not needed
because one GPU holds even a 2048x6144 disk.

The partition is the longest-processing-time rule on the disks' cell counts
(the cost of a DT grows with the cells): largest disk first, each to the
rank with the least work so far, ties to the lower rank.  It is
deterministic, so every rank computes the same partition without talking
to the others.
"""
from __future__ import annotations


def partition(cells: list, world: int) -> list:
    """Disk indices per rank: LPT on cells, deterministic."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    load = [0] * world
    shards = [[] for _ in range(world)]
    for k in sorted(range(len(cells)), key=lambda i: (-cells[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(k)
        load[r] += cells[k]
    for s in shards:
        s.sort()
    return shards


def shard_of(cells: list, rank: int, world: int) -> list:
    return partition(cells, world)[rank]


def gather_metrics(local: dict) -> list:
    """Every rank's metric dict, in rank order, on every rank (a host-side
    gather over the default process group; with no group, just [local])."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [local]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, local)
    return out


def combine(metrics: list) -> dict:
    """Whole-job figures from the per-rank metrics of one timed phase: the
    cell updates add up, the time is the slowest rank's."""
    upd = sum(m["cell_updates"] for m in metrics)
    sec = max(m["seconds"] for m in metrics)
    return {"ranks": len(metrics), "disks": sum(m["disks"] for m in metrics), "cell_updates": upd,
            "seconds": sec, "value": upd / sec if sec > 0 else 0.0,
            "per_rank_disks": [m["disks"] for m in metrics], "per_rank_cells": [m["cells"] for m in metrics]}
