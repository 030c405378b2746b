"""Replicas on several GPUs: one process per GPU, independent units of work.

Every unit of this path (a cluster, a wavelength of a sweep, a request of the
stream) is an independent solve, so several GPUs work as replicas: the units are
split over the ranks once, each rank solves its share on its own GPU with the
single-GPU code, and the only communication is host-side bookkeeping at the end
(the slowest rank's time, the gathered results).  There is no collective on the
data path.  The reference has no multi-device support (OpenMP on one host).
"""

from __future__ import annotations

import numpy as np

from .modes import lmax_to_rmax


def unit_cost(N, lmax, iterations=1.0):
    """Relative cost of one cluster solve: matrix elements streamed per product
    (packed pair blocks) plus the vector work."""
    B = 2 * lmax_to_rmax(int(lmax))
    return iterations * (N * (N - 1) / 2 * B * B + 16.0 * N * B)


def shard_balanced(costs, world):
    """Split units over world ranks, largest first onto the least loaded rank
    (ties to the lower rank): deterministic, the same on every rank.  Returns one
    sorted index list per rank."""
    costs = np.asarray(costs, float)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    parts = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def my_shard(costs, rank, world):
    return shard_balanced(costs, world)[rank]


def max_over_ranks(value, device=None):
    """The largest value over all ranks (the slowest replica's time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_objects(obj):
    """Every rank's object, in rank order (host-side pickles)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def aggregate_throughput(units_per_rank, seconds_per_rank):
    """Whole-job units/s: every rank's units over the slowest rank's time."""
    return float(np.sum(units_per_rank)) / float(np.max(seconds_per_rank))


def merge_sweeps(parts):
    """Concatenate SweepResult parts of disjoint wavelength shards, sorted by wavelength."""
    from .sweep import SweepResult
    wl = np.concatenate([p.wavelength for p in parts])
    order = np.argsort(wl, kind="stable")
    cat = lambda name: np.concatenate([getattr(p, name) for p in parts])[order]
    return SweepResult(wavelength=wl[order], lmax=cat("lmax"), C_sca=cat("C_sca"), C_abs=cat("C_abs"),
                       C_ext=cat("C_ext"), status=cat("status"), iterations=cat("iterations"))
