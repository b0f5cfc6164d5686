"""Sharding of independent solves across ranks (one process per GPU).

The batched small solves and the selector's labelling are sets of
independent systems: rank r takes a contiguous index range whose share of
the total work (sum of n^3 over its systems, the factorization cost) is as
close to 1/world as contiguous ranges allow.  Nothing on the data path is
exchanged; the per-system results (info, labels, timings) are gathered on
the host at the end (`gather`), over whatever process group is initialised
(gloo on CPU, NCCL on GPUs).
"""
import numpy as np


def balanced_ranges(work, world):
    """[(lo, hi)] for each rank: contiguous, covering 0..len(work), with the
    cut after the prefix whose cumulative work first reaches r/world of the
    total.  Ranks may be empty when there are fewer items than ranks."""
    work = np.asarray(work, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if np.any(work < 0):
        raise ValueError("work must be non-negative")
    n = len(work)
    cum = np.cumsum(work)
    total = cum[-1] if n else 0.0
    cuts = [0]
    for r in range(1, world):
        if total <= 0:
            c = (n * r) // world
        else:
            c = int(np.searchsorted(cum, total * r / world, side="left")) + 1
        cuts.append(min(max(c, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def shard(ns, rank, world, power=3):
    """This rank's (lo, hi) range of systems with sizes ns, balanced by n^power."""
    return balanced_ranges(np.asarray(ns, dtype=np.float64) ** power, world)[rank]


def gather(local, group=None):
    """All ranks' `local` objects in rank order (host-side all-gather); the
    single-process case returns [local]."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [local]
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, local, group=group)
    return out


def sharded_map(fn, items, work, rank, world, group=None):
    """fn applied to this rank's balanced range of items, results of all
    ranks concatenated in item order (every rank gets the full list)."""
    lo, hi = balanced_ranges(work, world)[rank]
    mine = [fn(it) for it in items[lo:hi]]
    parts = gather((lo, mine), group)
    out = [None] * len(items)
    for plo, res in parts:
        out[plo:plo + len(res)] = res
    return out
