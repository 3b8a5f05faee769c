"""Replica sharding across GPUs (one process per GPU).

The batched workload is a set of independent brush channels, so the step shards by replica with
no exchange at all: each rank advances its own replicas in its own context.  The global set of
replica shapes is drawn from the seed on every rank (cheap), split by greedy atom-count balancing
(longest-processing-time first), and each rank generates only its own replicas.  The only
collectives are host-side: the maximum of the per-rank timings and an end-of-run gather of
per-replica observables to rank 0.
"""
import numpy as np

from . import configs


def estimated_atoms(shape, rho=0.8):
    """Particle count of a replica shape (sigma_g, N, D, L): the channel filled to density rho."""
    sg, n, d, l = shape
    return rho * l * l * d


def partition(weights, world):
    """Greedy LPT split of items with the given weights into `world` parts.

    Items are taken heaviest first (ties by index) and each goes to the currently lightest part
    (ties by rank), so the result is deterministic.  Returns one ascending index list per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda k: (-float(weights[k]), k))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += float(weights[k])
    return [sorted(p) for p in parts]


def rank_replicas(n_per_rank, seed, rank, world, rho=0.8):
    """This rank's replicas of a global set of n_per_rank*world replicas drawn from the seed.

    Returns (global indices, replicas) with replicas as configs.replicas builds them; replica k
    of the global set is the same whatever the world size."""
    shapes = configs.draw_replica_shapes(n_per_rank * world, seed, rho)
    mine = partition([estimated_atoms(s, rho) for s in shapes], world)[rank]
    return mine, configs.replicas(seed=seed, rho=rho, shapes=shapes, indices=mine)


def max_over_ranks(t, dist=None, device=None):
    """Maximum of a per-rank float (a timing) over all ranks; t itself without a process group."""
    if dist is None or not dist.is_initialized():
        return float(t)
    import torch
    x = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def gather_per_replica(values, indices, n_total, dist=None):
    """Reassembles per-replica rows (values[k] belongs to global replica indices[k]) on rank 0.

    Returns an array of n_total rows in global replica order on rank 0 (and on a single
    process), None on the other ranks."""
    values = np.asarray(values)
    if dist is None or not dist.is_initialized():
        out = np.zeros((n_total,) + values.shape[1:], values.dtype)
        out[np.asarray(indices, dtype=np.int64)] = values
        return out
    world = dist.get_world_size()
    got = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object((list(indices), values), got, dst=0)
    if dist.get_rank() != 0:
        return None
    out = np.zeros((n_total,) + values.shape[1:], values.dtype)
    seen = np.zeros(n_total, bool)
    for idx, vals in got:
        idx = np.asarray(idx, dtype=np.int64)
        if seen[idx].any():
            raise RuntimeError("a replica was reported by two ranks")
        seen[idx] = True
        out[idx] = vals
    if not seen.all():
        raise RuntimeError("replicas missing from the gather: %s" % np.flatnonzero(~seen)[:8])
    return out
