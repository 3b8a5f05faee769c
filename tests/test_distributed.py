"""Multi-rank host logic on CPU: two gloo ranks shard a replica set, time, and gather.

The GPU step itself has no exchange (replicas are independent), so what needs checking with
more than one rank is the host side: every replica owned by exactly one rank, each rank's
replicas identical to the single-process ones, the max-over-ranks timing, and the end-of-run
gather of per-replica observables in global order."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mfa_brush_gb300 import configs, shard

SEED, PER_RANK, WORLD = 5, 4, 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _observables(reps):
    """Per-replica rows: particle count, mobile count, sum of positions (a fingerprint)."""
    return np.array([[r[0].n_part, r[0].n_mon_tot, float(np.sum(r[2]))] for r in reps])


def _worker(rank, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        idx, reps = shard.rank_replicas(PER_RANK, SEED, rank, WORLD)
        t = shard.max_over_ranks(1.0 + rank, dist)
        full = shard.gather_per_replica(_observables(reps), idx, PER_RANK * WORLD, dist)
        np.save(os.path.join(out_dir, "idx%d.npy" % rank), np.asarray(idx))
        np.save(os.path.join(out_dir, "t%d.npy" % rank), np.asarray([t]))
        if rank == 0:
            np.save(os.path.join(out_dir, "full.npy"), full)
        else:
            assert full is None
    finally:
        dist.destroy_process_group()


def test_partition_is_balanced_and_deterministic():
    w = [5, 1, 4, 2, 3, 3, 8, 1]
    parts = shard.partition(w, 3)
    assert sorted(k for p in parts for k in p) == list(range(len(w)))
    loads = [sum(w[k] for k in p) for p in parts]
    assert max(loads) - min(loads) <= max(w)
    assert parts == shard.partition(w, 3)
    assert shard.partition(w, 1) == [list(range(len(w)))]


def test_single_process_gather_orders_rows():
    vals = np.array([[10.0], [20.0], [30.0]])
    out = shard.gather_per_replica(vals, [2, 0, 1], 3)
    assert out[:, 0].tolist() == [20.0, 30.0, 10.0]


def test_two_gloo_ranks_shard_time_and_gather(tmp_path):
    mp.spawn(_worker, args=(_free_port(), str(tmp_path)), nprocs=WORLD, join=True)
    idx = [np.load(tmp_path / ("idx%d.npy" % r)).tolist() for r in range(WORLD)]
    assert sorted(idx[0] + idx[1]) == list(range(PER_RANK * WORLD))
    assert not set(idx[0]) & set(idx[1])
    # the timing reduction is the maximum on every rank
    assert [float(np.load(tmp_path / ("t%d.npy" % r))[0]) for r in range(WORLD)] == [2.0, 2.0]
    # rank 0 holds every replica's observables in global order, equal to a single-process build
    full = np.load(tmp_path / "full.npy")
    shapes = configs.draw_replica_shapes(PER_RANK * WORLD, SEED)
    ref = _observables(configs.replicas(seed=SEED, shapes=shapes))
    assert np.array_equal(full, ref)
