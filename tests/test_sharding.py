"""CPU: the N-replica query sharding, as world_size-2 gloo process groups.

Each rank computes its contiguous shard of the queries (here with the oracle,
the CPU stand-in for a rank's GPU) and the shards are gathered; the result must
equal the single-process answer bit for bit.  A rank that fails must surface
as an error on the others, not a hang."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from axom_gb300.sharding import shard_bounds


def test_shard_bounds_partition():
    for m in (0, 1, 7, 100, 12345):
        for world in (1, 2, 3, 8):
            ranges = [shard_bounds(m, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == m
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q, v, f, out_path, fail_rank):
    import torch
    import torch.distributed as dist

    import oracle
    from axom_gb300.sharding import gather_shards

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        if rank == fail_rank:
            raise RuntimeError("injected rank failure")
        lo, hi = shard_bounds(q.shape[0], rank, world)
        port_ = oracle.Port()
        h = port_.sdf(v[:, 0], v[:, 1], v[:, 2], f)
        d, _, _ = port_.sdf_eval(h, q[lo:hi])
        full = gather_shards(torch.from_numpy(d), q.shape[0], rank, world)
        if rank == 0:
            np.save(out_path, full.numpy())
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_sdf_equals_single(tmp_path, port):
    from axom_gb300 import workloads as W
    v, f = W.displaced_icosphere(3, 1)
    q = W.uniform_queries(v, 3001, 2)
    out = tmp_path / "d.npy"
    mp.start_processes(_worker, args=(2, _free_port(), q, v, f, str(out), -1), nprocs=2, join=True,
                       start_method="spawn")
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    ref, _, _ = port.sdf_eval(h, q)
    got = np.load(out)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


def test_failed_rank_is_reported(tmp_path):
    from axom_gb300 import workloads as W
    v, f = W.displaced_icosphere(2, 1)
    q = W.uniform_queries(v, 100, 2)
    os.environ["TORCH_GLOO_TIMEOUT"] = "20"
    with pytest.raises(Exception):
        mp.start_processes(_worker, args=(2, _free_port(), q, v, f, str(tmp_path / "x.npy"), 1), nprocs=2,
                           join=True, start_method="spawn")
