"""Multi-process sharding on the CPU: two gloo ranks each trace their ray ranges
with the CPU oracle and sum the tallies; the sum equals one single-process run."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from rayfactorcl_gb300.shard import shard_ranges


def test_shard_ranges_cover_every_ray_once():
    rays = np.array([0, 1, 3, 4, 5, 4097, 123457, 10**9 + 3])
    for world in (1, 2, 3, 8):
        seen = np.zeros_like(rays)
        prev_end = np.zeros_like(rays)
        for r in range(world):
            first, count = shard_ranges(rays, r, world)
            assert np.all(first == prev_end)                       # contiguous, in order
            assert np.all((first % 4 == 0) | (count == 0))          # on draw boundaries
            prev_end = first + count
            seen += count
        assert np.array_equal(seen, rays)
    with pytest.raises(ValueError):
        shard_ranges(rays, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    import torch.distributed as dist
    from helpers import golden_scene
    from oracle import oracle as O
    from rayfactorcl_gb300.shard import trace_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = golden_scene("gen_mixed64")
    p = O.params(compat=0)
    rays = np.full(sc.n, 1001, np.int64)
    rays[3] = 0

    def trace_range(first, count):
        hits = np.zeros((sc.n, sc.n), np.int64)
        for e in range(sc.n):
            if count[e]:
                h = O.trace_rays(sc, p, e, int(first[e]), int(first[e] + count[e]), threads=1)
                hits[e] += np.bincount(h[h >= 0], minlength=sc.n)
        return hits

    hits, F = trace_sharded(trace_range, rays)
    if rank == 0:
        np.save(out_path, hits)
    dist.destroy_process_group()


def test_two_rank_gloo_sum_equals_single_run(oracle_lib, tmp_path):
    from helpers import golden_scene
    from oracle import oracle as O
    out = str(tmp_path / "hits.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    sc = golden_scene("gen_mixed64")
    rays = np.full(sc.n, 1001, np.int64)
    rays[3] = 0
    single = O.tally(sc, O.params(compat=0), rays)
    assert np.array_equal(np.load(out), single)
