"""The multi-GPU path of bench.py is replicas only (weak scaling): each rank
solves its own seeded batch and the whole-job figure is the sum of the
ranks' solves over the slowest rank's time.  The host logic runs here as two
gloo ranks on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        orders, seed = bench.rank_shard(64, rank)
        # rank r: r + 10 accepted solves in (r + 1) * 100 ms
        acc, ms = bench.whole_job(rank + 10, (rank + 1) * 100.0, world, "cpu")
        out[rank] = (list(map(int, orders)), seed, acc, ms)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    (o0, s0, a0, m0), (o1, s1, a1, m1) = out[0], out[1]
    assert s0 != s1 and o0 != o1                 # each rank its own batch
    assert len(o0) == len(o1) == 64
    assert min(o0 + o1) >= 16 and max(o0 + o1) <= 512
    assert a0 == a1 == 21.0                      # 10 + 11 solves in total
    assert m0 == m1 == 200.0                     # the slowest rank's time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job(5, 12.5, 1, "cpu") == (5.0, 12.5)
    o_a, _ = bench.rank_shard(32, 0)
    o_b, _ = bench.rank_shard(32, 0)
    assert np.array_equal(o_a, o_b)              # deterministic per rank
