"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks.

Replicas run their own structures with no data exchange (weak scaling); the
job's value is the sum of the ranks' terms over the slowest rank's time.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as tmp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        assert (r, w, local) == (rank, world, rank)
        # rank-dependent terms and timings: rank 1 is the slow one on the first timing, rank 0 on the second
        terms, times = bench.aggregate_ranks(1000 + rank, [2.0 + rank, 5.0 - rank, 1.5], w)
        q.put((rank, terms, times))
    finally:
        dist.destroy_process_group()


def test_replicas_aggregate_over_two_gloo_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, terms, times in out:
        assert terms == 2001.0
        assert times == [3.0, 5.0, 1.5]


def test_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    terms, times = bench.aggregate_ranks(7, [1.0, 2.0], 1)
    assert terms == 7.0 and times == [1.0, 2.0]
