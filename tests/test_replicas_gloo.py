"""The multi-rank aggregation of bench.py (replicas: total work over the max-over-ranks time),
run as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench._max_over_ranks(dist, None, 1.0 + rank)
        s = bench._sum_over_ranks(dist, None, 10.0 * (rank + 1))
        bench._barrier(dist, None)
        out[rank] = (t, s)
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    assert out[0] == (2.0, 30.0) and out[1] == (2.0, 30.0)
