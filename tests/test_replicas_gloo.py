"""bench.py's multi-GPU mode runs independent replicas and takes the max
time over ranks; its rank plumbing (torch.distributed over gloo, world
size 2) is exercised here on the CPU."""
import os
import sys

import pytest


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, l = bench.dist_setup(world)
    bench.barrier(w)
    m = bench.allreduce_max(float(10 * (r + 1)), w)
    q.put((r, w, m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2, 20.0), (1, 2, 20.0)]
