"""Replica bookkeeping of bench.py across ranks (gloo, world size 2, CPU):
the barrier and the max-over-ranks reduction used for the whole-job time."""
import os
import socket
import sys

import torch.multiprocessing as tmp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(world)
    d.barrier()
    got = d.max(float(rank * 10 + 1))
    d.barrier()
    d.close()
    q.put((rank, got))


def test_replica_max_over_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 11.0, 1: 11.0}
