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


# ---------------------------------------------------------------------------
# Batch sharding: instances split by estimated work, flows gathered on rank 0.
def test_partition_covers_every_instance_once_and_balances():
    from wbpr_gb300 import shard

    rng = __import__("numpy").random.default_rng(0)
    works = list(rng.pareto(1.5, 997) + 1)
    for world in (1, 2, 3, 8):
        parts = shard.partition(works, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(works)))
        loads = [sum(works[i] for i in p) for p in parts]
        # longest-first greedy: no shard exceeds the mean by more than the largest instance
        assert max(loads) <= sum(works) / world + max(works) + 1e-9


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist

    import oracle
    from wbpr_gb300 import shard, workloads as WL

    dist.init_process_group("gloo")
    graphs = WL.config3(24)

    def solve_shard(gs):  # the CPU oracle stands in for the batched GPU solve
        return np.array([oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) for g in gs], np.int64)

    flows, mine, _ = shard.solve_sharded(graphs, rank, world, solve_shard, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, mine, None if flows is None else flows.tolist()))


def test_sharded_batch_gathers_exact_flows_on_rank_0():
    import numpy as np

    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    res = {r: (mine, fl) for r, mine, fl in (q.get(timeout=10) for _ in range(2))}
    sys.path.insert(0, ROOT)
    import oracle
    from wbpr_gb300 import workloads as WL

    graphs = WL.config3(24)
    want = [oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) for g in graphs]
    assert res[1][1] is None and res[0][1] == want
    assert sorted(res[0][0] + res[1][0]) == list(range(24)) and res[0][0] and res[1][0]
    # the pinned full-size values of these instances agree too
    import json
    pins = json.load(open(os.path.join(ROOT, "tests", "golden", "fullsize.json")))
    assert np.array_equal(pins["config3"]["flows"][:24], want)
