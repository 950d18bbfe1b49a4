"""Batched instances sharded across ranks (one process per GPU).

Instances of a batch are independent, so a batch splits across ranks with no
exchange on the data path: every rank solves the instances of its shard in
one batched launch (wbpr_batch_*), and the int64 flows are gathered to rank 0
on the host afterwards, back in the batch's order.  Shards are balanced by an
estimate of each instance's work, m * log2(U + 1) + n with U its largest
capacity (push-relabel's scan work grows with the arcs and, through the
number of relabels, with the capacity range), by the longest-first greedy
rule: instances in decreasing work, each to the rank with the least work so
far.  The single-instance solver does not shard (push-relabel exchanges labels
and excess every round): there, ranks run replicas.
"""
from __future__ import annotations

import heapq
import math

import numpy as np


def estimated_work(g) -> float:
    u = int(np.max(g.cap)) if g.m else 0
    return float(g.m) * math.log2(u + 1.0) + float(g.n)


def partition(works, world: int) -> list[list[int]]:
    """Indices of each rank's shard (longest-first greedy); every index once,
    each shard in increasing index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(works)), key=lambda k: (-works[k], k)):
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + works[i], r))
    return [sorted(p) for p in parts]


def gather_flows(count: int, mine: list[int], flows, rank: int, world: int, dist=None):
    """Flows of every shard on rank 0, in batch order (None on other ranks).
    `dist` is torch.distributed with an initialised process group (any
    backend that gathers Python objects: gloo on the host)."""
    local = (list(mine), [int(x) for x in np.asarray(flows, np.int64)])
    if world == 1:
        parts = [local]
    else:
        parts = [None] * world if rank == 0 else None
        dist.gather_object(local, parts, dst=0)
    if rank != 0:
        return None
    out = np.full(count, -1, np.int64)
    seen = np.zeros(count, bool)
    for idx, fl in parts:
        if len(idx) != len(fl):
            raise ValueError("a shard returned a flow count different from its instances")
        for i, f in zip(idx, fl):
            if seen[i]:
                raise ValueError(f"instance {i} solved by two ranks")
            seen[i] = True
            out[i] = f
    if not seen.all():
        raise ValueError("some instances were solved by no rank")
    return out


def solve_sharded(graphs, rank: int, world: int, solve_shard, dist=None):
    """Solve this rank's shard with solve_shard(list of graphs) -> int64 flows
    and gather every flow to rank 0.  Returns (flows on rank 0 or None, this
    rank's indices, whatever else solve_shard returned)."""
    parts = partition([estimated_work(g) for g in graphs], world)
    mine = parts[rank]
    res = solve_shard([graphs[i] for i in mine])
    flows, extra = (res[0], res[1:]) if isinstance(res, tuple) else (res, ())
    return gather_flows(len(graphs), mine, flows, rank, world, dist), mine, extra
