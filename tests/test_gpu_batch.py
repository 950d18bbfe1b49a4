"""Batched solver: many independent instances in one launch, every value
exact against the oracle."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def mixed_instances(k=60, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        kind = i % 5
        if kind == 0:
            out.append(W.gen_genrmf(int(rng.integers(3, 9)), int(rng.integers(2, 10)), 1, 10000, i))
        elif kind == 1:
            out.append(W.gen_layered(int(rng.integers(2, 12)), int(rng.integers(4, 40)), 3, 6, 1, 1000, i))
        elif kind == 2:
            n = int(rng.integers(2, 200))
            m = int(rng.integers(0, 6 * n))
            out.append(W.Graph.from_arcs(n, rng.integers(0, n, m), rng.integers(0, n, m),
                                         rng.integers(0, 50, m), 0, n - 1))
        elif kind == 3:
            out.append(W.gen_grid(int(rng.integers(3, 20)), int(rng.integers(3, 20)), i))
        else:
            out.append(W.gen_bipartite(int(rng.integers(5, 300)), int(rng.integers(5, 300)), 2.0, 64, i))
    return out


def test_batch_exact_all_tunings():
    gs = mixed_instances()
    expected = np.array([oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) for g in gs])
    with W.Batch(gs) as b:
        for tile in (8, 16, 32):
            for block in (128, 256, 512):
                flows, ms = b.solve(tile=tile, block=block)
                assert np.array_equal(flows, expected), (tile, block)
                assert ms > 0
        flows, _ = b.solve(gr_alpha=8.0, gr_rounds=4)
        assert np.array_equal(flows, expected)
        ms_i, rounds = b.instance_stats()
        assert (ms_i > 0).all() and (rounds >= 0).all()
        best, best_ms = b.autotune()
        assert best.tile in (8, 16, 32) and best_ms > 0
        flows, _ = b.solve(best)
        assert np.array_equal(flows, expected)


def test_batch_matches_single_solves_on_larger_instances():
    gs = [W.gen_genrmf(24, 20, 1, 10000, 5), W.gen_layered(40, 300, 3, 6, 1, 1000, 6), W.gen_rmat(13, 8, seed=2)]
    with W.Batch(gs) as b:
        flows, _ = b.solve()
    for g, f in zip(gs, flows):
        assert f == W.maxflow(g) == oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)


def test_batch_budget_reports_failed_instances():
    gs = mixed_instances(10, seed=9)
    with W.Batch(gs) as b:
        with pytest.raises(W.WbprError) as ei:
            b.solve(max_rounds=1, gr_alpha=1e9, gr_rounds=1 << 20)
        assert ei.value.status == 3
        flows, _ = b.solve()
        assert (flows >= 0).all()


def test_batch_clusters_exact():
    """Instances from a size threshold on run on 8-block thread-block
    clusters (distributed shared-memory control words, cluster barriers):
    every threshold, tile and block size gives the oracle's flows."""
    gs = mixed_instances(80, seed=5) + [W.gen_genrmf(12, 10, 1, 10000, 1), W.gen_layered(30, 200, 3, 6, 1, 1000, 2)]
    expected = np.array([oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) for g in gs])
    with W.Batch(gs) as b:
        for cl in (1, 200, 2000, 20000, -1):
            for tile, block in ((8, 512), (16, 256), (32, 128)):
                flows, ms = b.solve(tile=tile, block=block, batch_cluster=cl)
                assert np.array_equal(flows, expected), (cl, tile, block)
        ms_i, rounds = b.instance_stats()
        assert (ms_i > 0).all()
        with pytest.raises(W.WbprError) as ei:
            b.solve(max_rounds=1, gr_alpha=1e9, gr_rounds=1 << 20, batch_cluster=1)
        assert ei.value.status == 3
        flows, _ = b.solve(batch_cluster=1)
        assert np.array_equal(flows, expected)
