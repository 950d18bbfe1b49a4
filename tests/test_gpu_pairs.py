"""Many instances in one solve (wbpr_solve_pairs): the instances are stored as
one disjoint-union graph, every instance's source and sink become terminals
of one multi-pair solve on the whole GPU, and each sink's final excess must
equal the oracle's maximum flow of its instance."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def instances():
    rng = np.random.default_rng(21)
    out = [W.gen_genrmf(int(a), int(b), 1, 1000, i) for i, (a, b) in enumerate([(3, 4), (5, 6), (8, 4), (4, 12)])]
    out += [W.gen_layered(int(rng.integers(3, 12)), int(rng.integers(4, 40)), 2, 5, 1, 100, 40 + i) for i in range(8)]
    out += [W.gen_grid(16, 12, 3), W.gen_bipartite(200, 150, 2.0, 32, 5), W.gen_rmat(10, 8, seed=2)]
    for i in range(6):  # parallel and antiparallel arcs, zero capacities
        n, m = int(rng.integers(2, 60)), int(rng.integers(0, 300))
        out.append(W.Graph.from_arcs(n, rng.integers(0, n, m), rng.integers(0, n, m), rng.integers(0, 7, m), 0, n - 1))
    return out


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_union_solve_matches_each_instance(layout):
    gs = instances()
    expect = [oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) for g in gs]
    u, src, snk = W.disjoint_union(gs)
    with W.DeviceGraph(u, layout) as d:
        for algo in ("vc", "tc"):
            for grid in (0, 4096):
                flows, r = d.solve_pairs(src, snk, algo, grid_blocks=grid)
                assert flows.tolist() == expect, (algo, grid)
                assert r.flow == sum(expect)
        # a plain single-pair solve on the same handle afterwards
        assert d.solve("vc", int(src[1]), int(snk[1])).flow == expect[1]
        rep = d.verify()
        assert rep["ok"]


def test_one_pair_equals_solve():
    g = W.gen_rmat(12, 8, seed=4)
    with W.DeviceGraph(g, "bcsr") as d:
        flows, _ = d.solve_pairs([g.s], [g.t])
        assert flows[0] == d.solve("vc", g.s, g.t).flow == oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)


def test_invalid_pairs_rejected():
    g = W.gen_genrmf(3, 3, 1, 10, 1)
    with W.DeviceGraph(g, "bcsr") as d:
        for src, snk in (([0, 0], [5, 6]), ([0], [0]), ([0], [g.n]), ([-1], [3])):
            with pytest.raises(W.WbprError) as ei:
                d.solve_pairs(src, snk)
            assert ei.value.status == 1
