"""Min-cut adjoint (wbpr_mincut_adjoint): the exact integer (super)gradient of
the maximum-flow value with respect to every arc capacity.

side 0 is the cut in front of the vertices that can reach t, side 1 the cut
behind the vertices reachable from s once stranded excess is returned; both
are unique for a given graph, so they must equal the oracle's extreme cuts
arc for arc.  Any minimum cut's indicator g satisfies the one-sided finite
differences f(c + e) - f(c) <= g_e <= f(c) - f(c - e), checked by re-solves."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def graphs():
    yield W.gen_genrmf(5, 6, 1, 100, 1)
    yield W.gen_grid(24, 24, 3)
    yield W.gen_layered(8, 20, 3, 6, 1, 50, 4)
    yield W.gen_bipartite(300, 300, 2.0, 4096, 2)
    yield W.gen_rmat(11, 8, seed=6)
    rng = np.random.default_rng(7)
    for _ in range(4):
        n = 60
        m = 300
        yield W.Graph.from_arcs(n, rng.integers(0, n, m), rng.integers(0, n, m), rng.integers(0, 9, m), 0, n - 1)


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_indicators_equal_oracle_extreme_cuts(layout):
    for g in graphs():
        v, sink_side, src_side = oracle.mincut(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, layout) as d:
            r = d.solve("vc", g.s, g.t)
            assert r.flow == v
            g0, _ = d.mincut_adjoint(0)
            assert np.array_equal(g0, sink_side)
            g1, _ = d.mincut_adjoint(1)
            assert np.array_equal(g1, src_side)
            # phase 2 left a valid maximum flow: same value, certificate holds
            rep = d.verify()
            assert rep["ok"] and rep["flow_value"] == v
            assert int((g0.astype(np.int64) * g.cap).sum()) == v
            assert int((g1.astype(np.int64) * g.cap).sum()) == v


def test_finite_differences():
    rng = np.random.default_rng(11)
    for g in (W.gen_genrmf(4, 5, 1, 60, 2), W.gen_grid(12, 12, 5)):
        base = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, "bcsr") as d:
            d.solve("vc", g.s, g.t)
            ind = [d.mincut_adjoint(0)[0], d.mincut_adjoint(1)[0]]
        for e in rng.choice(g.m, size=min(60, g.m), replace=False):
            up = g.cap.copy()
            up[e] += 1
            d_plus = oracle.dinic(g.n, g.off, g.dst, up, g.s, g.t) - base
            d_minus = 0
            if g.cap[e] > 0:
                dn = g.cap.copy()
                dn[e] -= 1
                d_minus = base - oracle.dinic(g.n, g.off, g.dst, dn, g.s, g.t)
            for gi in ind:
                assert d_plus <= gi[e], (e, d_plus, gi[e])
                if g.cap[e] > 0:
                    assert gi[e] <= d_minus, (e, gi[e], d_minus)
