"""The matching kernel (wbpr_gb300/csrc/match.cu): unit-capacity bipartite
networks (s -> left -> right -> t, every capacity 1) are recognised at the
solve and matched by double-push rounds with alternating-path global
relabels, on both layouts.  Every flow is compared with the oracle's Dinic
value and with the general solver on the same handle (matching=-1); the state
left behind must pass the device certificate with valid labels, give a
maximum flow after wbpr_complete_flow, and let the next solve on the handle
start clean."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def dinic(g):
    return oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)


def network(L, R, pairs):
    pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
    return W.bipartite_network(L, R, pairs[:, 0], pairs[:, 1])


def random_pairs(rng, L, R, m):
    return np.stack([rng.integers(0, L, m), rng.integers(0, R, m)], axis=1)


def cases():
    rng = np.random.default_rng(11)
    yield "zipf_2000", W.gen_bipartite(2000, 2000, 2.0, 4096, 3)
    yield "zipf_30000", W.gen_bipartite(30000, 25000, 2.0, 4096, 4)
    yield "zipf_steep", W.gen_bipartite(5000, 8000, 4.0, 64, 5)
    yield "uniform_dense", network(300, 300, random_pairs(rng, 300, 300, 6000))
    yield "uniform_sparse", network(4000, 3000, random_pairs(rng, 4000, 3000, 5000))
    # a perfect matching along i -> i plus noise, shuffled
    p = np.concatenate([np.stack([np.arange(1000), np.arange(1000)], 1), random_pairs(rng, 1000, 1000, 3000)])
    yield "perfect_1000", network(1000, 1000, p[rng.permutation(len(p))])
    # parallel edges, one left vertex joined to every right vertex, every left
    # vertex joined to one right vertex
    yield "parallel", network(50, 40, np.concatenate([random_pairs(rng, 50, 40, 300)] * 3))
    yield "left_star", network(200, 500, np.stack([np.zeros(500, np.int64), np.arange(500)], 1))
    yield "right_star", network(500, 200, np.stack([np.arange(500), np.zeros(500, np.int64)], 1))
    # isolated vertices on both sides
    yield "isolated", network(100, 100, random_pairs(rng, 40, 30, 90))
    yield "single_edge", network(1, 1, [[0, 0]])
    # long augmenting paths: a chain x_i - y_i - x_{i+1} ... that a greedy
    # first pass matches wrongly
    k = 3000
    chain = [[i, i] for i in range(k)] + [[i + 1, i] for i in range(k - 1)]
    yield "chain", network(k, k, np.array(chain)[::-1])


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
@pytest.mark.parametrize("name,g", list(cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_matching_kernel_exact(name, g, layout):
    v = dinic(g)
    with W.DeviceGraph(g, layout) as d:
        r = d.solve("vc", g.s, g.t)
        assert r.matching == 1
        assert r.flow == v
        rep = d.verify()
        assert rep["ok"] and rep["flow_value"] == v
        assert rep["label_violations"] == 0
        h, e, f = d.read_state()
        inner = np.ones(g.n, bool)
        inner[[g.s, g.t]] = False
        assert np.all(e[inner] == 0) and e[g.t] == v
        assert np.all((h >= 0) & (h <= g.n)) and h[g.t] == 0 and h[g.s] == g.n
        # a flow already: every arc 0 or 1, conservation everywhere inside
        assert np.all((f >= 0) & (f <= g.cap))
        tails = np.repeat(np.arange(g.n), np.diff(g.off))
        net = np.zeros(g.n, np.int64)
        np.add.at(net, tails, -f.astype(np.int64))
        np.add.at(net, g.dst, f.astype(np.int64))
        assert np.all(net[inner] == 0) and net[g.t] == v
        d.complete_flow()
        assert np.array_equal(d.read_state()[2], f)
        # the general solver on the same handle starts from the capacities
        # again (BCSR16: one full rewrite after a matching; RCSR: always)
        r2 = d.solve("vc", g.s, g.t, matching=-1)
        assert r2.matching == 0 and r2.flow == v
        assert d.verify()["ok"]
        # and back, with thread-centric and every tile
        for algo, tile in (("tc", 0), ("vc", 8), ("vc", 32)):
            r3 = d.solve(algo, g.s, g.t, tile=tile)
            assert r3.matching == 1 and r3.flow == v
        assert d.verify()["ok"]


def test_matching_agrees_with_scipy_on_many_seeds():
    sg = pytest.importorskip("scipy.sparse.csgraph")
    import scipy.sparse as sp
    rng = np.random.default_rng(3)
    for i in range(12):
        L, R = int(rng.integers(1, 400)), int(rng.integers(1, 400))
        m = int(rng.integers(1, 3000))
        pr = random_pairs(rng, L, R, m)
        a = sp.csr_matrix((np.ones(m), (pr[:, 0], pr[:, 1])), shape=(L, R))
        want = int((sg.maximum_bipartite_matching(a, perm_type="column") >= 0).sum())
        size, pairs = W.bipartite_matching(L, R, pr[:, 0], pr[:, 1])
        assert size == want
        assert len(np.unique(pairs[:, 0])) == size and len(np.unique(pairs[:, 1])) == size


def not_matching_networks():
    base = network(30, 20, np.random.default_rng(2).integers(0, 20, (80, 2)) % [30, 20])
    tails = np.repeat(np.arange(base.n), np.diff(base.off))
    heads = base.dst.astype(np.int64)
    caps = base.cap.copy()
    s, t = base.s, base.t
    c2 = caps.copy()
    c2[np.flatnonzero((tails < 30) & (heads < 50))[0]] = 2  # an edge of capacity 2
    yield "capacity_2", W.Graph.from_arcs(base.n, tails, heads, c2, s, t)
    c0 = caps.copy()
    c0[np.flatnonzero(tails == s)[0]] = 0  # a source arc of capacity 0
    yield "capacity_0", W.Graph.from_arcs(base.n, tails, heads, c0, s, t)
    yield "left_to_left", W.Graph.from_arcs(base.n, np.append(tails, 0), np.append(heads, 1), np.append(caps, 1), s, t)
    yield "right_to_left", W.Graph.from_arcs(base.n, np.append(tails, 31), np.append(heads, 2), np.append(caps, 1), s, t)
    yield "source_to_sink", W.Graph.from_arcs(base.n, np.append(tails, s), np.append(heads, t), np.append(caps, 1), s, t)
    yield "parallel_source_arc", W.Graph.from_arcs(base.n, np.append(tails, s), np.append(heads, 0), np.append(caps, 1),
                                                   s, t)
    yield "into_source", W.Graph.from_arcs(base.n, np.append(tails, 0), np.append(heads, s), np.append(caps, 1), s, t)
    yield "out_of_sink", W.Graph.from_arcs(base.n, np.append(tails, t), np.append(heads, 35), np.append(caps, 1), s, t)
    yield "left_also_right", W.Graph.from_arcs(base.n, np.append(tails, 3), np.append(heads, t), np.append(caps, 1), s, t)


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
@pytest.mark.parametrize("name,g", list(not_matching_networks()), ids=lambda x: x if isinstance(x, str) else "")
def test_other_shapes_take_the_general_solver(name, g, layout):
    v = dinic(g)
    with W.DeviceGraph(g, layout) as d:
        r = d.solve("vc", g.s, g.t)
        assert r.matching == 0
        assert r.flow == v
        assert d.verify()["ok"]


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_detection_follows_terminals_and_capacities(layout):
    g = W.gen_bipartite(3000, 2000, 2.0, 256, 7)
    v = dinic(g)
    with W.DeviceGraph(g, layout) as d:
        assert d.solve("vc", g.s, g.t).matching == 1
        # other terminals on the same handle (s = 0, left vertices 1..3000):
        # the shape is checked per pair
        w = oracle.dinic(g.n, g.off, g.dst, g.cap, 1, g.t)
        r = d.solve("vc", 1, g.t)
        assert r.matching == 0 and r.flow == w
        assert d.solve("vc", g.s, g.t).matching == 1
        # new capacities drop the cached answer
        caps = g.cap.copy()
        caps[0] = 3
        d.set_capacities(caps)
        v3 = oracle.dinic(g.n, g.off, g.dst, caps, g.s, g.t)
        r = d.solve("vc", g.s, g.t)
        assert r.matching == 0 and r.flow == v3
        d.set_capacities(g.cap)
        r = d.solve("vc", g.s, g.t)
        assert r.matching == 1 and r.flow == v


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_round_budget_leaves_a_usable_handle(layout):
    g = W.gen_bipartite(20000, 20000, 2.0, 4096, 9)
    v = dinic(g)
    with W.DeviceGraph(g, layout) as d:
        with pytest.raises(W.WbprError) as ei:
            d.solve("vc", g.s, g.t, max_rounds=1)
        assert ei.value.status == 3  # WBPR_ERR_NO_CONVERGENCE
        # the stopped solve wrote the matching it had: a flow, below the maximum
        h, e, f = d.read_state()
        assert 0 < e[g.t] <= v
        r = d.solve("vc", g.s, g.t)
        assert r.matching == 1 and r.flow == v
        assert d.verify()["ok"]


def test_autotune_times_the_matching_kernel():
    g = W.gen_bipartite(20000, 20000, 2.0, 4096, 10)
    v = dinic(g)
    with W.DeviceGraph(g, "bcsr") as d:
        tu, ms = d.autotune("vc", g.s, g.t)
        assert ms > 0 and tu.matching == 0
        r = d.solve("vc", g.s, g.t, tile=tu.tile, gr_alpha=tu.gr_alpha)
        assert r.matching == 1 and r.flow == v


def test_repeated_solves_agree():
    """Many solves back to back on one handle, with both relabel triggers in
    play: every block must take the same branch at every round (a split
    would leave blocks meeting at barriers in different phases)."""
    g = W.gen_bipartite(200000, 200000, 2.0, 4096, 12)
    v = dinic(g)
    with W.DeviceGraph(g, "bcsr") as d:
        for i in range(40):
            r = d.solve("vc", g.s, g.t, gr_plateau=1 + i % 3)
            assert r.matching == 1 and r.flow == v
        assert d.verify()["ok"]
