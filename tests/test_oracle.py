"""Oracle pinned to the reference: the restatement of maxflow-serial must
reproduce the reference binary's values (golden.json, produced by running
the reference compiled from its own sources), and two independent exact
solvers must agree with it."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W
from conftest import graph_of


def test_golden_has_reference_fixtures(golden):
    names = {c["name"] for c in golden}
    for n in ("ref_test_DIMACS", "ref_serial_test_graph", "ref_cuda_test_graph", "ref_genrmf_network"):
        assert n in names
    vals = {c["name"]: c["reference"] for c in golden}
    # values the reference prints on its own fixtures
    assert vals["ref_test_DIMACS"] == 25
    assert vals["ref_serial_test_graph"] == 3
    assert vals["ref_cuda_test_graph"] == 4
    assert vals["ref_genrmf_network"] == 228


def test_serial_restatement_matches_reference_binary(golden):
    for c in golden:
        g = graph_of(c)
        v, st = oracle.serial_maxflow(g.n, g.off, g.dst, g.cap, g.s, g.t)
        assert st in (0, 1), c["name"]
        assert v == c["reference"], c["name"]


def test_exact_solvers_agree_with_golden(golden):
    for c in golden:
        g = graph_of(c)
        assert oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) == c["expected"], c["name"]
        assert oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t) == c["expected"], c["name"]
        if not c["reference_defect"]:
            assert c["reference"] == c["expected"], c["name"]


def test_reference_preflow_defect_is_reproduced():
    # two parallel s->v arcs: the reference assigns excess[v] = cap instead of
    # adding (maxflow-serial/graph.cpp:474), losing one arc's flow
    g = W.Graph.from_arcs(3, [0, 0, 1], [1, 1, 2], [5, 5, 10], 0, 2)
    assert oracle.serial_maxflow(g.n, g.off, g.dst, g.cap, 0, 2)[0] == 5
    assert oracle.dinic(g.n, g.off, g.dst, g.cap, 0, 2) == 10
    assert oracle.fifo_pr(g.n, g.off, g.dst, g.cap, 0, 2) == 10


@pytest.mark.parametrize("seed", range(40))
def test_random_three_way(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 40))
    m = int(rng.integers(0, 5 * n))
    tail = rng.integers(0, n, m)
    head = rng.integers(0, n, m)
    cap = rng.integers(0, 50, m)
    g = W.Graph.from_arcs(n, tail, head, cap, 0, n - 1)
    d = oracle.dinic(g.n, g.off, g.dst, g.cap, 0, n - 1)
    f = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, 0, n - 1)
    assert d == f
    # serial agrees whenever s has no parallel arcs (its preflow assigns)
    heads_of_s = g.dst[g.off[0]:g.off[1]]
    if len(np.unique(heads_of_s)) == len(heads_of_s):
        assert oracle.serial_maxflow(g.n, g.off, g.dst, g.cap, 0, n - 1)[0] == d


def test_mincut_indicators_are_min_cuts():
    for seed in range(10):
        g = W.gen_genrmf(3, 4, 1, 50, seed)
        v, sink_side, src_side = oracle.mincut(g.n, g.off, g.dst, g.cap, g.s, g.t)
        assert int((sink_side * g.cap).sum()) == v
        assert int((src_side * g.cap).sum()) == v
