"""Parity of the CUDA path with the oracle, through the C ABI.

Bit-exact integer parity: every maximum-flow value equals the oracle's (and
the reference binary's, recorded in golden.json).  Larger instances are
checked against the FIFO push-relabel oracle, and at full size through the
device certificate (capacity pair invariant, conservation at every vertex,
no residual path from s or any excess vertex to t, cut == flow)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import wbpr_gb300 as W
from wbpr_gb300 import build as wb
from conftest import graph_of

pytestmark = pytest.mark.gpu

COMBOS = [("rcsr", "tc", 0), ("rcsr", "vc", 32), ("bcsr", "tc", 0), ("bcsr", "vc", 8), ("bcsr", "vc", 16),
          ("bcsr", "vc", 32)]


def solve_all(g, combos=COMBOS, **kw):
    out = {}
    for layout in sorted({c[0] for c in combos}):
        with W.DeviceGraph(g, layout) as d:
            for lay, algo, tile in combos:
                if lay != layout:
                    continue
                r = d.solve(algo, g.s, g.t, tile=tile, **kw)
                rep = d.verify()
                assert rep["ok"], (layout, algo, tile, rep)
                assert rep["label_violations"] == 0, (layout, algo, tile, rep)
                out[(layout, algo, tile)] = r.flow
    return out


@pytest.mark.parametrize("grid", [0, 4096])
def test_golden_cases(golden, grid):
    # grid 0: small graphs run on one block (block barriers); 4096: every
    # resident block of the device (grid barriers)
    for c in golden:
        g = graph_of(c)
        if g.n < 2 or g.s == g.t:
            continue
        for key, v in solve_all(g, grid_blocks=grid).items():
            assert v == c["expected"], (c["name"], key)
            if not c["reference_defect"]:
                assert v == c["reference"], (c["name"], key)


def test_parallel_source_arcs_are_not_lost():
    g = W.Graph.from_arcs(3, [0, 0, 1], [1, 1, 2], [5, 5, 10], 0, 2)
    assert set(solve_all(g).values()) == {10}


@pytest.mark.parametrize("grid", [0, 4096])
@pytest.mark.parametrize("seed", range(30))
def test_random_graphs(seed, grid):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(2, 300))
    m = int(rng.integers(0, 8 * n))
    tail = rng.integers(0, n, m)
    head = rng.integers(0, n, m)
    cap = rng.integers(0, int(rng.choice([2, 20, 1000, 2**20])), m)
    s, t = 0, n - 1
    g = W.Graph.from_arcs(n, tail, head, cap, s, t)
    expected = oracle.dinic(g.n, g.off, g.dst, g.cap, s, t)
    for key, v in solve_all(g, grid_blocks=grid).items():
        assert v == expected, key


def test_edge_cases():
    # no arcs at all
    g = W.Graph.from_arcs(2, [], [], [], 0, 1)
    assert set(solve_all(g).values()) == {0}
    # s -> t directly, self loops, zero capacities, unreachable component
    g = W.Graph.from_arcs(6, [0, 0, 1, 1, 2, 3, 4, 5], [5, 1, 1, 2, 5, 4, 5, 3], [7, 3, 9, 0, 4, 8, 8, 1], 0, 5)
    assert set(solve_all(g).values()) == {7 + 0}
    # max int32 capacities on one path
    g = W.Graph.from_arcs(3, [0, 1], [1, 2], [2**31 - 1, 2**31 - 1], 0, 2)
    assert set(solve_all(g).values()) == {2**31 - 1}
    # sink with out-arcs and source with in-arcs
    g = W.Graph.from_arcs(4, [0, 1, 2, 3, 3, 1], [1, 3, 0, 0, 2, 2], [10, 4, 6, 5, 5, 3], 0, 3)
    exp = oracle.dinic(g.n, g.off, g.dst, g.cap, 0, 3)
    assert set(solve_all(g).values()) == {exp}


def test_solver_reuse_and_terminal_override():
    g = W.gen_genrmf(5, 6, 1, 100, 3)
    with W.DeviceGraph(g, "bcsr") as d:
        a = d.solve("vc", g.s, g.t).flow
        b = d.solve("vc", g.s, g.t).flow
        assert a == b == oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        r = d.solve("vc", 5, g.n - 7)
        assert r.flow == oracle.dinic(g.n, g.off, g.dst, g.cap, 5, g.n - 7)
        with pytest.raises(W.WbprError):
            d.solve("vc", 3, 3)


def test_read_state_conservation():
    g = W.gen_rmat(11, 8, seed=4)
    with W.DeviceGraph(g, "bcsr") as d:
        r = d.solve("vc", g.s, g.t)
        h, e, f = d.read_state()
        tail, head, cap = g.arcs()
        assert ((f >= 0) & (f <= cap)).all()
        net = np.zeros(g.n, np.int64)
        np.add.at(net, head, f)
        np.add.at(net, tail, -f)
        mask = np.arange(g.n) != g.s
        assert np.array_equal(net[mask], e[mask].astype(np.int64))
        assert e[g.t] == r.flow


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_labels_after_repeated_global_relabels(layout):
    """A global relabel marks the vertices that cannot reach the sink and
    later relabels of the same solve skip them: with a relabel forced every
    round the flow stays exact, every label read back lies in [0, n], and
    every vertex that can reach the sink is labelled below n."""
    graphs = [W.gen_rmat(15, 8, seed=9), W.gen_bipartite(20000, 20000, 2.0, 256, 3),
              W.gen_genrmf(8, 16, 1, 10000, 5)]
    most = 0
    for g in graphs:
        v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, layout) as d:
            for gr_rounds in (1, 4):
                r = d.solve("vc", g.s, g.t, gr_rounds=gr_rounds)
                assert r.flow == v
                most = max(most, r.global_relabels)
                h, e, f = d.read_state()
                assert h.min() >= 0 and h.max() <= g.n
                reach = d.cut_sides(0).astype(bool)
                assert (h[reach] < g.n).all()
                assert d.verify()["ok"]
            d.complete_flow()
            h, e, f = d.read_state()
            assert h.min() >= 0 and h.max() <= g.n
            inner = np.ones(g.n, bool)
            inner[[g.s, g.t]] = False
            assert np.all(e[inner] == 0)
    assert most >= 3


@pytest.mark.parametrize("algo", [0, 1])
def test_reference_dropin(algo, golden):
    for c in golden[:20]:
        g = graph_of(c)
        roff, rdst, fidx = W.build_rcsr(g)
        state = W.rcsr_preflow(g, roff, rdst, fidx)
        flow, total, _ = W.rcsr_push_relabel(algo, g, state, roff, rdst, fidx)
        assert flow == c["expected"], c["name"]
        h, e, ff, bf, _ = state
        assert ((ff >= 0) & (bf >= 0) & (ff + bf == g.cap)).all()
        assert total == e[g.s] + e[g.t]


def test_cli_output_lines(tmp_path, golden):
    c = next(x for x in golden if x["name"] == "ref_genrmf_network")
    g = graph_of(c)
    p = str(tmp_path / "g.dimacs")
    W.write_dimacs(p, g)
    for algo in ("0", "1"):
        for lay in ("rcsr", "bcsr", "bcsr2"):
            r = subprocess.run([wb.CLI, "-v", "2", "-f", p, "-a", algo, "-l", lay, "-V"], capture_output=True,
                               text=True, timeout=120)
            assert r.returncode == 0, r.stdout + r.stderr
            assert "Total kernel time:" in r.stdout
            assert ("The maximum flow value of this flow network as calculated by the parallel implementation "
                    "is 228, 228") in r.stdout


@pytest.mark.parametrize("scale", [12, 14, 16])
def test_rmat_against_fifo_oracle(scale):
    g = W.gen_rmat(scale, 16, seed=scale)
    expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
    for key, v in solve_all(g, [("bcsr", "vc", 32), ("bcsr", "vc", 8), ("rcsr", "vc", 32),
                                ("bcsr", "tc", 0)]).items():
        assert v == expected, key


def test_genrmf_config0_seeds():
    for seed in range(8):
        g = W.gen_genrmf(8, 16, 1, 10000, seed)
        expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
        for key, v in solve_all(g, [("rcsr", "tc", 0), ("bcsr", "vc", 16)]).items():
            assert v == expected, (seed, key)


def test_bipartite_and_layered_and_grid():
    cases = [W.gen_bipartite(3000, 3000, 2.0, 4096, 1), W.gen_layered(20, 200, 3, 6, 1, 1000, 2),
             W.gen_grid(64, 64, 3)]
    for g in cases:
        expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
        for key, v in solve_all(g, [("bcsr", "vc", 8), ("bcsr", "vc", 32), ("rcsr", "tc", 0)]).items():
            assert v == expected, key


def test_budget_exhaustion_is_reported():
    g = W.gen_genrmf(8, 16, 1, 10000, 1)
    with W.DeviceGraph(g, "bcsr") as d:
        with pytest.raises(W.WbprError) as ei:
            d.solve("vc", g.s, g.t, max_rounds=2, gr_alpha=1e9)
        assert ei.value.status == 3
        # the handle stays usable
        assert d.solve("vc", g.s, g.t).flow == oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)


@pytest.mark.parametrize("tune", [
    dict(heavy_degree=64), dict(heavy_degree=256, gr_alpha=2.0), dict(heavy_degree=256, gr_alpha=8.0),
    dict(gr_alpha=0.05), dict(tile=8, heavy_degree=2048, gr_alpha=4.0), dict(blocks_per_sm=1, tile=16),
    dict(block=128, heavy_degree=128, gr_alpha=3.0), dict(grid_blocks=1), dict(grid_blocks=7, tile=8)])
def test_tuning_space_exact_and_valid(tune):
    """Every tuning gives the exact value, a valid final labelling and the
    certificate, within a bounded time (a livelock would hit max_ms)."""
    for g in (W.gen_rmat(16, 16, seed=5), W.gen_genrmf(12, 12, 1, 10000, 2)):
        expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
        for layout in ("bcsr", "rcsr"):
            with W.DeviceGraph(g, layout) as d:
                for algo in ("vc", "tc"):
                    r = d.solve(algo, g.s, g.t, max_ms=20000.0, **tune)
                    rep = d.verify()
                    assert r.flow == expected, (layout, algo, tune)
                    assert rep["ok"] and rep["label_violations"] == 0, (layout, algo, tune, rep)


def test_sparse_work_tail_terminates():
    """Rounds that do little work still lead to global relabels (a large
    work threshold alone once left ping-ponging vertices climbing to n)."""
    g = W.gen_rmat(20, 16, seed=1)
    expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
    with W.DeviceGraph(g, "bcsr") as d:
        for tune in (dict(heavy_degree=256, gr_alpha=2.0), dict(gr_alpha=50.0)):
            r = d.solve("vc", g.s, g.t, max_ms=30000.0, **tune)
            assert r.flow == expected, tune


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_rmat20_certificate(layout):
    """Size-independent property at a large size, where hub rows take the
    chunked deep passes in both layouts: the device certificate, and the
    completed flow conserving flow exactly."""
    g = W.gen_rmat(20, 16, seed=1)
    expected = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
    with W.DeviceGraph(g, layout) as d:
        for algo in ("vc", "tc"):
            r = d.solve(algo, g.s, g.t)
            rep = d.verify()
            assert rep["ok"] and rep["label_violations"] == 0 and rep["cut_value"] == r.flow == expected
        d.complete_flow()
        _, e, f = d.read_state()
        inner = np.ones(g.n, bool)
        inner[[g.s, g.t]] = False
        assert np.all(e[inner] == 0)
        tails = np.repeat(np.arange(g.n), np.diff(g.off))
        net = np.zeros(g.n, np.int64)
        np.add.at(net, tails, -f.astype(np.int64))
        np.add.at(net, g.dst, f.astype(np.int64))
        assert np.all(net[inner] == 0) and net[g.t] == expected


def test_long_path_is_not_relabel_bound():
    """One unit of excess walks a 20,000-vertex path one arc per round; the
    global relabel (20,000 BFS levels) must not run every few rounds."""
    n = 20000
    tail = np.arange(n - 1)
    cap = np.full(n - 1, 2)
    cap[0] = 1
    g = W.Graph.from_arcs(n, tail, tail + 1, cap, 0, n - 1)
    with W.DeviceGraph(g, "bcsr") as d:
        r = d.solve("vc", 0, n - 1)
        assert r.flow == 1
        assert r.solve_ms < 5000.0, r.solve_ms
        assert d.verify()["ok"]
