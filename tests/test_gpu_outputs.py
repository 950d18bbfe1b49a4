"""What comes after the solve: the maximum flow itself (wbpr_complete_flow
then per-arc flows), the vertex sides of the two extreme minimum cuts
(wbpr_cut_sides), the DIMACS solution written by the CLI (-o), the graph
cache (-c / -v 3) and the bipartite-matching front end.  Checked against the
oracle's exact values and by exact conservation on the host."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import wbpr_gb300 as W
from wbpr_gb300 import build as wb

pytestmark = pytest.mark.gpu


def graphs():
    yield W.gen_genrmf(5, 6, 1, 100, 1)
    yield W.gen_rmat(12, 8, seed=3)
    yield W.gen_grid(32, 32, 2)
    yield W.gen_bipartite(500, 400, 2.0, 64, 3)
    rng = np.random.default_rng(5)
    n, m = 80, 600  # parallel and antiparallel arcs, zero capacities
    yield W.Graph.from_arcs(n, rng.integers(0, n, m), rng.integers(0, n, m), rng.integers(0, 6, m), 0, n - 1)


def check_flow(g, f, value):
    assert np.all(f >= 0) and np.all(f <= g.cap)
    tails = np.repeat(np.arange(g.n), np.diff(g.off))
    net = np.zeros(g.n, np.int64)
    np.add.at(net, tails, -f.astype(np.int64))
    np.add.at(net, g.dst, f.astype(np.int64))
    inner = np.ones(g.n, bool)
    inner[[g.s, g.t]] = False
    assert np.all(net[inner] == 0)
    assert net[g.t] == value and net[g.s] == -value


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_completed_flow_is_a_maximum_flow(layout):
    for g in graphs():
        v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, layout) as d:
            r = d.solve("vc", g.s, g.t)
            assert r.flow == v
            d.complete_flow()
            h, e, f = d.read_state()
            check_flow(g, f, v)
            inner = np.ones(g.n, bool)
            inner[[g.s, g.t]] = False
            assert np.all(e[inner] == 0)
            rep = d.verify()
            assert rep["ok"] and rep["flow_value"] == v
            # a second call finds nothing left to return
            d.complete_flow()
            assert np.array_equal(d.read_state()[2], f)


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_cut_sides_give_the_extreme_cuts(layout):
    for g in graphs():
        v, sink_side, src_side = oracle.mincut(g.n, g.off, g.dst, g.cap, g.s, g.t)
        tails = np.repeat(np.arange(g.n), np.diff(g.off))
        with W.DeviceGraph(g, layout) as d:
            d.solve("vc", g.s, g.t)
            T = d.cut_sides(0).astype(bool)
            S = d.cut_sides(1).astype(bool)
        assert T[g.t] and not T[g.s] and S[g.s] and not S[g.t]
        assert np.array_equal((~T[tails] & T[g.dst]).astype(np.int8), sink_side)
        assert np.array_equal((S[tails] & ~S[g.dst]).astype(np.int8), src_side)
        assert int(g.cap[~T[tails] & T[g.dst]].astype(np.int64).sum()) == v
        assert not np.any(S & T)


def test_bipartite_matching():
    scipy_graph = pytest.importorskip("scipy.sparse.csgraph")
    import scipy.sparse as sp

    rng = np.random.default_rng(8)
    for L, R, k in ((1, 1, 1), (50, 40, 200), (3000, 2000, 12000)):
        left = rng.integers(0, L, k)
        right = rng.integers(0, R, k)
        size, pairs = W.bipartite_matching(L, R, left, right)
        a = sp.csr_matrix((np.ones(k), (left, right)), shape=(L, R))
        match = scipy_graph.maximum_bipartite_matching(a, perm_type="column")
        assert size == int((match >= 0).sum())
        assert len(np.unique(pairs[:, 0])) == size and len(np.unique(pairs[:, 1])) == size
        edges = set(zip(left.tolist(), right.tolist()))
        assert all((int(x), int(y)) in edges for x, y in pairs)
        g = W.bipartite_network(L, R, left, right)
        assert size == oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)


def test_cli_solution_and_cache(tmp_path):
    g = W.gen_genrmf(4, 5, 1, 300, 4)
    src = tmp_path / "g.dimacs"
    W.write_dimacs(str(src), g)
    sol, cache = tmp_path / "sol.txt", tmp_path / "g.wgc"
    r = subprocess.run([wb.CLI, "-v", "2", "-f", str(src), "-a", "1", "-l", "bcsr", "-o", str(sol), "-c", str(cache)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
    assert f"is {v}, {v}" in r.stdout
    lines = sol.read_text().splitlines()
    assert f"s {v}" in lines
    f = np.zeros(g.m, np.int64)
    pos = {}
    tails = np.repeat(np.arange(g.n), np.diff(g.off))
    for i in range(g.m):
        pos.setdefault((int(tails[i]) + 1, int(g.dst[i]) + 1), []).append(i)
    for line in lines:
        if line.startswith("f "):
            _, a, b, x = line.split()
            f[pos[(int(a), int(b))].pop(0)] = int(x)
    check_flow(g, f, v)
    r2 = subprocess.run([wb.CLI, "-v", "3", "-f", str(cache), "-a", "0"], capture_output=True, text=True)
    assert r2.returncode == 0 and f"is {v}, {v}" in r2.stdout


def test_caller_stream_and_device_indicator():
    torch = pytest.importorskip("torch")
    g = W.gen_grid(48, 48, 6)
    v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
    with W.DeviceGraph(g, "bcsr") as d:
        host0 = None
        r = d.solve("vc", g.s, g.t)
        host0, _ = d.mincut_adjoint(0)
        s = torch.cuda.Stream()
        d.set_stream(s.cuda_stream)
        r2 = d.solve("vc", g.s, g.t)
        assert r.flow == r2.flow == v
        assert d.verify()["ok"]
        dev = torch.zeros(g.m, dtype=torch.int8, device="cuda")
        ms = W.api.C.c_float(0)
        st = W.lib().wbpr_mincut_adjoint(d._h, 0, W.api.C.cast(dev.data_ptr(), W.api._i8p), W.api.C.byref(ms))
        assert st == 0
        torch.cuda.synchronize()
        assert np.array_equal(dev.cpu().numpy(), host0)
        d.set_stream(None)
        assert d.solve("tc", g.s, g.t).flow == v


def test_single_graph_autotune():
    for g in (W.gen_rmat(14, 16, seed=2), W.gen_genrmf(10, 10, 1, 1000, 3)):
        v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, "bcsr") as d:
            best, ms = d.autotune("vc", g.s, g.t)
            assert best.tile in (8, 16, 32) and best.gr_alpha in (0.5, 1.0, 1.5, 3.0)
            assert best.heavy_degree in (32, 64) and ms > 0
            r = d.solve("vc", g.s, g.t, tile=best.tile, gr_alpha=best.gr_alpha, heavy_degree=best.heavy_degree)
            assert r.flow == v
            tc, _ = d.autotune("tc", g.s, g.t)
            assert tc.tile == 0


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_new_capacities_without_rebuild(layout):
    g = W.gen_grid(40, 30, 2)
    rng = np.random.default_rng(3)
    with W.DeviceGraph(g, layout) as d:
        assert d.solve("vc", g.s, g.t).flow == oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        for trial in range(3):
            cap = rng.integers(0, 2000, g.m).astype(np.int32)
            d.set_capacities(cap)
            v = oracle.dinic(g.n, g.off, g.dst, cap, g.s, g.t)
            r = d.solve("vc", g.s, g.t)
            assert r.flow == v and d.verify()["ok"]
        # rejected updates leave the graph as it was
        bad = cap.copy()
        bad[5] = -1
        with pytest.raises(W.WbprError) as ei:
            d.set_capacities(bad)
        assert ei.value.status == 1
        big = np.full(g.m, 2**30, np.int32)
        with pytest.raises(W.WbprError) as ei:
            d.set_capacities(big)
        assert ei.value.status == 4
        assert d.solve("tc", g.s, g.t).flow == v


def test_memory_pool_keeps_and_releases():
    """Graphs take device memory from the library's pool: what a destroyed
    graph held stays reserved for the next one (same results), and
    memory_cache(0) hands it back to the driver."""
    torch = pytest.importorskip("torch")
    g = W.gen_rmat(17, 16, seed=2)
    v = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
    W.memory_cache(16 << 30)
    held = 0
    for layout in ("bcsr", "rcsr", "bcsr"):
        with W.DeviceGraph(g, layout) as d:
            assert d.solve("vc", g.s, g.t).flow == v
            assert d.verify()["ok"]
            held = max(held, d.device_bytes)
    free_kept = torch.cuda.mem_get_info()[0]
    W.memory_cache(0)
    free_released = torch.cuda.mem_get_info()[0]
    assert free_released - free_kept >= held // 2
    W.memory_cache(16 << 30)
    with W.DeviceGraph(g, "bcsr") as d:
        assert d.solve("vc", g.s, g.t).flow == v
    with pytest.raises(W.WbprError):
        W.memory_cache(-1)
