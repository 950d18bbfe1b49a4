"""On-device residual-graph build (wbpr_graph_create): the graph it leaves in
HBM must be the host builder's entry for entry -- BCSR offsets, heads,
capacities and twin indices (wbpr_build_bcsr, the layout of
maxflow-bcsr/src/graph.cpp:317-360), RCSR reverse offsets, reverse heads and
flow_index (wbpr_build_rcsr, maxflow-cuda/src/graph.cpp:317-402) -- for every
shape the sort and the length classes see: empty rows, isolated vertices,
parallel arcs, rows longer than the push chunk, heads that need one to four
radix passes, more arcs than one window of the sorted-position pass."""
import numpy as np
import pytest

import wbpr_gb300 as W
from conftest import graph_of

pytestmark = pytest.mark.gpu


def same_as_host(g):
    with W.DeviceGraph(g, "bcsr") as d:
        dev = d.read_bcsr()
    host = W.build_bcsr(g)
    for a, b, name in zip(dev, host, ("offsets", "destinations", "capacities", "backward_idx")):
        assert np.array_equal(a, b), name
    with W.DeviceGraph(g, "rcsr") as d:
        dev = d.read_rcsr()
    host = W.build_rcsr(g)
    for a, b, name in zip(dev, host, ("roffsets", "rdestinations", "flow_index")):
        assert np.array_equal(a, b), name


def random_graph(n, m, seed, max_cap=100, hot=None):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    if hot is not None:  # a vertex with many arcs in and out
        k = m // 3
        src[:k] = hot
        dst[k:2 * k] = hot
    cap = rng.integers(0, max_cap, m)
    return W.Graph.from_arcs(n, src, dst, cap, 0, n - 1)


def test_golden_cases(golden):
    for case in golden:
        same_as_host(graph_of(case))


@pytest.mark.parametrize("n,m", [(2, 1), (3, 0), (7, 40), (257, 3000), (300, 20000), (65537, 200000)])
def test_random_shapes(n, m):
    same_as_host(random_graph(n, m, n + m))


def test_long_rows_and_hot_vertex():
    # rows far longer than the 2048-arc push chunk, in and out of one vertex
    same_as_host(random_graph(5000, 120000, 3, hot=17))


def test_sorted_positions_in_several_windows():
    # more arcs than one window of arc ids (half the L2 in 4-byte entries,
    # about 16M on GB300): the sorted positions are written in two or more
    # passes, the in-capacity sums are skipped below the int32 bound
    same_as_host(W.gen_rmat(21, 16, seed=3))


def test_four_radix_passes():
    # heads need 25 bits: four 8-bit passes
    same_as_host(random_graph((1 << 24) + 5, 100000, 4))


def test_generators():
    same_as_host(W.gen_rmat(14, 16, seed=2))
    same_as_host(W.gen_genrmf(6, 8, 1, 100, 3))
    same_as_host(W.gen_bipartite(3000, 3000, 4.0, 8192, 5))
    same_as_host(W.gen_grid(40, 30, 1))


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_device_overflow_check(layout):
    g = W.Graph.from_arcs(3, [0, 0, 1, 1], [1, 2, 2, 2], [2**31 - 1, 2**31 - 1, 2**31 - 1, 5], 0, 2)
    with pytest.raises(W.WbprError) as ei:
        W.DeviceGraph(g, layout)
    assert ei.value.status == 4
    # at the limit exactly it builds
    g = W.Graph.from_arcs(3, [0, 1], [2, 2], [2**31 - 2, 1], 0, 2)
    same_as_host(g)
    # a head whose 100 incoming arcs span several warps of the sorted order,
    # between arcs into other vertices: exactly at the limit, then one above
    k = 100
    c = (2**31 - 1) // k
    tails = [0] * k + [2] * 40
    heads = [1] * k + [3] * 40
    caps = [c] * (k - 1) + [2**31 - 1 - c * (k - 1)] + [7] * 40
    order = np.random.default_rng(1).permutation(len(tails))
    g = W.Graph.from_arcs(4, np.array(tails)[order], np.array(heads)[order], np.array(caps)[order], 0, 3)
    same_as_host(g)
    caps[0] += 1
    g = W.Graph.from_arcs(4, np.array(tails)[order], np.array(heads)[order], np.array(caps)[order], 0, 3)
    with pytest.raises(W.WbprError) as ei:
        W.DeviceGraph(g, layout)
    assert ei.value.status == 4


def test_read_back_matches_the_layout():
    g = random_graph(50, 200, 1)
    with W.DeviceGraph(g, "rcsr") as d:
        with pytest.raises(W.WbprError) as ei:
            d.read_bcsr()
        assert ei.value.status == 1
    with W.DeviceGraph(g, "bcsr") as d:
        with pytest.raises(W.WbprError) as ei:
            d.read_rcsr()
        assert ei.value.status == 1


@pytest.mark.parametrize("layout", ["bcsr", "rcsr"])
def test_device_build_rejects_invalid_input(layout):
    # the O(n + m) input checks run on the device while it builds
    def make(off, dst, cap):
        return W.Graph(4, np.array(off, np.int32), np.array(dst, np.int32), np.array(cap, np.int32), 0, 3)
    bad = [make([0, 2, 3, 4, 4], [1, 4, 2, 3], [1, 1, 1, 1]),     # head out of range
           make([0, 2, 3, 4, 4], [1, 2, 2, 3], [1, -1, 1, 1]),    # negative capacity
           make([0, 3, 1, 4, 4], [1, 2, 2, 3], [1, 1, 1, 1]),     # offsets decrease
           make([0, 2, 3, 4, 4], [1, -1, 2, 3], [1, 1, 1, 1])]    # negative head
    for g in bad:
        with pytest.raises(W.WbprError) as ei:
            W.DeviceGraph(g, layout)
        assert ei.value.status == 1
    ok = make([0, 2, 3, 4, 4], [1, 2, 2, 3], [1, 1, 1, 1])
    with W.DeviceGraph(ok, layout) as d:
        assert d.solve("vc", 0, 3).flow == 1
