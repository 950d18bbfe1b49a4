"""The allocation-free solve (wbpr_solve_bcsr_noalloc) through the C ABI.

Some callers cannot allocate device memory -- code that runs inside a
caller-owned memory pool, or a framework that forbids cudaMalloc while it
serves requests.  They hand the residual graph over in device buffers they
own and the solver keeps its scratch in one fixed device array.  The tests
allocate those caller buffers themselves (with torch), then check that two
calls in a row give exactly the maximum flow of the regular entry point and
of the oracle (the value is an integer: the tolerance is zero), that a call
leaves the device's free memory unchanged, and that malformed buffers are
refused before any solver kernel reads them.  This file is collected last on
purpose.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _host_buffers(g):
    off, dst, cap, bidx = W.build_bcsr(g)
    arc = np.stack([dst, cap], axis=1).astype(np.int32).ravel()
    arx = np.stack([bidx, cap], axis=1).astype(np.int32).ravel()
    return off.astype(np.int32), arc, arx


def _device(torch, *arrays):
    bufs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in arrays]
    torch.cuda.synchronize()
    return bufs


def _call(lib, n, na, d_row, d_arc, d_arx, s, t, algo):
    flow = C.c_int64(-1)
    st = lib.wbpr_solve_bcsr_noalloc(n, na, d_row.data_ptr(), d_arc.data_ptr(), d_arx.data_ptr(), s, t, algo,
                                     None, C.byref(flow))
    return st, flow.value


def test_noalloc_matches_regular_solve_twice():
    torch = _torch()
    lib = W.lib()
    graphs = [W.gen_genrmf(8, 16, 1, 10000, 2), W.gen_rmat(14, 16, seed=3),
              W.gen_bipartite(2000, 2000, 2.0, 4096, 4)]
    for g in graphs:
        exact = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        with W.DeviceGraph(g, "bcsr") as d:
            expected = {algo: d.solve(algo, g.s, g.t).flow for algo in ("tc", "vc")}
        assert expected == {"tc": exact, "vc": exact}
        d_row, d_arc, d_arx = _device(torch, *_host_buffers(g))
        for call in range(2):  # the second call reuses the shared array
            for algo in (0, 1):
                st, flow = _call(lib, g.n, 2 * g.m, d_row, d_arc, d_arx, g.s, g.t, algo)
                assert st == 0, (W.status_str(st), lib.wbpr_last_error().decode())
                assert flow == exact, (call, algo)


def test_noalloc_leaves_device_memory_unchanged():
    torch = _torch()
    lib = W.lib()
    g = W.gen_rmat(13, 16, seed=5)
    d_row, d_arc, d_arx = _device(torch, *_host_buffers(g))
    # the first call on the device may load the module that holds the array
    st, first = _call(lib, g.n, 2 * g.m, d_row, d_arc, d_arx, g.s, g.t, 1)
    assert st == 0, lib.wbpr_last_error().decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        st, flow = _call(lib, g.n, 2 * g.m, d_row, d_arc, d_arx, g.s, g.t, 1)
        assert st == 0 and flow == first
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_malformed_buffers():
    torch = _torch()
    lib = W.lib()
    g = W.gen_genrmf(6, 8, 1, 10000, 3)
    row, arc, arx = _host_buffers(g)
    na = 2 * g.m
    # rows that claim more arcs than declared: refused before anything sizes work by them
    bad = row.copy()
    bad[-1] = na + 4096
    d = _device(torch, bad, arc, arx)
    st, _ = _call(lib, g.n, na, *d, g.s, g.t, 1)
    assert st == 1 and b"d_row" in lib.wbpr_last_error()
    bad = row.copy()
    bad[5] = bad[6] + 1  # a negative row length
    d = _device(torch, bad, arc, arx)
    st, _ = _call(lib, g.n, na, *d, g.s, g.t, 1)
    assert st == 1 and b"d_row" in lib.wbpr_last_error()
    # a head outside [0, n)
    bad = arc.copy()
    bad[2 * 7] = g.n + 100
    d = _device(torch, row, bad, arx)
    st, _ = _call(lib, g.n, na, *d, g.s, g.t, 1)
    assert st == 1 and b"head" in lib.wbpr_last_error()
    # an unpaired twin
    bad = arx.copy()
    bad[2 * 3] = (bad[2 * 3] + 1) % na
    d = _device(torch, row, arc, bad)
    st, _ = _call(lib, g.n, na, *d, g.s, g.t, 1)
    assert st == 1 and b"twin" in lib.wbpr_last_error()
    # incoming capacities past int32: two arcs into t of 2^30 + 2^30
    h = W.Graph.from_arcs(4, np.array([0, 0, 1, 2]), np.array([1, 2, 3, 3]),
                          np.array([2 ** 30, 2 ** 30, 2 ** 30, 2 ** 30]), 0, 3)
    d = _device(torch, *_host_buffers(h))
    st, _ = _call(lib, h.n, 2 * h.m, *d, h.s, h.t, 1)
    assert st == 4 and b"int32" in lib.wbpr_last_error()
    # the good buffers still solve exactly afterwards
    d = _device(torch, row, arc, arx)
    st, flow = _call(lib, g.n, na, *d, g.s, g.t, 1)
    assert st == 0 and flow == oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)


def test_noalloc_rejects_oversized_graphs():
    lib = W.lib()
    flow = C.c_int64(-1)
    st = lib.wbpr_solve_bcsr_noalloc(70000, 10, None, None, None, 0, 1, 1, None, C.byref(flow))
    assert st == 1 and b"65536" in lib.wbpr_last_error()
    st = lib.wbpr_solve_bcsr_noalloc(100, 1 << 21, None, None, None, 0, 1, 1, None, C.byref(flow))
    assert st == 1 and b"1048576" in lib.wbpr_last_error()
