"""The allocation-free solve (wbpr_solve_bcsr_noalloc) against the regular
one (wbpr_solve), through the C ABI.

Some callers cannot allocate device memory -- code that runs inside a
caller-owned memory pool, or a framework that forbids cudaMalloc while it
serves requests.  They hand the residual graph over in device buffers they
own and the solver keeps its scratch in one fixed device array.  The test
allocates those caller buffers itself (with torch), then checks that two
calls in a row give exactly the maximum flow the regular entry point gives
(the value is an integer: the tolerance is zero).  This file is collected
last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def _caller_buffers(torch, g):
    off, dst, cap, bidx = W.build_bcsr(g)
    arc = np.stack([dst, cap], axis=1).astype(np.int32).ravel()
    arx = np.stack([bidx, cap], axis=1).astype(np.int32).ravel()
    bufs = [torch.from_numpy(x.copy()).cuda() for x in (off, arc, arx)]
    torch.cuda.synchronize()
    return bufs, 2 * g.m


def test_noalloc_matches_regular_solve_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = W.lib()
    graphs = [W.gen_genrmf(8, 16, 1, 10000, 2), W.gen_rmat(14, 16, seed=3),
              W.gen_bipartite(2000, 2000, 2.0, 4096, 4)]
    for g in graphs:
        with W.DeviceGraph(g, "bcsr") as d:
            expected = {algo: d.solve(algo, g.s, g.t).flow for algo in ("tc", "vc")}
        (d_row, d_arc, d_arx), na = _caller_buffers(torch, g)
        for call in range(2):  # the second call reuses the shared array
            for algo, name in ((0, "tc"), (1, "vc")):
                flow = C.c_int64(-1)
                st = lib.wbpr_solve_bcsr_noalloc(g.n, na, d_row.data_ptr(), d_arc.data_ptr(), d_arx.data_ptr(),
                                                 g.s, g.t, algo, None, C.byref(flow))
                assert st == 0, (W.status_str(st), lib.wbpr_last_error().decode())
                assert flow.value == expected[name], (call, name)


def test_noalloc_rejects_oversized_graphs():
    lib = W.lib()
    flow = C.c_int64(-1)
    st = lib.wbpr_solve_bcsr_noalloc(70000, 10, None, None, None, 0, 1, 1, None, C.byref(flow))
    assert st == 1 and b"65536" in lib.wbpr_last_error()
    st = lib.wbpr_solve_bcsr_noalloc(100, 1 << 21, None, None, None, 0, 1, 1, None, C.byref(flow))
    assert st == 1 and b"1048576" in lib.wbpr_last_error()
