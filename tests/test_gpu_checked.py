"""The solver kernels built with bounds-checked accessors (libwbpr_checked.so,
-DWBPR_CHECKED): every arc index is checked against the residual arc count
and every vertex against n.  An out-of-range index is counted and the solve
fails with WBPR_ERR_VERIFY.  This stands in for a memory checker, which this
GPU pool does not offer.  Both layouts, TC and VC, one-block and full grids,
on the golden cases and on seeded graphs of every generator must solve
exactly with no index out of range."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import wbpr_gb300 as W
from conftest import ROOT, graph_of

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import json, sys
sys.path.insert(0, %r)
import numpy as np
import wbpr_gb300 as W
cases = json.loads(sys.stdin.read())
out = []
for c in cases:
    g = W.Graph(c["n"], np.array(c["off"], np.int32), np.array(c["dst"], np.int32), np.array(c["cap"], np.int32),
                c["s"], c["t"])
    row = []
    for layout in ("bcsr", "rcsr"):
        with W.DeviceGraph(g, layout) as d:
            for algo in ("tc", "vc"):
                for grid in (0, 4096):
                    r = d.solve(algo, g.s, g.t, grid_blocks=grid)
                    rep = d.verify()
                    row.append([int(r.flow), int(rep["ok"])])
    out.append(row)
print(json.dumps(out))
"""


def test_checked_kernels_stay_in_bounds(golden):
    graphs = [graph_of(c) for c in golden if c["n"] >= 2 and c["s"] != c["t"]][:12]
    graphs += [W.gen_rmat(12, 8, seed=5), W.gen_genrmf(6, 6, 1, 500, 2), W.gen_grid(24, 24, 1),
               W.gen_bipartite(800, 600, 2.0, 64, 4), W.gen_layered(10, 50, 3, 6, 1, 100, 2)]
    rng = np.random.default_rng(9)
    for _ in range(4):
        n, m = 60, 400
        graphs.append(W.Graph.from_arcs(n, rng.integers(0, n, m), rng.integers(0, n, m), rng.integers(0, 9, m),
                                        0, n - 1))
    cases = [dict(n=g.n, off=g.off.tolist(), dst=g.dst.tolist(), cap=g.cap.tolist(), s=g.s, t=g.t) for g in graphs]
    env = dict(os.environ, WBPR_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT], input=json.dumps(cases), capture_output=True,
                       text=True, env=env, timeout=1200)
    assert r.returncode == 0, r.stderr[-3000:]
    rows = json.loads(r.stdout.strip().splitlines()[-1])
    for g, row in zip(graphs, rows):
        v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
        assert all(f == v and ok == 1 for f, ok in row), (g.n, v, row)
