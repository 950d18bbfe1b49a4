"""Generate tests/golden/golden.json (run in a container that has the
reference tree; the committed JSON is what tests read everywhere else).

For every case the expected maximum flow comes from running the reference's
own serial solver, compiled from its sources by oracle/build_oracle.py
(oracle/_ref/maxflow-serial), on a DIMACS or SNAP file.  Cases:
  * the reference's fixtures (maxflow-serial/input/test_DIMACS.txt,
    maxflow-serial/test_graph.txt, maxflow-cuda/test/test_graph.txt,
    maxflow-cuda/snap_test.txt, network/DIMACS/genrmf/network.dimacs and
    network/DIMACS/genrmf/test_graph.txt), re-encoded as arc lists;
  * seeded graphs from this project's generators and from a numpy RNG
    (parallel and antiparallel arcs, unreachable parts, zero capacities).
Where the reference's value differs from the true maximum flow (its preflow
assigns instead of adding excess, and its reverse pairing takes the first
parallel arc), the case records both and is flagged `reference_defect`.
Each generator case also records a hash of the generated CSR, pinning the
generators to the same bits on every host.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import wbpr_gb300 as W  # noqa: E402
from oracle.build_oracle import REF_TREE, build_ref  # noqa: E402

REF = REF_TREE  # WBPR_REFERENCE, else the default tree of the recipe
FIXTURES = [
    ("ref_test_DIMACS", "maxflow-serial/input/test_DIMACS.txt", 2, None, None),
    ("ref_serial_test_graph", "maxflow-serial/test_graph.txt", 0, 0, 4),
    ("ref_cuda_test_graph", "maxflow-cuda/test/test_graph.txt", 0, 0, 7),
    ("ref_snap_test", "maxflow-cuda/snap_test.txt", 0, 0, 3),
    ("ref_genrmf_network", "network/DIMACS/genrmf/network.dimacs", 2, None, None),
    ("ref_genrmf_test_graph", "network/DIMACS/genrmf/test_graph.txt", 2, None, None),
]


def csr_hash(g: W.Graph) -> str:
    h = hashlib.sha256()
    for a in (np.asarray(g.off, np.int32), np.asarray(g.dst, np.int32), np.asarray(g.cap, np.int32)):
        h.update(a.tobytes())
    h.update(np.asarray([g.n, g.s, g.t], np.int64).tobytes())
    return h.hexdigest()[:16]


def encode(g: W.Graph) -> dict:
    tail, head, cap = g.arcs()
    return {"n": int(g.n), "s": int(g.s), "t": int(g.t),
            "arcs": [[int(a), int(b), int(c)] for a, b, c in zip(tail, head, cap)]}


def ref_value(g: W.Graph) -> int:
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "g.dimacs")
        W.write_dimacs(p, g)
        v = oracle.run_ref_serial(p, 2)
    return 0 if v is None else v


def random_graph(rng, n, m, cmax, parallel: bool, s_parallel: bool) -> W.Graph:
    tail = rng.integers(0, n, m)
    head = rng.integers(0, n, m)
    keep = tail != head
    tail, head = tail[keep], head[keep]
    if not parallel:
        key = np.unique(tail.astype(np.int64) * n + head)
        tail, head = key // n, key % n
    if not s_parallel:
        # at most one arc s -> v for each v (the reference preflow assigns)
        key = tail.astype(np.int64) * n + head
        first = np.zeros(len(key), bool)
        _, idx = np.unique(key, return_index=True)
        first[idx] = True
        keep = (tail != 0) | first
        tail, head = tail[keep], head[keep]
    cap = rng.integers(0, cmax + 1, len(tail))
    return W.Graph.from_arcs(n, tail, head, cap, 0, n - 1)


def main() -> None:
    if build_ref() is None:
        raise SystemExit("reference sources not found; golden.json cannot be regenerated here")
    cases = []
    for name, rel, ft, s, t in FIXTURES:
        path = os.path.join(REF, rel)
        g = W.read_graph(path, ft)
        if ft != 2:
            g.s, g.t = s, t
        v = oracle.run_ref_serial(path, ft, s, t)
        d = encode(g)
        d.update(name=name, source_file=rel, reference=v, expected=oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t))
        cases.append(d)
    gens = []
    for seed in range(4):
        gens.append((f"genrmf_a4_b6_s{seed}", W.gen_genrmf(4, 6, 1, 10000, seed), "genrmf(4,6,1,10000)"))
    gens.append(("genrmf_a8_b16_s1", W.gen_genrmf(8, 16, 1, 10000, 1), "genrmf(8,16,1,10000)"))
    gens.append(("layered_6x12_s3", W.gen_layered(6, 12, 3, 6, 1, 1000, 3), "layered(6,12,3,6,1,1000)"))
    gens.append(("bipartite_40x30_s5", W.gen_bipartite(40, 30, 2.0, 4096, 5), "bipartite(40,30,2.0,4096)"))
    gens.append(("grid_8x8_s2", W.gen_grid(8, 8, 2), "grid(8,8)"))
    gens.append(("rmat_s7_s1", W.gen_rmat(7, 8, 0.57, 0.19, 0.19, 1, 100, 1), "rmat(7,8,.57,.19,.19,1,100)"))
    for name, g, spec in gens:
        d = encode(g)
        d.update(name=name, generator=spec, csr_hash=csr_hash(g), reference=ref_value(g),
                 expected=oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t))
        cases.append(d)
    rng = np.random.default_rng(20261203)
    for k in range(24):
        n = int(rng.integers(6, 60))
        m = int(rng.integers(n, 6 * n))
        parallel = bool(k % 3 == 0)
        s_par = bool(k % 6 == 0)
        g = random_graph(rng, n, m, int(rng.choice([1, 7, 100, 100000])), parallel, s_par)
        d = encode(g)
        d.update(name=f"random_{k}", reference=ref_value(g),
                 expected=oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t))
        cases.append(d)
    for d in cases:
        d["reference_defect"] = bool(d["reference"] != d["expected"])
    out = os.path.join(HERE, "golden.json")
    with open(out, "w") as f:
        json.dump({"generated_by": "tests/golden/make_golden.py",
                   "reference_binary": "oracle/_ref/maxflow-serial (built from maxflow-serial/*.cpp, mmio.c)",
                   "cases": cases}, f, separators=(",", ":"))
    bad = [d["name"] for d in cases if d["reference_defect"]]
    print(f"wrote {out}: {len(cases)} cases; reference differs from max flow on {bad}")


if __name__ == "__main__":
    main()
