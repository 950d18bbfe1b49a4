"""Generate tests/golden/fullsize.json: the exact maximum-flow values of the
five benchmark workloads at their full sizes, from the CPU oracle.

Every value comes from the oracle's Dinic solver; the single large instances
(configs 1 and 2) are also solved by its FIFO push-relabel, and the two must
agree.  Each record keeps the generator's CSR hash, so a generator that ever
produced other bits on another host would show up as a hash mismatch before
any flow is compared.  The GPU tests and bench.py check the CUDA path against
these values; nothing here needs a GPU or the reference tree.

Run: python tests/golden/make_fullsize.py [--jobs N]   (about 10-20 minutes
on 8 cores, most of it the 256 grids of config 4)
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "fullsize.json")
CONFIG0_SEEDS = 20
CONFIG3_COUNT = 4096
CONFIG4_GRIDS = 256


def _solve(job):
    import oracle
    from wbpr_gb300 import workloads as WL

    kind, arg = job
    if kind == "c0":
        g = WL.config0(arg)
    elif kind == "c3":
        g = WL.config3_instance(arg)
    elif kind == "c4":
        g = WL.config4(arg)
    elif kind == "c1":
        g = WL.config1()
    else:
        g = WL.config2()
    t0 = time.perf_counter()
    v = oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t)
    rec = {"n": int(g.n), "m": int(g.m), "s": int(g.s), "t": int(g.t), "csr_hash": WL.csr_hash(g), "flow": v,
           "dinic_s": round(time.perf_counter() - t0, 3)}
    if kind in ("c1", "c2"):
        t0 = time.perf_counter()
        rec["fifo_pr"] = oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t)
        rec["fifo_pr_s"] = round(time.perf_counter() - t0, 3)
        if rec["fifo_pr"] != v:
            raise AssertionError(f"{kind}: Dinic {v} != FIFO push-relabel {rec['fifo_pr']}")
    return job, rec


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    from wbpr_gb300 import workloads as WL

    c3 = WL.config3_params(CONFIG3_COUNT)
    jobs = [("c1", None), ("c2", None)] + [("c4", s) for s in range(CONFIG4_GRIDS)]
    jobs += [("c0", s) for s in range(CONFIG0_SEEDS)] + [("c3", p) for p in c3]
    res = {}
    t0 = time.time()
    with mp.get_context("spawn").Pool(args.jobs) as pool:
        for i, (job, rec) in enumerate(pool.imap_unordered(_solve, jobs, chunksize=1)):
            res[(job[0], job[1] if job[0] != "c3" else tuple(job[1]))] = rec
            if job[0] in ("c1", "c2") or i % 500 == 0:
                print(f"[{time.time() - t0:7.1f}s] {i + 1}/{len(jobs)} {job[0]} {rec['flow']}", flush=True)
    c0 = [res[("c0", s)] for s in range(CONFIG0_SEEDS)]
    c3r = [res[("c3", tuple(p))] for p in c3]
    c4 = [res[("c4", s)] for s in range(CONFIG4_GRIDS)]
    out = {
        "generated_by": "tests/golden/make_fullsize.py (oracle Dinic; FIFO push-relabel cross-check on configs 1-2)",
        "config0": {"workload": "GENRMF a=8 b=16 caps [1, 10000]", "seeds": CONFIG0_SEEDS,
                    "flows": [r["flow"] for r in c0], "csr_hashes": [r["csr_hash"] for r in c0]},
        "config1": dict(res[("c1", None)], workload="R-MAT scale 22 ef 16 (0.57, 0.19, 0.19) caps [1, 100] seed 1"),
        "config2": dict(res[("c2", None)], workload="bipartite 2M x 2M Zipf(2.0) [1, 4096] seed 1"),
        "config3": {"workload": f"{CONFIG3_COUNT} instances, numpy seed 7 (wbpr_gb300.workloads.config3_params)",
                    "count": CONFIG3_COUNT, "flows": [r["flow"] for r in c3r],
                    "flows_hash": WL.flows_hash([r["flow"] for r in c3r]),
                    "csr_hashes_hash": WL.flows_hash([int(r["csr_hash"], 16) >> 1 for r in c3r]),
                    "m_total": int(sum(r["m"] for r in c3r)), "n_total": int(sum(r["n"] for r in c3r))},
        "config4": {"workload": "512 x 512 graph-cut grids, seeds 0..255", "grids": CONFIG4_GRIDS,
                    "flows": [r["flow"] for r in c4], "csr_hashes": [r["csr_hash"] for r in c4]},
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT, f"in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
