"""The benchmark workloads, seeded, built from the library's generators.

The WBPR paper measures on SNAP, KONECT and DIMACS instances that are not
available here; these seeded synthetic inputs have their shapes:

  config 0  GENRMF a=8, b=16 (1,024 vertices, 4,544 arcs), capacities
            [1, 10000], one instance per seed; TC over RCSR
  config 1  R-MAT scale 22, edge factor 16, (0.57, 0.19, 0.19, 0.05), self
            loops and duplicates removed, capacities [1, 100], seed 1; s = max
            out-degree vertex, t = max in-degree vertex
  config 2  unit-capacity bipartite matching, 2M left x 2M right, left
            degrees Zipf(2.0) clipped to [1, 4096], seed 1
  config 3  4,096 uneven instances: even indices GENRMF with a and b
            log-uniform in [4, 32] x [4, 64], odd indices layered networks of
            8-64 layers x 16-512 vertices, 3-6 arcs per vertex, capacities
            [1, 1000]
  config 4  512 x 512 graph-cut grids (4-connected n-links, t-links from a
            smooth seeded field), one per seed
"""
from __future__ import annotations

import hashlib

import numpy as np

from . import api as W

RMAT = dict(scale=22, edge_factor=16, a=0.57, b=0.19, c=0.19, cap_lo=1, cap_hi=100, seed=1)


def config0(seed: int = 0) -> W.Graph:
    return W.gen_genrmf(8, 16, 1, 10000, seed)


def config1(scale: int = RMAT["scale"]) -> W.Graph:
    w = RMAT
    return W.gen_rmat(scale, w["edge_factor"], w["a"], w["b"], w["c"], w["cap_lo"], w["cap_hi"], w["seed"])


def config2() -> W.Graph:
    return W.gen_bipartite(2000000, 2000000, 2.0, 4096, 1)


def config3_params(count: int = 4096, seed: int = 7) -> list[tuple]:
    """(kind, args) per instance: ("genrmf", a, b, seed) or ("layered",
    layers, width, seed), drawn from one seeded numpy stream."""
    rng = np.random.default_rng(seed)
    aw = np.arange(4, 33)
    aw_p = (1.0 / aw) / (1.0 / aw).sum()  # log-uniform over the integers
    bw = np.arange(4, 65)
    bw_p = (1.0 / bw) / (1.0 / bw).sum()
    out = []
    for i in range(count):
        if i % 2 == 0:
            out.append(("genrmf", int(rng.choice(aw, p=aw_p)), int(rng.choice(bw, p=bw_p)), i))
        else:
            out.append(("layered", int(rng.integers(8, 65)), int(rng.integers(16, 513)), i))
    return out


def config3_instance(p: tuple) -> W.Graph:
    if p[0] == "genrmf":
        return W.gen_genrmf(p[1], p[2], 1, 10000, p[3])
    return W.gen_layered(p[1], p[2], 3, 6, 1, 1000, p[3])


def config3(count: int = 4096, seed: int = 7) -> list[W.Graph]:
    return [config3_instance(p) for p in config3_params(count, seed)]


def config4(seed: int = 0) -> W.Graph:
    return W.gen_grid(512, 512, seed)


def csr_hash(g: W.Graph) -> str:
    """16 hex digits of SHA-256 over the CSR arrays and (n, s, t)."""
    h = hashlib.sha256()
    for a in (np.asarray(g.off, np.int32), np.asarray(g.dst, np.int32), np.asarray(g.cap, np.int32)):
        h.update(a.tobytes())
    h.update(np.asarray([g.n, g.s, g.t], np.int64).tobytes())
    return h.hexdigest()[:16]


def flows_hash(flows) -> str:
    return hashlib.sha256(np.asarray(flows, np.int64).tobytes()).hexdigest()[:16]
