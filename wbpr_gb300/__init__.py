"""GB300-native push-relabel maximum-flow solver (drop-in for WBPR's path).

The compute path is libwbpr.so (CUDA for sm_103a behind the C ABI in
include/wbpr.h); this package only binds it.
"""
from .api import (ALGOS, EXPORTED, LAYOUTS, Batch, DeviceGraph, Graph, WbprError, bipartite_matching,
                  bipartite_network, build_bcsr, build_bcsr2, build_rcsr, default_tuning, device_count,
                  disjoint_union, gen_bipartite, gen_genrmf, gen_grid, gen_layered, gen_rmat, lib, maxflow,
                  memory_cache, rcsr_preflow,
                  rcsr_push_relabel, read_dimacs, read_graph, read_graph_cache, read_snap_bin, read_snap_txt,
                  status_str, write_dimacs, write_dimacs_flow, write_graph_cache, write_snap_bin)

__all__ = [
    "ALGOS", "EXPORTED", "LAYOUTS", "Batch", "DeviceGraph", "Graph", "WbprError", "bipartite_matching",
    "bipartite_network", "build_bcsr", "build_bcsr2", "build_rcsr", "default_tuning", "device_count",
    "disjoint_union", "gen_bipartite", "gen_genrmf", "gen_grid", "gen_layered", "gen_rmat", "lib", "maxflow",
    "memory_cache", "rcsr_preflow",
    "rcsr_push_relabel", "read_dimacs", "read_graph", "read_graph_cache", "read_snap_bin", "read_snap_txt",
    "status_str", "write_dimacs", "write_dimacs_flow", "write_graph_cache", "write_snap_bin",
]
