"""ctypes binding of libwbpr (include/wbpr.h).

Host-side mirror of the reference's solve path for Python callers and tests:
read or generate a CSR graph, create a device residual graph (RCSR or BCSR),
solve (thread-centric or vertex-centric), verify, read back state, min-cut
adjoint, and the reference drop-ins ``rcsr_preflow`` / ``rcsr_push_relabel``
(maxflow-cuda/src/preflow.cu:3-31, maxflow-cuda/src/push_relabel.cu:35-221).

Every call goes through the compiled library; there is no Python fallback.
A missing library or CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

_i32p = C.POINTER(C.c_int32)
_i8p = C.POINTER(C.c_int8)


class WbprError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: {status_str(status)} (status {status})"
        if detail:
            msg += f" [{detail}]"
        super().__init__(msg)


class CsrView(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_edges", C.c_int64), ("offsets", _i32p),
                ("destinations", _i32p), ("capacities", _i32p), ("source", C.c_int32),
                ("sink", C.c_int32)]


class HostCsr(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_edges", C.c_int64), ("num_edges_declared", C.c_int64),
                ("offsets", _i32p), ("destinations", _i32p), ("capacities", _i32p),
                ("source", C.c_int32), ("sink", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("tile", C.c_int32), ("block", C.c_int32), ("heavy_degree", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("gr_alpha", C.c_double), ("max_rounds", C.c_int64),
                ("max_ms", C.c_double), ("verify", C.c_int32), ("trace", C.c_int32),
                ("gr_rounds", C.c_int32), ("grid_blocks", C.c_int32), ("gr_stall", C.c_int32),
                ("barrier_timeout_ns", C.c_int64), ("greedy", C.c_int32), ("bfs_alpha", C.c_int32),
                ("gr_plateau", C.c_int32), ("matching", C.c_int32),
                ("pad2", C.c_int32), ("batch_cluster", C.c_int64)]


class Result(C.Structure):
    _fields_ = [("flow", C.c_int64), ("solve_ms", C.c_float), ("kernel_ms", C.c_float),
                ("gr_ms", C.c_float), ("arcs_scanned", C.c_uint64), ("pushes", C.c_uint64),
                ("relabels", C.c_uint64), ("vertex_visits", C.c_uint64), ("bfs_arcs", C.c_uint64),
                ("bfs_vertices", C.c_uint64), ("alg_bytes", C.c_uint64), ("rounds", C.c_int32),
                ("global_relabels", C.c_int32), ("stranded", C.c_int32), ("launch_ms", C.c_float),
                ("push_ms", C.c_float), ("bfs_levels", C.c_int32), ("bfs_bottom_up_levels", C.c_int32),
                ("heavy_visits", C.c_uint64), ("bytes_push", C.c_uint64), ("bytes_deep", C.c_uint64),
                ("bytes_relabel", C.c_uint64), ("bytes_gr", C.c_uint64), ("deep_ms", C.c_float),
                ("matching", C.c_int32), ("deep_arcs_scanned", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class VerifyReport(C.Structure):
    _fields_ = [("ok", C.c_int32), ("capacity_violations", C.c_int32),
                ("conservation_violations", C.c_int32), ("source_reaches_sink", C.c_int32),
                ("excess_reaches_sink", C.c_int32), ("label_violations", C.c_int32),
                ("cut_value", C.c_int64), ("flow_value", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


LAYOUTS = {"rcsr": 0, "bcsr": 1, "bcsr2": 2}
ALGOS = {"tc": 0, "vc": 1, 0: 0, 1: 1}

# every symbol declared in include/wbpr.h
EXPORTED = [
    "wbpr_status_str", "wbpr_abi_version", "wbpr_default_tuning", "wbpr_device_count",
    "wbpr_last_error", "wbpr_read_snap_txt", "wbpr_read_snap_bin", "wbpr_read_dimacs",
    "wbpr_write_snap_bin", "wbpr_write_dimacs", "wbpr_write_graph_cache", "wbpr_read_graph_cache",
    "wbpr_write_dimacs_flow", "wbpr_bipartite_network", "wbpr_complete_flow", "wbpr_cut_sides",
    "wbpr_host_csr_copy", "wbpr_host_csr_free",
    "wbpr_gen_genrmf", "wbpr_gen_rmat", "wbpr_gen_bipartite", "wbpr_gen_layered", "wbpr_gen_grid",
    "wbpr_build_rcsr", "wbpr_build_bcsr", "wbpr_build_bcsr2", "wbpr_graph_create",
    "wbpr_graph_destroy", "wbpr_graph_device_bytes", "wbpr_graph_read_bcsr", "wbpr_graph_read_rcsr", "wbpr_graph_set_stream", "wbpr_graph_set_capacities", "wbpr_autotune", "wbpr_solve_pairs", "wbpr_solve", "wbpr_read_state",
    "wbpr_verify", "wbpr_mincut_adjoint", "wbpr_rcsr_preflow", "wbpr_rcsr_push_relabel",
    "wbpr_read_trace", "wbpr_solve_bcsr_noalloc", "wbpr_batch_create", "wbpr_batch_destroy",
    "wbpr_batch_device_bytes", "wbpr_batch_solve", "wbpr_batch_instance_stats", "wbpr_batch_autotune",
    "wbpr_memory_cache",
]

_lib = None


def lib() -> C.CDLL:
    """Load libwbpr.so (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if os.environ.get("WBPR_CHECKED") == "1":  # bounds-checked solver kernels
        path = _build.build_checked()
    elif not os.path.exists(path) or os.environ.get("WBPR_REBUILD"):
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    hp = C.POINTER(C.POINTER(HostCsr))
    sig = {
        "wbpr_status_str": (C.c_char_p, [C.c_int]),
        "wbpr_abi_version": (C.c_int32, []),
        "wbpr_default_tuning": (None, [C.POINTER(Tuning)]),
        "wbpr_device_count": (C.c_int32, []),
        "wbpr_last_error": (C.c_char_p, []),
        "wbpr_read_snap_txt": (C.c_int, [C.c_char_p, hp]),
        "wbpr_read_snap_bin": (C.c_int, [C.c_char_p, hp]),
        "wbpr_read_dimacs": (C.c_int, [C.c_char_p, hp]),
        "wbpr_write_snap_bin": (C.c_int, [C.c_char_p, C.POINTER(CsrView)]),
        "wbpr_write_dimacs": (C.c_int, [C.c_char_p, C.POINTER(CsrView)]),
        "wbpr_write_graph_cache": (C.c_int, [C.c_char_p, C.POINTER(CsrView)]),
        "wbpr_read_graph_cache": (C.c_int, [C.c_char_p, hp]),
        "wbpr_write_dimacs_flow": (C.c_int, [C.c_char_p, C.POINTER(CsrView), C.c_int64, _i32p]),
        "wbpr_bipartite_network": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, _i32p, _i32p, hp]),
        "wbpr_complete_flow": (C.c_int, [vp, C.POINTER(C.c_float)]),
        "wbpr_cut_sides": (C.c_int, [vp, C.c_int32, _i8p]),
        "wbpr_host_csr_copy": (C.c_int, [C.POINTER(CsrView), hp]),
        "wbpr_host_csr_free": (None, [C.POINTER(HostCsr)]),
        "wbpr_gen_genrmf": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, hp]),
        "wbpr_gen_rmat": (C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                                    C.c_int32, C.c_int32, C.c_uint64, hp]),
        "wbpr_gen_bipartite": (C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_uint64, hp]),
        "wbpr_gen_layered": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_int32, C.c_uint64, hp]),
        "wbpr_gen_grid": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, hp]),
        "wbpr_build_rcsr": (C.c_int, [C.POINTER(CsrView), _i32p, _i32p, _i32p]),
        "wbpr_build_bcsr": (C.c_int, [C.POINTER(CsrView), _i32p, _i32p, _i32p, _i32p]),
        "wbpr_build_bcsr2": (C.c_int, [C.POINTER(CsrView), _i32p, _i32p, _i32p]),
        "wbpr_graph_create": (C.c_int, [C.POINTER(CsrView), C.c_int, C.POINTER(vp)]),
        "wbpr_graph_destroy": (C.c_int, [vp]),
        "wbpr_graph_device_bytes": (C.c_int64, [vp]),
        "wbpr_memory_cache": (C.c_int, [C.c_int64]),
        "wbpr_graph_read_bcsr": (C.c_int, [vp, _i32p, _i32p, _i32p, _i32p]),
        "wbpr_graph_read_rcsr": (C.c_int, [vp, _i32p, _i32p, _i32p]),
        "wbpr_graph_set_stream": (C.c_int, [vp, vp]),
        "wbpr_graph_set_capacities": (C.c_int, [vp, _i32p]),
        "wbpr_solve_pairs": (C.c_int, [vp, C.c_int32, _i32p, _i32p, C.c_int, C.POINTER(Tuning),
                                       C.POINTER(C.c_int64), C.POINTER(Result)]),
        "wbpr_autotune": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_float)]),
        "wbpr_solve": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int, C.POINTER(Tuning), C.POINTER(Result)]),
        "wbpr_read_state": (C.c_int, [vp, _i32p, _i32p, _i32p]),
        "wbpr_read_trace": (C.c_int32, [vp, C.POINTER(C.c_int64), C.c_int32]),
        "wbpr_batch_create": (C.c_int, [C.POINTER(CsrView), C.c_int32, C.POINTER(vp)]),
        "wbpr_batch_destroy": (C.c_int, [vp]),
        "wbpr_batch_device_bytes": (C.c_int64, [vp]),
        "wbpr_batch_solve": (C.c_int, [vp, C.POINTER(Tuning), C.POINTER(C.c_int64), C.POINTER(C.c_float)]),
        "wbpr_batch_instance_stats": (C.c_int, [vp, C.POINTER(C.c_float), _i32p]),
        "wbpr_batch_autotune": (C.c_int, [vp, C.POINTER(Tuning), C.POINTER(C.c_float)]),
        "wbpr_solve_bcsr_noalloc": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                              C.POINTER(C.c_int64)]),
        "wbpr_verify": (C.c_int, [vp, C.POINTER(VerifyReport)]),
        "wbpr_mincut_adjoint": (C.c_int, [vp, C.c_int32, _i8p, C.POINTER(C.c_float)]),
        "wbpr_rcsr_preflow": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, _i32p, _i32p, _i32p, _i32p,
                                          _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]),
        "wbpr_rcsr_push_relabel": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                               _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p,
                                               _i32p, _i32p, _i32p, _i32p, C.POINTER(C.c_float)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def status_str(st: int) -> str:
    return lib().wbpr_status_str(st).decode()


def _check(st: int, what: str) -> None:
    if st != 0:
        raise WbprError(st, what, lib().wbpr_last_error().decode())


def device_count() -> int:
    return int(lib().wbpr_device_count())


def memory_cache(max_bytes: int) -> None:
    """Keep at most max_bytes of freed device memory reserved in the
    library's pool on the current device (0 returns it all to the driver)."""
    _check(lib().wbpr_memory_cache(int(max_bytes)), "wbpr_memory_cache")


def _p(a: np.ndarray):
    return a.ctypes.data_as(_i32p)


@dataclass
class Graph:
    """Host CSR graph (the reference's CSRGraph, maxflow-cuda/include/graph.h:28-58)."""
    n: int
    off: np.ndarray
    dst: np.ndarray
    cap: np.ndarray
    s: int = -1
    t: int = -1
    m_declared: int = -1
    _keep: list = field(default_factory=list, repr=False)

    @property
    def m(self) -> int:
        return int(len(self.dst))

    def view(self) -> CsrView:
        self.off = np.ascontiguousarray(self.off, dtype=np.int32)
        self.dst = np.ascontiguousarray(self.dst, dtype=np.int32)
        self.cap = np.ascontiguousarray(self.cap, dtype=np.int32)
        d = self.dst if len(self.dst) else np.zeros(1, np.int32)
        c = self.cap if len(self.cap) else np.zeros(1, np.int32)
        self._keep = [d, c]
        return CsrView(self.n, self.m, _p(self.off), _p(d), _p(c), self.s, self.t)

    def arcs(self):
        """(tail, head, cap) arrays, input order."""
        tail = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.off))
        return tail, self.dst, self.cap

    @staticmethod
    def from_arcs(n: int, tail, head, cap, s: int, t: int) -> "Graph":
        """CSR grouped by tail, keeping the given order inside each row."""
        tail = np.asarray(tail, np.int64)
        order = np.argsort(tail, kind="stable")
        off = np.zeros(n + 1, np.int64)
        np.add.at(off, tail + 1, 1)
        return Graph(n, np.cumsum(off).astype(np.int32), np.asarray(head, np.int32)[order],
                     np.asarray(cap, np.int32)[order], s, t)


class _HostCsrMemory:
    """A wbpr_host_csr the library returned: its arrays are viewed in place
    (no copy) and released with the last numpy array that views them."""

    def __init__(self, ptr):
        self._ptr = ptr

    def __del__(self):
        if self._ptr is not None:
            try:
                lib().wbpr_host_csr_free(self._ptr)
            except Exception:  # interpreter shutdown
                pass
            self._ptr = None


def _viewed(owner, cptr, count: int) -> np.ndarray:
    if count == 0:
        return np.zeros(0, np.int32)
    buf = (C.c_int32 * count).from_address(C.cast(cptr, C.c_void_p).value)
    buf._owner = owner  # the ctypes array keeps the C memory, the numpy array keeps the ctypes array
    return np.frombuffer(buf, dtype=np.int32)


def _take(ptr) -> Graph:
    h = ptr.contents
    n, m = h.num_nodes, h.num_edges
    owner = _HostCsrMemory(ptr)
    off = _viewed(owner, h.offsets, n + 1)
    dst = _viewed(owner, h.destinations, m)
    cap = _viewed(owner, h.capacities, m)
    return Graph(n, off, dst, cap, h.source, h.sink, h.num_edges_declared)


def _reader(fn: str, path: str) -> Graph:
    out = C.POINTER(HostCsr)()
    _check(getattr(lib(), fn)(os.fsencode(path), C.byref(out)), fn)
    return _take(out)


def read_snap_txt(path: str) -> Graph:
    return _reader("wbpr_read_snap_txt", path)


def read_snap_bin(path: str) -> Graph:
    return _reader("wbpr_read_snap_bin", path)


def read_dimacs(path: str) -> Graph:
    return _reader("wbpr_read_dimacs", path)


def read_graph_cache(path: str) -> Graph:
    """The library's own cache format (capacities and terminals included)."""
    return _reader("wbpr_read_graph_cache", path)


def read_graph(path: str, file_type: int) -> Graph:
    """file_type as the CLI's -v: 0 SNAP text, 1 SNAP binary, 2 DIMACS, 3 cache."""
    return [read_snap_txt, read_snap_bin, read_dimacs, read_graph_cache][file_type](path)


def write_graph_cache(path: str, g: Graph) -> None:
    v = g.view()
    _check(lib().wbpr_write_graph_cache(os.fsencode(path), C.byref(v)), "wbpr_write_graph_cache")


def write_dimacs_flow(path: str, g: Graph, flow: int, arc_flow) -> None:
    """DIMACS solution: "s <flow>" and "f u v x" for every arc carrying flow."""
    v = g.view()
    f = np.ascontiguousarray(arc_flow, np.int32)
    if f.shape != (g.m,):
        raise ValueError("arc_flow must hold one value per input arc")
    _check(lib().wbpr_write_dimacs_flow(os.fsencode(path), C.byref(v), int(flow), _p(f)),
           "wbpr_write_dimacs_flow")


def bipartite_network(L: int, R: int, left, right) -> Graph:
    """Unit-capacity matching network: left 0..L-1, right L..L+R-1,
    s = L+R, t = L+R+1 (pairs are 0-based within their side)."""
    lt = np.ascontiguousarray(left, np.int32)
    rt = np.ascontiguousarray(right, np.int32)
    if lt.shape != rt.shape:
        raise ValueError("left and right must have the same length")
    out = C.POINTER(HostCsr)()
    _check(lib().wbpr_bipartite_network(L, R, lt.size, _p(lt), _p(rt), C.byref(out)), "wbpr_bipartite_network")
    return _take(out)


def bipartite_matching(L: int, R: int, left, right, **tuning):
    """Maximum matching of a bipartite graph: (size, pairs) with pairs an
    (size, 2) array of (left id, right id)."""
    g = bipartite_network(L, R, left, right)
    with DeviceGraph(g, "bcsr") as d:
        r = d.solve("vc", g.s, g.t, **tuning)
        d.complete_flow()
        _, _, f = d.read_state()
    tails = np.repeat(np.arange(g.n, dtype=np.int64), np.diff(g.off))
    sel = (tails < L) & (f > 0)
    pairs = np.stack([tails[sel], g.dst[sel].astype(np.int64) - L], axis=1)
    if len(pairs) != r.flow:
        raise WbprError(5, "matching size differs from the flow value")
    return int(r.flow), pairs


def write_dimacs(path: str, g: Graph) -> None:
    v = g.view()
    _check(lib().wbpr_write_dimacs(os.fsencode(path), C.byref(v)), "wbpr_write_dimacs")


def write_snap_bin(path: str, g: Graph) -> None:
    v = g.view()
    _check(lib().wbpr_write_snap_bin(os.fsencode(path), C.byref(v)), "wbpr_write_snap_bin")


def _gen(fn: str, *args) -> Graph:
    out = C.POINTER(HostCsr)()
    _check(getattr(lib(), fn)(*args, C.byref(out)), fn)
    return _take(out)


def gen_genrmf(a: int, b: int, c1: int = 1, c2: int = 10000, seed: int = 0) -> Graph:
    return _gen("wbpr_gen_genrmf", a, b, c1, c2, seed)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             cap_lo: int = 1, cap_hi: int = 100, seed: int = 1) -> Graph:
    return _gen("wbpr_gen_rmat", scale, edge_factor, a, b, c, cap_lo, cap_hi, seed)


def gen_bipartite(left: int, right: int, zipf_s: float = 2.0, dmax: int = 4096, seed: int = 0) -> Graph:
    return _gen("wbpr_gen_bipartite", left, right, zipf_s, dmax, seed)


def gen_layered(layers: int, width: int, deg_lo: int = 3, deg_hi: int = 6, cap_lo: int = 1,
                cap_hi: int = 1000, seed: int = 0) -> Graph:
    return _gen("wbpr_gen_layered", layers, width, deg_lo, deg_hi, cap_lo, cap_hi, seed)


def gen_grid(w: int, h: int, seed: int = 0) -> Graph:
    return _gen("wbpr_gen_grid", w, h, seed)


def build_rcsr(g: Graph):
    v = g.view()
    roff = np.zeros(g.n + 1, np.int32)
    rdst = np.zeros(max(g.m, 1), np.int32)
    fidx = np.zeros(max(g.m, 1), np.int32)
    _check(lib().wbpr_build_rcsr(C.byref(v), _p(roff), _p(rdst), _p(fidx)), "wbpr_build_rcsr")
    return roff, rdst[:g.m], fidx[:g.m]


def build_bcsr(g: Graph):
    v = g.view()
    off = np.zeros(g.n + 1, np.int32)
    k = max(2 * g.m, 1)
    dst, cap, bidx = (np.zeros(k, np.int32) for _ in range(3))
    _check(lib().wbpr_build_bcsr(C.byref(v), _p(off), _p(dst), _p(cap), _p(bidx)), "wbpr_build_bcsr")
    return off, dst[:2 * g.m], cap[:2 * g.m], bidx[:2 * g.m]


def build_bcsr2(g: Graph):
    v = g.view()
    off = np.zeros(g.n + 1, np.int32)
    dst = np.zeros(max(2 * g.m, 1), np.int32)
    flows = np.zeros(max(4 * g.m, 1), np.int32)
    _check(lib().wbpr_build_bcsr2(C.byref(v), _p(off), _p(dst), _p(flows)), "wbpr_build_bcsr2")
    return off, dst[:2 * g.m], flows[:4 * g.m]


def default_tuning(**kw) -> Tuning:
    t = Tuning()
    lib().wbpr_default_tuning(C.byref(t))
    for k, v in kw.items():
        if not hasattr(t, k):
            raise TypeError(f"unknown tuning field {k}")
        setattr(t, k, v)
    return t


class DeviceGraph:
    """Device residual graph (library-owned device memory)."""

    def __init__(self, g: Graph, layout: str = "bcsr"):
        self._h = None
        self.n, self.m = g.n, g.m
        self.s, self.t = g.s, g.t
        self.layout = layout
        v = g.view()
        h = C.c_void_p()
        _check(lib().wbpr_graph_create(C.byref(v), LAYOUTS[layout], C.byref(h)), "wbpr_graph_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().wbpr_graph_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(lib().wbpr_graph_device_bytes(self._h))

    def solve(self, algo="vc", s: int | None = None, t: int | None = None, **tuning) -> Result:
        r = Result()
        tu = default_tuning(**tuning)
        _check(lib().wbpr_solve(self._h, -1 if s is None else s, -1 if t is None else t, ALGOS[algo],
                                C.byref(tu), C.byref(r)), "wbpr_solve")
        if s is not None:
            self.s = s
        if t is not None:
            self.t = t
        return r

    def trace(self, cap: int = 1 << 14) -> np.ndarray:
        """Event records of the last solve run with trace=1: rows of
        (kind, aux, t_ns, v0, v1, max_block_ns, min_block_ns)."""
        buf = np.zeros((cap, 6), np.int64)
        n = lib().wbpr_read_trace(self._h, buf.ctypes.data_as(C.POINTER(C.c_int64)), cap)
        b = buf[:n]
        return np.stack([b[:, 0] & 0xffffffff, b[:, 0] >> 32, b[:, 1], b[:, 2], b[:, 3], b[:, 4], b[:, 5]],
                        axis=1)

    def verify(self) -> dict:
        rep = VerifyReport()
        _check(lib().wbpr_verify(self._h, C.byref(rep)), "wbpr_verify")
        return rep.as_dict()

    def read_bcsr(self):
        """The device-built BCSR arrays, as build_bcsr returns them."""
        off = np.zeros(self.n + 1, np.int32)
        k = max(2 * self.m, 1)
        dst, cap, bidx = (np.zeros(k, np.int32) for _ in range(3))
        _check(lib().wbpr_graph_read_bcsr(self._h, _p(off), _p(dst), _p(cap), _p(bidx)), "wbpr_graph_read_bcsr")
        return off, dst[:2 * self.m], cap[:2 * self.m], bidx[:2 * self.m]

    def read_rcsr(self):
        """The device-built RCSR reverse arrays, as build_rcsr returns them."""
        roff = np.zeros(self.n + 1, np.int32)
        k = max(self.m, 1)
        rdst, fidx = np.zeros(k, np.int32), np.zeros(k, np.int32)
        _check(lib().wbpr_graph_read_rcsr(self._h, _p(roff), _p(rdst), _p(fidx)), "wbpr_graph_read_rcsr")
        return roff, rdst[:self.m], fidx[:self.m]

    def read_state(self):
        h = np.zeros(self.n, np.int32)
        e = np.zeros(self.n, np.int32)
        f = np.zeros(max(self.m, 1), np.int32)
        _check(lib().wbpr_read_state(self._h, _p(h), _p(e), _p(f)), "wbpr_read_state")
        return h, e, f[:self.m]

    def solve_pairs(self, sources, sinks, algo="vc", **tuning):
        """Flows for many (source, sink) pairs in one solve (exact per pair when
        each pair has its own connected component); returns (flows, Result)."""
        src = np.ascontiguousarray(sources, np.int32)
        snk = np.ascontiguousarray(sinks, np.int32)
        if src.shape != snk.shape or src.ndim != 1:
            raise ValueError("sources and sinks must be 1-d and of the same length")
        flows = np.zeros(len(src), np.int64)
        r = Result()
        tu = default_tuning(**tuning)
        _check(lib().wbpr_solve_pairs(self._h, len(src), _p(src), _p(snk), ALGOS[algo], C.byref(tu),
                                      flows.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(r)), "wbpr_solve_pairs")
        return flows, r

    def autotune(self, algo="vc", s: int | None = None, t: int | None = None):
        """(best Tuning, its solve ms) over tile, relabel frequency and long-row threshold."""
        tu = Tuning()
        ms = C.c_float(0)
        _check(lib().wbpr_autotune(self._h, -1 if s is None else s, -1 if t is None else t, ALGOS[algo],
                                   C.byref(tu), C.byref(ms)), "wbpr_autotune")
        return tu, float(ms.value)

    def set_capacities(self, cap) -> None:
        """New capacities (input order) for the same topology; used by the next solve."""
        c = np.ascontiguousarray(cap, np.int32)
        if c.shape != (self.m,):
            raise ValueError("one capacity per input arc")
        _check(lib().wbpr_graph_set_capacities(self._h, _p(c) if self.m else None), "wbpr_graph_set_capacities")

    def set_stream(self, stream: int | None) -> None:
        """Queue this graph's device work on a caller's CUDA stream (a raw
        cudaStream_t handle, e.g. torch.cuda.Stream().cuda_stream); None
        returns to the graph's own stream."""
        _check(lib().wbpr_graph_set_stream(self._h, stream), "wbpr_graph_set_stream")

    def complete_flow(self) -> float:
        """Return stranded excess to s so the arc flows form a maximum flow."""
        ms = C.c_float(0)
        _check(lib().wbpr_complete_flow(self._h, C.byref(ms)), "wbpr_complete_flow")
        return float(ms.value)

    def cut_sides(self, side: int = 0) -> np.ndarray:
        """Per-vertex membership (int8) of T (side 0) or S (side 1)."""
        out = np.zeros(self.n, np.int8)
        _check(lib().wbpr_cut_sides(self._h, side, out.ctypes.data_as(_i8p)), "wbpr_cut_sides")
        return out

    def mincut_adjoint(self, side: int = 0):
        ind = np.zeros(max(self.m, 1), np.int8)
        ms = C.c_float(0)
        _check(lib().wbpr_mincut_adjoint(self._h, side, ind.ctypes.data_as(_i8p), C.byref(ms)),
               "wbpr_mincut_adjoint")
        return ind[:self.m], float(ms.value)


class Batch:
    """Many independent instances solved in one launch (wbpr_batch_*)."""

    def __init__(self, graphs: list):
        self._h = None
        views = (CsrView * len(graphs))()
        self._graphs = list(graphs)
        for i, g in enumerate(self._graphs):
            views[i] = g.view()
        h = C.c_void_p()
        _check(lib().wbpr_batch_create(views, len(graphs), C.byref(h)), "wbpr_batch_create")
        self._h = h
        self.count = len(graphs)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().wbpr_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(lib().wbpr_batch_device_bytes(self._h))

    def solve(self, tuning: Tuning | None = None, **kw):
        """Returns (flows array, device ms)."""
        tu = tuning if tuning is not None else default_tuning(**kw)
        flows = np.zeros(self.count, np.int64)
        ms = C.c_float(0)
        _check(lib().wbpr_batch_solve(self._h, C.byref(tu), flows.ctypes.data_as(C.POINTER(C.c_int64)),
                                      C.byref(ms)), "wbpr_batch_solve")
        return flows, float(ms.value)

    def instance_stats(self):
        ms = np.zeros(self.count, np.float32)
        rounds = np.zeros(self.count, np.int32)
        _check(lib().wbpr_batch_instance_stats(self._h, ms.ctypes.data_as(C.POINTER(C.c_float)), _p(rounds)),
               "wbpr_batch_instance_stats")
        return ms, rounds

    def autotune(self):
        t = Tuning()
        ms = C.c_float(0)
        _check(lib().wbpr_batch_autotune(self._h, C.byref(t), C.byref(ms)), "wbpr_batch_autotune")
        return t, float(ms.value)


def disjoint_union(graphs: list):
    """One graph holding every graph of the list as its own component: returns
    (graph, sources, sinks) with each graph's terminals at their new ids."""
    offs, dsts, caps, srcs, snks = [np.zeros(1, np.int64)], [], [], [], []
    base, arc_base = 0, 0
    for g in graphs:
        offs.append(g.off[1:].astype(np.int64) + arc_base)
        dsts.append(g.dst.astype(np.int64) + base)
        caps.append(g.cap)
        srcs.append(g.s + base)
        snks.append(g.t + base)
        base += g.n
        arc_base += g.m
    u = Graph(base, np.concatenate(offs).astype(np.int32), np.concatenate(dsts).astype(np.int32),
              np.concatenate(caps).astype(np.int32), int(srcs[0]), int(snks[0]))
    return u, np.array(srcs, np.int32), np.array(snks, np.int32)


def maxflow(g: Graph, algo="vc", layout="bcsr", **tuning) -> int:
    with DeviceGraph(g, layout) as d:
        return int(d.solve(algo, g.s, g.t, **tuning).flow)


def rcsr_preflow(g: Graph, roff, rdst, fidx):
    """Reference preflow() over host RCSR arrays; returns the mutable state."""
    n = g.n
    h = np.zeros(n, np.int32)
    e = np.zeros(n, np.int32)
    ff = g.cap.astype(np.int32).copy()
    bf = np.zeros_like(ff)
    tot = C.c_int32(0)
    _check(lib().wbpr_rcsr_preflow(n, g.s, g.t, _p(h), _p(e), _p(g.off), _p(g.dst), _p(g.cap), _p(ff),
                                   _p(bf), _p(roff), _p(rdst), _p(fidx), C.byref(tot)), "wbpr_rcsr_preflow")
    return h, e, ff, bf, int(tot.value)


def rcsr_push_relabel(algo_type: int, g: Graph, state, roff, rdst, fidx):
    """Reference push_relabel() drop-in; mutates `state` in place and returns
    (max flow = excess[sink], Excess_total, kernel_ms)."""
    h, e, ff, bf, _ = state
    tot = C.c_int32(0)
    ms = C.c_float(0)
    _check(lib().wbpr_rcsr_push_relabel(algo_type, g.n, g.m, g.s, g.t, _p(h), _p(e), _p(g.off), _p(g.dst),
                                        _p(g.cap), _p(ff), _p(bf), _p(roff), _p(rdst), _p(fidx),
                                        C.byref(tot), C.byref(ms)), "wbpr_rcsr_push_relabel")
    return int(e[g.t]), int(tot.value), float(ms.value)
