"""Host logic of libwbpr without a GPU: ABI surface, readers and writers,
residual builders (exact reverse pairing), seeded generators, CLI errors."""
import os
import re
import subprocess

import numpy as np
import pytest

import wbpr_gb300 as W
from wbpr_gb300 import build as wb
from conftest import ROOT, graph_of


def header_functions():
    src = open(os.path.join(ROOT, "include", "wbpr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(wbpr_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = W.lib()
    declared = header_functions()
    assert set(declared) == set(W.EXPORTED)
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.wbpr_abi_version() == 2


def test_status_strings():
    for s in range(9):
        assert W.status_str(s)
    assert W.status_str(0) == "ok"


def test_no_device_is_reported_not_faked(has_gpu):
    if has_gpu:
        pytest.skip("host has a GPU")
    g = W.gen_genrmf(3, 3, 1, 10, 0)
    with pytest.raises(W.WbprError) as ei:
        W.DeviceGraph(g, "bcsr")
    assert ei.value.status == 7  # WBPR_ERR_NO_DEVICE
    with pytest.raises(W.WbprError) as ei:
        W.memory_cache(1 << 30)
    assert ei.value.status == 7


def test_memory_cache_rejects_negative_sizes():
    # checked before any device is touched
    with pytest.raises(W.WbprError) as ei:
        W.memory_cache(-1)
    assert ei.value.status == 1


def test_dimacs_roundtrip(tmp_path, golden):
    for c in golden[:12]:
        g = graph_of(c)
        p = str(tmp_path / "g.dimacs")
        W.write_dimacs(p, g)
        h = W.read_dimacs(p)
        assert (h.n, h.s, h.t) == (g.n, g.s, g.t)
        assert np.array_equal(h.off, g.off) and np.array_equal(h.dst, g.dst)
        assert np.array_equal(h.cap, g.cap)


def test_snap_readers(tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("# Directed graph\n# Nodes: 5 Edges: 6\n0 3\n0 1\n0 2\n1 4\n2 4\n3 4\n")
    g = W.read_snap_txt(str(p))
    assert g.n == 5 and g.m == 6
    assert list(g.dst[g.off[0]:g.off[1]]) == [1, 2, 3]  # rows sorted by head
    assert (g.cap == 1).all()
    b = str(tmp_path / "g.bin")
    W.write_snap_bin(b, g)
    h = W.read_snap_bin(b)
    assert np.array_equal(h.off, g.off) and np.array_equal(h.dst, g.dst) and (h.cap == 1).all()


@pytest.mark.parametrize("text", [
    "p max 3 1\na 1 4 5\n",          # head out of range
    "p max 3 1\na 1 2\n",            # truncated arc line
    "a 1 2 3\n",                     # arc before problem line
    "p max 3 1\na 1 2 -4\n",         # negative capacity
    "p max 3 1\nq 1 2 3\n",          # unknown line type
    "p max -2 1\n",                  # bad vertex count
])
def test_malformed_dimacs_is_an_io_error(tmp_path, text):
    p = tmp_path / "bad.dimacs"
    p.write_text(text)
    with pytest.raises(W.WbprError) as ei:
        W.read_dimacs(str(p))
    assert ei.value.status == 6


def test_missing_and_truncated_files(tmp_path):
    with pytest.raises(W.WbprError) as ei:
        W.read_dimacs(str(tmp_path / "nope"))
    assert ei.value.status == 6
    b = tmp_path / "t.bin"
    b.write_bytes(np.asarray([5, 6, 6, 1, 2], np.int32).tobytes())
    with pytest.raises(W.WbprError):
        W.read_snap_bin(str(b))


def _check_pairing_bcsr(g, off, dst, cap, bidx):
    n, m = g.n, g.m
    assert off[-1] == 2 * m
    tail = np.repeat(np.arange(n), np.diff(off))
    assert (bidx[bidx] == np.arange(2 * m)).all()          # involution
    assert (dst[bidx] == tail).all() and (tail[bidx] == dst).all()
    assert ((cap == 0) | (cap[bidx] == 0)).all()           # one side of each pair is a twin
    assert cap.sum() == g.cap.sum()


def test_bcsr_builders_pair_exactly():
    # parallel and antiparallel arcs included
    g = W.Graph.from_arcs(4, [0, 0, 1, 2, 1, 3, 2], [1, 1, 0, 3, 2, 1, 3], [3, 4, 5, 6, 7, 8, 9], 0, 3)
    off, dst, cap, bidx = W.build_bcsr(g)
    _check_pairing_bcsr(g, off, dst, cap, bidx)
    off2, dst2, flows = W.build_bcsr2(g)
    assert np.array_equal(off2, off) and np.array_equal(dst2, dst)
    assert np.array_equal(flows[0::2], cap) and np.array_equal(flows[1::2], bidx)
    for seed in range(5):
        h = W.gen_rmat(8, 8, seed=seed)
        _check_pairing_bcsr(h, *W.build_bcsr(h))


def test_rcsr_builder_pairs_exactly():
    g = W.Graph.from_arcs(4, [0, 0, 1, 2, 1, 3, 2], [1, 1, 0, 3, 2, 1, 3], [3, 4, 5, 6, 7, 8, 9], 0, 3)
    roff, rdst, fidx = W.build_rcsr(g)
    tail = np.repeat(np.arange(g.n), np.diff(g.off))
    assert sorted(fidx.tolist()) == list(range(g.m))        # a permutation (no first-match aliasing)
    rhead = np.repeat(np.arange(g.n), np.diff(roff))
    assert (g.dst[fidx] == rhead).all() and (tail[fidx] == rdst).all()


def test_generator_shapes():
    g = W.gen_genrmf(8, 16, 1, 10000, 1)
    assert (g.n, g.m, g.s, g.t) == (1024, 4544, 0, 1023)
    tail, head, cap = g.arcs()
    inframe = (tail // 64) == (head // 64)
    assert (cap[inframe] == 640000).all()
    assert ((cap[~inframe] >= 1) & (cap[~inframe] <= 10000)).all()
    r = W.gen_rmat(10, 16, seed=3)
    tail, head, cap = r.arcs()
    assert (tail != head).all()
    assert len(np.unique(tail.astype(np.int64) * r.n + head)) == r.m
    assert cap.min() >= 1 and cap.max() <= 100
    deg = np.diff(r.off)
    assert r.s == int(np.argmax(deg))
    b = W.gen_bipartite(200, 150, 2.0, 4096, 2)
    assert b.n == 352 and b.s == 0 and b.t == 351 and (b.cap == 1).all()
    lay = W.gen_layered(5, 7, 3, 6, 1, 1000, 1)
    assert lay.n == 37
    grid = W.gen_grid(16, 12, 4)
    assert grid.n == 16 * 12 + 2 and grid.m == 2 * (15 * 12 + 16 * 11) + 2 * 16 * 12


def test_generators_are_pinned(golden):
    """Same seed, same bits: hashes recorded by the golden script."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    make = {
        "genrmf_a4_b6_s0": lambda: W.gen_genrmf(4, 6, 1, 10000, 0),
        "genrmf_a8_b16_s1": lambda: W.gen_genrmf(8, 16, 1, 10000, 1),
        "layered_6x12_s3": lambda: W.gen_layered(6, 12, 3, 6, 1, 1000, 3),
        "bipartite_40x30_s5": lambda: W.gen_bipartite(40, 30, 2.0, 4096, 5),
        "grid_8x8_s2": lambda: W.gen_grid(8, 8, 2),
        "rmat_s7_s1": lambda: W.gen_rmat(7, 8, 0.57, 0.19, 0.19, 1, 100, 1),
    }
    hashes = {c["name"]: c.get("csr_hash") for c in golden}
    for name, fn in make.items():
        assert mg.csr_hash(fn()) == hashes[name], name


def test_rmat_independent_of_thread_count():
    env = dict(os.environ, WBPR_HOST_THREADS="1")
    code = ("import sys; sys.path.insert(0, %r); import wbpr_gb300 as W, hashlib;"
            "g=W.gen_rmat(12,16,seed=9); print(hashlib.sha256(g.dst.tobytes()+g.cap.tobytes()).hexdigest())" % ROOT)
    one = subprocess.run(["python3", "-c", code], env=env, capture_output=True, text=True, check=True).stdout
    many = subprocess.run(["python3", "-c", code], capture_output=True, text=True, check=True).stdout
    assert one == many


def test_overflowing_arc_count_is_rejected_on_the_host():
    # more than 2^31 - 1 input arcs: refused by the host checks before any
    # array is read or any device call is made (incoming-capacity sums that
    # overflow int32 are refused by the device build, see the GPU tests)
    dummy = np.zeros(4, np.int32)
    v = W.api.CsrView()
    v.num_nodes = 3
    v.num_edges = 2**31
    v.offsets = v.destinations = v.capacities = dummy.ctypes.data_as(W.api._i32p)
    for layout in (0, 1):
        h = W.api.C.c_void_p()
        assert W.lib().wbpr_graph_create(W.api.C.byref(v), layout, W.api.C.byref(h)) == 4


def test_cli_usage_and_errors(tmp_path):
    cli = wb.CLI
    r = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Vertex-centric push-relabel" in r.stdout
    r = subprocess.run([cli, "-v", "2", "-f", str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([cli, "-v", "9", "-f", "x"], capture_output=True, text=True)
    assert r.returncode == 1 and "Invalid file type" in r.stdout


# ---- graph cache, DIMACS solution writer, bipartite network ---------------
def test_graph_cache_round_trip(tmp_path):
    g = W.gen_genrmf(4, 6, 1, 500, 2)
    p = str(tmp_path / "g.wgc")
    W.write_graph_cache(p, g)
    h = W.read_graph_cache(p)
    assert (h.n, h.m, h.s, h.t) == (g.n, g.m, g.s, g.t)
    assert np.array_equal(h.off, g.off) and np.array_equal(h.dst, g.dst) and np.array_equal(h.cap, g.cap)
    # without capacities the cache stores none and reads back capacity 1
    v = g.view()
    v.capacities = None
    q = str(tmp_path / "u.wgc")
    assert W.lib().wbpr_write_graph_cache(os.fsencode(q), W.api.C.byref(v)) == 0
    u = W.read_graph_cache(q)
    assert np.array_equal(u.dst, g.dst) and np.all(u.cap == 1)
    assert os.path.getsize(q) == 48 + 4 * (g.n + 1 + g.m)


def test_graph_cache_rejects_damage(tmp_path):
    g = W.gen_genrmf(3, 3, 1, 50, 1)
    p = tmp_path / "g.wgc"
    W.write_graph_cache(str(p), g)
    raw = p.read_bytes()
    for bad in (raw[:-4], raw + b"\0\0\0\0", b"WBPRCSR2" + raw[8:], raw[:8] + b"\2\0\0\0" + raw[12:]):
        p.write_bytes(bad)
        with pytest.raises(W.WbprError) as ei:
            W.read_graph_cache(str(p))
        assert ei.value.status == 6
    # an arc head out of range
    arr = bytearray(raw)
    at = 48 + 4 * (g.n + 1)
    arr[at:at + 4] = (g.n + 5).to_bytes(4, "little")
    p.write_bytes(bytes(arr))
    with pytest.raises(W.WbprError):
        W.read_graph_cache(str(p))


def test_dimacs_reader_is_thread_count_independent(tmp_path):
    g = W.gen_rmat(12, 8, seed=4)
    p = str(tmp_path / "r.dimacs")
    W.write_dimacs(p, g)
    # comments and a terminal line among the arcs; the last "n s" counts
    lines = open(p).read().splitlines()
    lines.insert(len(lines) // 2, "c a comment in the middle")
    lines.insert(len(lines) // 3, f"n {g.t + 1} t")
    lines.append(f"n {g.s + 1} s")
    open(p, "w").write("\n".join(lines) + "\n")
    code = ("import sys, hashlib; sys.path.insert(0, %r); import wbpr_gb300 as W; g = W.read_dimacs(%r);"
            "print(g.n, g.m, g.s, g.t, hashlib.sha256(g.off.tobytes() + g.dst.tobytes() + g.cap.tobytes())"
            ".hexdigest())" % (ROOT, p))
    one = subprocess.run(["python3", "-c", code], env=dict(os.environ, WBPR_HOST_THREADS="1"),
                         capture_output=True, text=True, check=True).stdout
    many = subprocess.run(["python3", "-c", code], env=dict(os.environ, WBPR_HOST_THREADS="7"),
                          capture_output=True, text=True, check=True).stdout
    assert one == many
    h = W.read_dimacs(p)
    assert np.array_equal(h.dst, g.dst) and np.array_equal(h.cap, g.cap) and (h.s, h.t) == (g.s, g.t)


def test_dimacs_problem_line_after_arcs_is_rejected(tmp_path):
    p = tmp_path / "bad.dimacs"
    p.write_text("p max 3 2\nn 1 s\nn 3 t\na 1 2 5\np max 3 2\na 2 3 5\n")
    with pytest.raises(W.WbprError) as ei:
        W.read_dimacs(str(p))
    assert ei.value.status == 6


def test_dimacs_flow_writer(tmp_path):
    g = W.Graph.from_arcs(4, [0, 0, 1, 2, 1], [1, 2, 3, 3, 2], [3, 2, 2, 3, 1], 0, 3)
    flow = np.array([2, 2, 0, 2, 0], np.int32)  # in CSR order: 0->1, 0->2, 1->3, 1->2, 2->3
    p = str(tmp_path / "sol.txt")
    W.write_dimacs_flow(p, g, 4, flow)
    text = open(p).read().splitlines()
    assert text[1] == "s 4"
    f_lines = [t for t in text if t.startswith("f ")]
    heads = {(int(a), int(b)): int(c) for _, a, b, c in (t.split() for t in f_lines)}
    tails = np.repeat(np.arange(g.n), np.diff(g.off))
    expect = {(int(tails[i]) + 1, int(g.dst[i]) + 1): int(flow[i]) for i in range(g.m) if flow[i] > 0}
    assert heads == expect
    with pytest.raises(ValueError):
        W.write_dimacs_flow(p, g, 4, flow[:3])


def test_bipartite_network_shape():
    g = W.bipartite_network(3, 2, [0, 1, 1, 2, 0], [0, 0, 1, 1, 0])
    assert (g.n, g.s, g.t) == (7, 5, 6)
    tails = np.repeat(np.arange(g.n), np.diff(g.off))
    arcs = sorted(zip(tails.tolist(), g.dst.tolist()))
    assert arcs == sorted([(0, 3), (1, 3), (1, 4), (2, 4), (3, 6), (4, 6), (5, 0), (5, 1), (5, 2)])
    assert np.all(g.cap == 1)
    for left, right in (([3], [0]), ([0], [2]), ([-1], [0])):
        with pytest.raises(W.WbprError) as ei:
            W.bipartite_network(3, 2, left, right)
        assert ei.value.status == 1


def test_header_is_plain_c_and_links(tmp_path):
    """A C99 caller (the reference's host code is C-style) compiles against
    include/wbpr.h and links libwbpr.so; calls with bad arguments return
    status codes instead of exiting."""
    src = tmp_path / "caller.c"
    src.write_text(r"""
#include <stdio.h>
#include "wbpr.h"
int main(void) {
  wbpr_tuning tu;
  wbpr_graph* g = 0;
  wbpr_default_tuning(&tu);
  if (wbpr_graph_create(0, WBPR_LAYOUT_BCSR, &g) != WBPR_ERR_INVALID_ARG) return 1;
  if (wbpr_solve(0, 0, 1, WBPR_ALGO_VC, &tu, 0) != WBPR_ERR_INVALID_ARG) return 2;
  if (wbpr_read_dimacs("/nonexistent/file", 0) == WBPR_OK) return 3;
  printf("abi %d tile %d gr_alpha %.2f\n", wbpr_abi_version(), tu.tile, tu.gr_alpha);
  return 0;
}
""")
    exe = tmp_path / "caller"
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(wb.LIB)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", inc, str(src),
                    "-L", libdir, "-lwbpr", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("abi "), (r.returncode, r.stdout, r.stderr)


def test_dimacs_reader_shuffled_and_grouped_arcs(tmp_path):
    """Arc lines in any order are grouped by tail keeping file order inside
    each row; arcs already grouped take the direct path.  Both give the same
    CSR for 1 or 7 threads, with LF or CRLF line ends, blank and comment lines
    among the arcs, and rows without arcs at both ends."""
    import hashlib
    rng = np.random.default_rng(3)
    n, m = 300, 4000
    tail = rng.integers(5, n - 40, m)  # vertices 0-4 and the last 40 have no out-arcs
    head = rng.integers(0, n, m)
    cap = rng.integers(0, 1000, m)
    expect = W.Graph.from_arcs(n, tail, head, cap, 0, n - 1)
    want = "%d %d %d %d %s" % (n, m, 0, n - 1, hashlib.sha256(
        expect.off.tobytes() + expect.dst.tobytes() + expect.cap.tobytes()).hexdigest())
    grouped = np.argsort(tail, kind="stable")
    for name, order in (("shuffled", np.arange(m)), ("grouped", grouped)):
        lines = ["c generated", f"p max {n} {m}", "n 1 s", f"n {n} t"]
        for k, i in enumerate(order):
            lines.append(f"a {tail[i] + 1} {head[i] + 1} {cap[i]}" + (" trailing" if k % 211 == 0 else ""))
            if k % 97 == 0:
                lines.append("c a comment")
            if k % 131 == 0:
                lines.append("   ")
            if k % 173 == 0:
                lines.append("")
        for eol in ("\n", "\r\n"):
            p = str(tmp_path / f"{name}{len(eol)}.dimacs")
            with open(p, "wb") as f:
                f.write((eol.join(lines) + eol).encode())
            code = ("import sys, hashlib; sys.path.insert(0, %r); import wbpr_gb300 as W; g = W.read_dimacs(%r);"
                    "print(g.n, g.m, g.s, g.t, hashlib.sha256(g.off.tobytes() + g.dst.tobytes() + g.cap.tobytes())"
                    ".hexdigest())" % (ROOT, p))
            for threads in ("1", "7"):
                got = subprocess.run(["python3", "-c", code], env=dict(os.environ, WBPR_HOST_THREADS=threads),
                                     capture_output=True, text=True, check=True).stdout.strip()
                assert got == want, (name, repr(eol), threads)


def test_snap_reader_pieces_headers_and_page_sized_files(tmp_path):
    """SNAP text in any line order, LF or CRLF, 1 or 7 threads: rows come out
    sorted by head; the last "# Nodes: N Edges: M" header counts wherever it
    stands, other '#' lines are comments; without a header n is the largest
    id + 1.  A file of exactly 8192 bytes ending in a comment reads too (the
    header search never leaves its own line)."""
    import hashlib
    rng = np.random.default_rng(5)
    n, m = 400, 5000
    tail = rng.integers(0, n - 30, m)
    head = rng.integers(0, n - 30, m)
    g = W.Graph.from_arcs(n, tail, head, np.ones(m, np.int32), 0, n - 1)
    dst = g.dst.copy()
    for u in range(n):
        dst[g.off[u]:g.off[u + 1]].sort()

    def digest(n_, off, d):
        return "%d %d %s" % (n_, len(d), hashlib.sha256(off.tobytes() + d.tobytes()).hexdigest())

    want = digest(n, g.off, dst)
    code = ("import sys, hashlib; sys.path.insert(0, %r); import wbpr_gb300 as W; g = W.read_snap_txt(sys.argv[1]);"
            "assert (g.cap == 1).all();"
            "print(g.n, g.m, hashlib.sha256(g.off.tobytes() + g.dst.tobytes()).hexdigest())" % ROOT)
    for name, order in (("shuffled", rng.permutation(m)), ("grouped", np.argsort(tail, kind="stable"))):
        body = [f"{tail[i]}\t{head[i]}" for i in order]
        body.insert(m // 2, "# FromNodeId\tToNodeId, a comment after the header")
        lines = ["# Directed graph", f"# Nodes: {n + 7} Edges: 1"] + body[:m // 3] + \
                [f"# Nodes: {n} Edges: {m}"] + body[m // 3:]  # the later header counts
        for eol in ("\n", "\r\n"):
            p = str(tmp_path / f"{name}{len(eol)}.txt")
            with open(p, "wb") as f:
                f.write((eol.join(lines) + eol).encode())
            for threads in ("1", "7"):
                got = subprocess.run(["python3", "-c", code, p], env=dict(os.environ, WBPR_HOST_THREADS=threads),
                                     capture_output=True, text=True, check=True).stdout.strip()
                assert got == want, (name, repr(eol), threads)
    # no header: n = largest id + 1; padded to one page size exactly, ending in a comment
    text = "\n".join(f"{tail[i]} {head[i]}" for i in range(50)) + "\n# trailing comment "
    text += "x" * (8192 - len(text))
    p = tmp_path / "page.txt"
    p.write_bytes(text.encode())
    assert os.path.getsize(p) == 8192
    h = W.read_snap_txt(str(p))
    assert h.n == int(max(tail[:50].max(), head[:50].max())) + 1 and h.m == 50


@pytest.mark.parametrize("text,off,dst", [
    ("p max 3 0\nn 1 s\nn 3 t\n", [0, 0, 0, 0], []),                      # no arcs
    ("p max 3 0\r\nn 1 s\r\nn 3 t", [0, 0, 0, 0], []),                     # CRLF, no final newline
    ("p max 3 1\nn 1 s\nn 3 t\na 1 3 5", [0, 1, 1, 1], [2]),               # last arc without newline
    ("p max 3 1\nn 1 s\nn 3 t\n\n   \n\ta 1 3 5\n\n", [0, 1, 1, 1], [2]),  # blank lines, tab-indented arc
])
def test_dimacs_reader_edges(tmp_path, text, off, dst):
    p = tmp_path / "e.dimacs"
    p.write_bytes(text.encode())
    g = W.read_dimacs(str(p))
    assert list(g.off) == off and list(g.dst) == dst and (g.s, g.t) == (0, 2)


def test_snap_reader_edges(tmp_path):
    p = tmp_path / "a.txt"
    p.write_text("# only a comment\n")
    with pytest.raises(W.WbprError) as ei:  # no header and no arc: n would be 0
        W.read_snap_txt(str(p))
    assert ei.value.status == 6
    p.write_text("# Nodes: 4 Edges: 0\n")
    g = W.read_snap_txt(str(p))
    assert g.n == 4 and g.m == 0 and list(g.off) == [0] * 5
    p.write_text("0 1")
    g = W.read_snap_txt(str(p))
    assert g.n == 2 and list(g.off) == [0, 1, 1] and list(g.dst) == [1]


def test_python_structs_match_the_header(tmp_path):
    """The ctypes mirrors of wbpr_tuning, wbpr_result and wbpr_verify_report
    (wbpr_gb300/api.py) have the C header's size and field offsets."""
    import ctypes as C
    from wbpr_gb300 import api
    mirrors = {"wbpr_tuning": api.Tuning, "wbpr_result": api.Result, "wbpr_verify_report": api.VerifyReport}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "wbpr.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            a, b, v = ln.split()
            got[(a, b)] = int(v)
    for cname, py in mirrors.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
