"""CPU oracle for the push-relabel path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker / baseline.  The product (wbpr_gb300) never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from .build_oracle import ORACLE_LIB, REF_SERIAL, build_oracle

_lib = None
_i32p = C.POINTER(C.c_int32)


def _load():
    global _lib
    if _lib is None:
        build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        lib.oracle_serial_maxflow.restype = C.c_int64
        lib.oracle_serial_maxflow.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32, C.c_int32,
                                              C.c_int64, _i32p]
        lib.oracle_dinic.restype = C.c_int64
        lib.oracle_dinic.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32, C.c_int32]
        lib.oracle_fifo_pr.restype = C.c_int64
        lib.oracle_fifo_pr.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32, C.c_int32]
        lib.oracle_mincut.restype = C.c_int64
        lib.oracle_mincut.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_int8), C.POINTER(C.c_int8)]
        _lib = lib
    return _lib


def _arrs(off, dst, cap):
    off = np.ascontiguousarray(off, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    cap = np.ascontiguousarray(cap if cap is not None else np.ones(len(dst)), dtype=np.int32)
    if len(dst) == 0:  # keep valid pointers
        dst = np.zeros(1, np.int32)
        cap = np.zeros(1, np.int32)
    return off, dst, cap


def _p(a):
    return a.ctypes.data_as(_i32p)


def serial_maxflow(n, off, dst, cap, s, t, max_ops=0):
    """Restatement of the reference maxflow-serial; returns (value, status)
    with status 0 ok, 1 no s-t path (value 0), 2 op budget exhausted."""
    lib = _load()
    off, dst, cap = _arrs(off, dst, cap)
    st = C.c_int32(0)
    v = lib.oracle_serial_maxflow(n, _p(off), _p(dst), _p(cap), s, t, max_ops, C.byref(st))
    return int(v), int(st.value)


def dinic(n, off, dst, cap, s, t):
    lib = _load()
    off, dst, cap = _arrs(off, dst, cap)
    return int(lib.oracle_dinic(n, _p(off), _p(dst), _p(cap), s, t))


def fifo_pr(n, off, dst, cap, s, t):
    lib = _load()
    off, dst, cap = _arrs(off, dst, cap)
    return int(lib.oracle_fifo_pr(n, _p(off), _p(dst), _p(cap), s, t))


def mincut(n, off, dst, cap, s, t):
    """(value, sink_side_indicator, source_side_indicator) per input arc."""
    lib = _load()
    m = int(off[n])
    off, dst, cap = _arrs(off, dst, cap)
    a = np.zeros(max(m, 1), np.int8)
    b = np.zeros(max(m, 1), np.int8)
    v = lib.oracle_mincut(n, _p(off), _p(dst), _p(cap), s, t, a.ctypes.data_as(C.POINTER(C.c_int8)),
                          b.ctypes.data_as(C.POINTER(C.c_int8)))
    return int(v), a[:m], b[:m]


def ref_serial_available() -> bool:
    return os.path.exists(REF_SERIAL)


def run_ref_serial(path: str, file_type: int, s: int | None = None, t: int | None = None,
                   timeout: float = 300.0) -> int | None:
    """Run the reference maxflow-serial binary; parse its "Max flow: X" line.
    Returns None when it printed no value (no s-t path)."""
    cmd = [REF_SERIAL, "-v", str(file_type), "-f", path]
    cmd += ["-s", str(-1 if s is None else s), "-t", str(-1 if t is None else t)]
    if file_type == 2:
        cmd[-4:] = ["-s", "0", "-t", "0"]  # required by its CLI, ignored for DIMACS
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=timeout)
    for line in r.stdout.splitlines():
        if line.startswith("Max flow:"):
            return int(line.split(":")[1])
    return None
