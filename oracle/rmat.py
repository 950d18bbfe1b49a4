"""numpy restatement of the project's seeded R-MAT generator (wbpr_gen_rmat in
wbpr_gb300/csrc/host_graph.cpp) -- TEST AND BASELINE INFRASTRUCTURE ONLY.

bench.py's reference arm builds its R-MAT samples with this copy, so the
process that times the reference's CPU solver loads none of the project's
compiled code.  A CPU test holds it equal, array for array, to the library's
generator.

The generator: M = 2^scale * edge_factor draws; draw k runs a splitmix64
stream seeded by (seed, 0x4D41, k) and, per level, takes 32 bits and picks
a quadrant by integer thresholds on (a, a+b, a+b+c) * 2^32; the keys
(u << 32 | v) are sorted, self loops and duplicates dropped; arc i of the
sorted list gets capacity lo + mulhi(next, hi - lo + 1) from the stream
(seed, 0xCA9, i).  s is the vertex of largest out-degree, t the vertex other
than s of largest in-degree (lowest ids on ties).
"""
from __future__ import annotations

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z: np.ndarray) -> np.ndarray:
    # splitmix64 finalizer (Steele, Lea, Flood 2014); numpy uint64 wraps mod 2^64
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _stream_init(seed: int, a: int, b: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        s = np.uint64(seed)
        ha = _mix64(np.asarray([np.uint64(a) * GOLD + np.uint64(0x632BE59BD9B4E019)], np.uint64))[0]
        hb = _mix64(b.astype(np.uint64) + np.uint64(0xD1B54A32D192ED03))
        return _mix64(s ^ ha ^ hb)


def _next(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    with np.errstate(over="ignore"):
        x = x + GOLD
        return x, _mix64(x)


def _mulhi(x: np.ndarray, span: int) -> np.ndarray:
    """(x * span) >> 64 for span <= 2^32, in 64-bit pieces."""
    sp = np.uint64(span)
    hi = x >> np.uint64(32)
    lo = x & np.uint64(0xFFFFFFFF)
    with np.errstate(over="ignore"):
        return (hi * sp + ((lo * sp) >> np.uint64(32))) >> np.uint64(32)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             cap_lo: int = 1, cap_hi: int = 100, seed: int = 1):
    """Returns (n, off, dst, cap, s, t) as int32 numpy arrays and ints."""
    n = 1 << scale
    M = n * edge_factor
    TA = np.uint64(int(np.floor(a * 4294967296.0)))
    TB = np.uint64(int(np.floor((a + b) * 4294967296.0)))
    TC = np.uint64(int(np.floor((a + b + c) * 4294967296.0)))
    x = _stream_init(seed, 0x4D41, np.arange(M, dtype=np.uint64))
    u = np.zeros(M, np.uint64)
    v = np.zeros(M, np.uint64)
    w = np.zeros(M, np.uint64)
    for lvl in range(scale):
        if lvl % 2 == 0:
            x, w = _next(x)
            q = w & np.uint64(0xFFFFFFFF)
        else:
            q = w >> np.uint64(32)
        bit = np.uint64(1 << (scale - 1 - lvl))
        u |= np.where(q >= TB, bit, np.uint64(0))
        v |= np.where(((q >= TA) & (q < TB)) | (q >= TC), bit, np.uint64(0))
    keys = np.unique((u << np.uint64(32)) | v)  # sorted, duplicates dropped
    keys = keys[(keys >> np.uint64(32)) != (keys & np.uint64(0xFFFFFFFF))]
    tail = (keys >> np.uint64(32)).astype(np.int64)
    dst = (keys & np.uint64(0xFFFFFFFF)).astype(np.int32)
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, tail + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    xc = _stream_init(seed, 0xCA9, np.arange(len(keys), dtype=np.uint64))
    _, r = _next(xc)
    cap = (cap_lo + _mulhi(r, cap_hi - cap_lo + 1).astype(np.int64)).astype(np.int32)
    outdeg = np.diff(off)
    s = int(np.argmax(outdeg))
    indeg = np.bincount(dst, minlength=n)
    indeg_ex = indeg.astype(np.int64)
    indeg_ex[s] = -1
    t = int(np.argmax(indeg_ex))
    return n, off, dst, cap, s, t
