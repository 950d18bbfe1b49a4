"""Build recipe for the CPU oracle (test infrastructure only).

  oracle/_build/liboracle.so   the C restatement in oracle/oracle.c
  oracle/_ref/maxflow-serial   the reference's own serial solver compiled from
                               its sources where they lie (read-only) under
                               /root/reference/maxflow-serial, when that tree
                               exists.  The reference Makefile names mmio.cpp
                               while the tree ships mmio.c, so the recipe
                               compiles mmio.c as C++ and links the three units
                               directly.  Outputs go only to oracle/_ref/.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
REF_SERIAL = os.path.join(REF_OUT, "maxflow-serial")
REF_SRC = "/root/reference/maxflow-serial"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    with open(src, "rb") as f:
        stamp = hashlib.sha256(f.read() + platform.machine().encode()).hexdigest()
    sfile = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(ORACLE_LIB) and os.path.exists(sfile) and open(sfile).read() == stamp:
        return ORACLE_LIB
    cc = shutil.which("gcc") or "gcc"
    _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-Wall", src, "-o", ORACLE_LIB])
    with open(sfile, "w") as f:
        f.write(stamp)
    return ORACLE_LIB


def build_ref(force: bool = False) -> str | None:
    """Compile the reference maxflow-serial; None when its sources are absent."""
    if not os.path.isdir(REF_SRC):
        return None
    if os.path.exists(REF_SERIAL) and not force:
        return REF_SERIAL
    os.makedirs(REF_OUT, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    obj = os.path.join(REF_OUT, "mmio_cpp.o")
    _run([cxx, "-O3", "-std=c++11", "-x", "c++", "-c", os.path.join(REF_SRC, "mmio.c"), "-o", obj])
    _run([cxx, "-O3", "-std=c++11", "-o", REF_SERIAL, os.path.join(REF_SRC, "main.cpp"),
          os.path.join(REF_SRC, "graph.cpp"), obj])
    return REF_SERIAL


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_ref(force)


if __name__ == "__main__":
    build_all(force=True)
    print(ORACLE_LIB, REF_SERIAL if os.path.exists(REF_SERIAL) else "(reference sources absent)")
