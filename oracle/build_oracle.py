"""Build recipes for the CPU oracle and the reference's own programs (test and
baseline infrastructure only).

  oracle/_build/liboracle.so   the C restatement in oracle/oracle.c
  oracle/_ref/maxflow-serial   the reference's serial solver (maxflow-serial/)
  oracle/_ref/maxflow-cuda     the reference's CUDA solver (maxflow-cuda/),
                               built for sm_103a without its WORKLOAD timers,
                               only on request (build_ref_cuda)

The reference tree is read where it lies ($WBPR_REFERENCE, default
/root/reference) and never written.  Machines that do not have it (the GPU
host) build from a staged copy of the few source files these recipes need,
which stage_reference() keeps under baseline/_ref/src/ -- git-ignored, like
every output here, so no reference source enters the repository's history.
The reference Makefile of maxflow-serial names a mmio.cpp while the tree ships
mmio.c, so the recipe compiles mmio.c as C++ and links the units directly;
-march=native is left out so the same recipe builds on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
REF_SERIAL = os.path.join(REF_OUT, "maxflow-serial")
REF_CUDA = os.path.join(REF_OUT, "maxflow-cuda")
REF_TREE = os.environ.get("WBPR_REFERENCE", "/root/reference")
STAGE = os.path.join(ROOT, "baseline", "_ref", "src")

SERIAL_FILES = ["maxflow-serial/main.cpp", "maxflow-serial/graph.cpp", "maxflow-serial/graph.h",
                "maxflow-serial/mmio.c", "maxflow-serial/mmio.h"]
CUDA_CU = ["main.cu", "io_par.cu", "preflow.cu", "push_relabel.cu", "push_relabel_kernel.cu", "global_relabel.cu"]
CUDA_CPP = ["graph.cpp", "graph_s.cpp"]
CUDA_FILES = ([f"maxflow-cuda/src/{f}" for f in CUDA_CU + CUDA_CPP + ["mmio.c"]] +
              [f"maxflow-cuda/include/{f}" for f in ("graph.h", "mmio.h", "parallel_graph.cuh", "serial_graph.h",
                                                     "utils.cuh")])


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, cwd=cwd)
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


def stage_reference() -> bool:
    """Copy the reference sources the recipes need into baseline/_ref/src
    (when the reference tree is on this machine).  True if a staged copy exists."""
    if os.path.isdir(REF_TREE):
        for rel in SERIAL_FILES + CUDA_FILES:
            src, dst = os.path.join(REF_TREE, rel), os.path.join(STAGE, rel)
            if not os.path.exists(src):
                continue
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            if not os.path.exists(dst) or open(src, "rb").read() != open(dst, "rb").read():
                shutil.copyfile(src, dst)
    return all(os.path.exists(os.path.join(STAGE, rel)) for rel in SERIAL_FILES)


def _src_root() -> str | None:
    if os.path.isdir(os.path.join(REF_TREE, "maxflow-serial")):
        return REF_TREE
    if stage_reference():
        return STAGE
    return None


def _stamp_ok(out: str, stamp: str) -> bool:
    sf = out + ".stamp"
    return os.path.exists(out) and os.path.exists(sf) and open(sf).read() == stamp


def _write_stamp(out: str, stamp: str) -> None:
    with open(out + ".stamp", "w") as f:
        f.write(stamp)


def build_ref(force: bool = False) -> str | None:
    """Compile the reference maxflow-serial; None when its sources are absent."""
    root = _src_root()
    if root is None:
        return None
    src = os.path.join(root, "maxflow-serial")
    stamp = platform.machine() + hashlib.sha256(b"".join(
        open(os.path.join(root, rel), "rb").read() for rel in SERIAL_FILES)).hexdigest()
    if not force and _stamp_ok(REF_SERIAL, stamp):
        return REF_SERIAL
    os.makedirs(REF_OUT, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    obj = os.path.join(REF_OUT, "mmio_cpp.o")
    _run([cxx, "-O3", "-std=c++11", "-x", "c++", "-c", os.path.join(src, "mmio.c"), "-o", obj])
    _run([cxx, "-O3", "-std=c++11", "-o", REF_SERIAL, os.path.join(src, "main.cpp"),
          os.path.join(src, "graph.cpp"), obj])
    _write_stamp(REF_SERIAL, stamp)
    return REF_SERIAL


def build_ref_cuda(force: bool = False) -> str | None:
    """Compile the reference maxflow-cuda for sm_103a (without WORKLOAD, the
    clock64 instrumentation its Makefile turns on); None without sources."""
    root = REF_TREE if os.path.isdir(os.path.join(REF_TREE, "maxflow-cuda")) else None
    if root is None:
        stage_reference()
        root = STAGE if all(os.path.exists(os.path.join(STAGE, r)) for r in CUDA_FILES) else None
    if root is None:
        return None
    stamp = platform.machine() + hashlib.sha256(b"".join(
        open(os.path.join(root, rel), "rb").read() for rel in CUDA_FILES)).hexdigest()
    if not force and _stamp_ok(REF_CUDA, stamp):
        return REF_CUDA
    nvcc = os.environ.get("NVCC") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc")
                                      else shutil.which("nvcc"))
    if not nvcc:
        return None
    cxx = shutil.which("g++") or "g++"
    src = os.path.join(root, "maxflow-cuda", "src")
    obj_dir = os.path.join(REF_OUT, "maxflow-cuda.obj")
    os.makedirs(obj_dir, exist_ok=True)
    jobs, objs = [], []
    for f in CUDA_CU:
        o = os.path.join(obj_dir, f + ".o")
        jobs.append([nvcc, "-O3", "-gencode=arch=compute_103a,code=sm_103a", "-c", os.path.join(src, f), "-o", o])
        objs.append(o)
    for f in CUDA_CPP + ["mmio.c"]:
        o = os.path.join(obj_dir, f + ".o")
        jobs.append([cxx, "-O3", "-c", os.path.join(src, f), "-o", o])
        objs.append(o)
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    _run([nvcc, "-O3", "-gencode=arch=compute_103a,code=sm_103a", *objs, "-o", REF_CUDA])
    _write_stamp(REF_CUDA, stamp)
    return REF_CUDA


def build_all(force: bool = False) -> None:
    stage_reference()  # keeps the staged copy current for machines without the tree
    build_oracle(force)
    build_ref(force)


if __name__ == "__main__":
    build_all(force=True)
    print(ORACLE_LIB, REF_SERIAL if os.path.exists(REF_SERIAL) else "(reference sources absent)")
