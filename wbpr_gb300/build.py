"""Build libwbpr.so and the `maxflow` CLI in-tree (wbpr_gb300/_build/).

CUDA sources are compiled for sm_103a only; translation units compile in
parallel.  A stamp (hash of sources, flags and host machine) skips rebuilds;
a missing output always forces one, so a copy of the tree taken to another
host architecture rebuilds there.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwbpr.so")
LIB_CHECKED = os.path.join(OUT, "libwbpr_checked.so")
CHECKED_SOURCES = ["pr_bcsr.cu", "pr_rcsr.cu"]  # the solver kernels
CLI = os.path.join(OUT, "maxflow")

ARCH = ["-gencode=arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["pr_bcsr.cu", "pr_rcsr.cu", "graph_dev.cu", "noalloc.cu", "batch.cu", "match.cu"]
CPP_SOURCES = ["host_graph.cpp"]
HEADERS = ["pr_kernel.cuh", "pr_launch.h", "wbpr_internal.h", "match.h"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
             "-ffp-contract=off", "-pthread"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libwbpr needs the CUDA toolkit to build")


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def _stamp() -> str:
    h = hashlib.sha256()
    for name in CU_SOURCES + CPP_SOURCES + HEADERS + ["maxflow_main.cpp"]:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + f.read())
    with open(os.path.join(INCLUDE, "wbpr.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip() and os.environ.get("WBPR_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout)


def build(force: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile libwbpr.so and the maxflow CLI; return the library path."""
    os.makedirs(OUT, exist_ok=True)
    stamp_file = os.path.join(OUT, "stamp")
    stamp = _stamp()
    if (not force and os.path.exists(LIB) and os.path.exists(CLI) and os.path.exists(stamp_file)
            and open(stamp_file).read() == stamp):
        return LIB
    nvcc, cxx = _nvcc(), _cxx()
    inc = ["-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        extra = ["-Xptxas", "-v"] if ptxas_verbose else []
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, *inc, "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    for src in CPP_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        jobs.append([cxx, *CXX_FLAGS, *inc, "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-pthread", "-ldl"])
    _run([cxx, "-O2", "-std=c++17", "-Wall", *inc, os.path.join(CSRC, "maxflow_main.cpp"),
          "-o", CLI, "-L", OUT, "-lwbpr", "-Wl,-rpath,$ORIGIN"])
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


def build_checked() -> str:
    """libwbpr_checked.so: the solver kernels compiled with bounds-checked
    arc and vertex accessors (-DWBPR_CHECKED), linked with the other objects
    of the normal build.  An out-of-range index is counted instead of used,
    and the solve returns WBPR_ERR_VERIFY.  Built on demand (debugging and
    its GPU test), not by build()."""
    build()
    stamp = _stamp() + "checked"
    stamp_file = os.path.join(OUT, "stamp_checked")
    if os.path.exists(LIB_CHECKED) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
        return LIB_CHECKED
    nvcc = _nvcc()
    inc = ["-I", INCLUDE, "-I", CSRC]
    jobs, objs = [], []
    for src in CU_SOURCES:
        if src in CHECKED_SOURCES:
            obj = os.path.join(OUT, src + ".checked.o")
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-DWBPR_CHECKED", *inc, "-c", os.path.join(CSRC, src),
                         "-o", obj])
        else:
            obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
    objs += [os.path.join(OUT, src + ".o") for src in CPP_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    _run([nvcc, *ARCH, "-shared", "-o", LIB_CHECKED, *objs, "-Xcompiler", "-pthread", "-ldl"])
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB_CHECKED


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
