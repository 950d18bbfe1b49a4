#!/usr/bin/env python3
"""Benchmark: exact maximum flow on the scale-22 R-MAT instance.

Workload (one "step" = one full device solve: residual reset, preflow,
push/relabel rounds and global relabels until the maximum preflow):
  seeded R-MAT, scale 22 (4,194,304 vertices), edge factor 16, quadrant
  probabilities (0.57, 0.19, 0.19, 0.05), self loops and duplicates removed
  (65,244,956 arcs), capacities uniform in [1, 100]; s = max out-degree
  vertex, t = max in-degree vertex.  The residual graph (2.1 GB) is far
  larger than L2, so no flush is needed between steps.

Metric: MTEPS = input arcs / solve time / 1e6 (higher is better), every
step's flow value exact (checked equal across steps and by the device
certificate: conservation, capacities, cut == flow).

  value   whole-job MTEPS with the graph resident in HBM (device time)
  e2e     MTEPS through the public C ABI from pinned host buffers: graph
          create (host->device copy of the input CSR, residual graph built on
          the device), solve, read-back, destroy
  roofline  algorithmic bytes of the persistent solver kernel per launch /
          its CUDA-event time, against the measured HBM copy bandwidth
  cpu_baseline  the oracle's restatement of the reference CPU solver
          (maxflow-serial) on a bounded scale-11 sample of the same workload

`--impl reference` times the reference's CPU implementation of the path
(the same restatement; the reference sources do not travel to the GPU host)
on bounded samples using every host core.

Multi-GPU: replicas only -- each rank solves its own copy (no collective on
the data path); value sums the ranks' arcs over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(scale=22, edge_factor=16, a=0.57, b=0.19, c=0.19, cap_lo=1, cap_hi=100, seed=1)
SAMPLE_SCALE = 11  # bounded CPU sample: ~8 s of serial push-relabel on one core
METRIC = "max-flow MTEPS (input arcs / solve time, exact flow)"
UNIT = "MTEPS"
FALLBACK_HBM_GBS = 6800.0


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Dist:
    """Barrier and max-reduction across torchrun ranks (gloo on the host)."""

    def __init__(self, world: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.gpu), "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the solver kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "pr_persistent_rmat22_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
# CPU baselines.  The samples come from oracle.rmat, a numpy restatement of
# the project's R-MAT generator, so these processes load none of the
# project's compiled code; the solver is the reference's own maxflow-serial
# (built from its sources by oracle/build_oracle.py) when it is available,
# else the oracle's restatement of it.
def _write_dimacs_sample(path, n, off, dst, cap, s, t):
    import numpy as np

    tail = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    with open(path, "w") as f:
        f.write(f"p max {n} {len(dst)}\nn {s + 1} s\nn {t + 1} t\n")
        f.write("".join(f"a {u + 1} {v + 1} {c}\n" for u, v, c in zip(tail.tolist(), dst.tolist(), cap.tolist())))


def _serial_sample(seed: int, scale: int = SAMPLE_SCALE, use_ref: bool = True):
    """One bounded CPU sample: maxflow-serial on a small R-MAT (scale 11 by
    default) with the workload's parameters.  Returns (arcs, solve seconds,
    flow, kind); only the solve is timed (the reference binary's time also
    covers its read of the ~0.4 MB sample file, a few milliseconds)."""
    import oracle
    from oracle import rmat

    w = WORKLOAD
    n, off, dst, cap, s, t = rmat.gen_rmat(scale, w["edge_factor"], w["a"], w["b"], w["c"], w["cap_lo"],
                                            w["cap_hi"], seed)
    if use_ref and oracle.ref_serial_available():
        fd, path = tempfile.mkstemp(suffix=".dimacs")
        os.close(fd)
        try:
            _write_dimacs_sample(path, n, off, dst, cap, s, t)
            t0 = time.perf_counter()
            v = oracle.run_ref_serial(path, 2, timeout=600)
            dt = time.perf_counter() - t0
        finally:
            os.unlink(path)
        if v is None:
            raise RuntimeError("reference maxflow-serial printed no flow")
        return len(dst), dt, v, "reference"
    t0 = time.perf_counter()
    v, st = oracle.serial_maxflow(n, off, dst, cap, s, t)
    dt = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError(f"serial sample status {st}")
    return len(dst), dt, v, "port"


def _ref_serial_ready() -> bool:
    """Build the reference maxflow-serial from its staged sources if needed."""
    try:
        from oracle.build_oracle import build_ref

        return build_ref() is not None
    except Exception:  # no compiler or no sources: the oracle port stands in
        return False


SOLVER_TEXT = {"reference": "the reference's maxflow-serial binary (compiled from its sources, g++ -O3)",
               "port": "oracle/oracle.c's restatement of maxflow-serial"}


def cpu_baseline_once(scale: int = SAMPLE_SCALE) -> dict:
    _ref_serial_ready()
    m, dt, _, kind = _serial_sample(WORKLOAD["seed"], scale)
    return {"value": m / dt / 1e6, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"R-MAT scale {scale} (n={1 << scale}, m={m}) of the workload's generator, "
                      f"seed {WORKLOAD['seed']}: {SOLVER_TEXT[kind]}, {dt:.2f} s on 1 core"}


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    _ref_serial_ready()
    ctx = mp.get_context("spawn")
    kinds = set()
    with ctx.Pool(cores) as pool:
        def step(k):
            outs = pool.starmap(_serial_sample, [(1000 + k * cores + i, args.sample_scale) for i in range(cores)])
            kinds.update(o[3] for o in outs)
            # the instances run side by side: a step lasts as long as its slowest
            return sum(o[0] for o in outs), max(o[1] for o in outs)
        for k in range(args.warmup):
            step(k)
        arcs, secs = 0, 0.0
        for k in range(args.steps):
            a, dt = step(args.warmup + k)
            arcs += a
            secs += dt
    kind = "reference" if kinds == {"reference"} else "port"
    value = arcs / secs / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT samples)",
        "config": {"workload": f"rmat22_ef16_cap1-100 (bounded samples: scale-{args.sample_scale} instances of "
                               "the same generator, one per host core per step)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{cores} scale-{args.sample_scale} R-MAT instances per step, side by side, "
                                   f"one per core; {SOLVER_TEXT[kind]}; a step's time is its slowest solve"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _timed_lines(cmd, timeout_s):
    """Run cmd with line-buffered output; return ([(t_seconds, line)], rc,
    timed_out).  On timeout the process is sent SIGTERM, then SIGKILL."""
    import shutil
    import signal
    import threading

    if shutil.which("stdbuf"):
        cmd = ["stdbuf", "-oL", "-eL"] + cmd
    t0 = time.perf_counter()
    p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, errors="replace",
                         start_new_session=True)
    lines = []

    def pump():
        for ln in p.stdout:
            lines.append((time.perf_counter() - t0, ln.rstrip("\n")))

    th = threading.Thread(target=pump, daemon=True)
    th.start()
    timed_out = False
    try:
        rc = p.wait(timeout=timeout_s)
    except subprocess.TimeoutExpired:
        timed_out = True
        os.killpg(p.pid, signal.SIGTERM)
        try:
            rc = p.wait(timeout=30)
        except subprocess.TimeoutExpired:
            os.killpg(p.pid, signal.SIGKILL)
            rc = p.wait()
    th.join(timeout=30)
    return lines, rc, timed_out


def _ref_cuda_once(binary, path, algo, m, timeout_s):
    """One run of the reference maxflow-cuda on a DIMACS file: its solve wall
    time (from "Starting preflow", after its reader and residual builder, to
    its "Total kernel time" line: host preflow, device copies, every
    cooperative launch, host global relabels), its own kernel-only total, the
    flow it prints, and the reader + builder time before it."""
    lines, rc, to = _timed_lines([binary, "-v", "2", "-f", path, "-a", str(algo)], timeout_s)
    t_pre = next((t for t, ln in lines if ln.startswith("Starting preflow")), None)
    t_end = next((t for t, ln in lines if ln.startswith("Total kernel time")), None)
    kern = next((float(ln.split(":")[1].split()[0]) for _, ln in lines if ln.startswith("Total kernel time")), None)
    flow = next((int(ln.rsplit("is", 1)[1].split(",")[0]) for _, ln in lines
                 if ln.startswith("The maximum flow value")), None)
    iters = sum(1 for _, ln in lines if ln.startswith("Invoking kernel"))
    out = {"rc": rc, "timed_out": to, "flow": flow, "kernel_ms": kern, "host_iterations": iters,
           "build_s": t_pre, "solve_s": (t_end - t_pre) if (t_pre is not None and t_end is not None) else None,
           "wall_s": lines[-1][0] if lines else None}
    if out["solve_s"]:
        out["mteps"] = m / out["solve_s"] / 1e6
    if kern:
        out["kernel_mteps"] = m / (kern * 1e-3) / 1e6
    if rc != 0 and not to:
        out["tail"] = [ln for _, ln in lines[-5:]]
    return out


def run_reference_cuda(args) -> None:
    """The reference's own CUDA build (maxflow-cuda, RCSR, compiled from its
    sources for sm_103a without its WORKLOAD timers) on the same workloads:
    config 0 (GENRMF 8x16, -a 0 and -a 1) or config 1 (the R-MAT, -a 1), each
    run capped at --ref-timeout seconds.  Not part of the default run."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from oracle.build_oracle import build_ref_cuda

    t0 = time.perf_counter()
    binary = build_ref_cuda()
    build_s = time.perf_counter() - t0
    if binary is None:
        print(json.dumps({"impl": "reference-cuda", "unavailable": "reference maxflow-cuda sources not staged "
                          "(baseline/_ref/src) and no reference tree"}), flush=True)
        return
    import wbpr_gb300 as W
    from wbpr_gb300 import workloads as WL

    tmp = tempfile.mkdtemp(prefix="wbpr_ref_")
    runs = []
    if args.config == 0:
        seeds = range(args.instances or 5)
        for sd in seeds:
            g = WL.config0(sd)
            path = os.path.join(tmp, f"genrmf_{sd}.dimacs")
            W.write_dimacs(path, g)
            for algo in (0, 1):
                r = _ref_cuda_once(binary, path, algo, g.m, args.ref_timeout)
                r.update(seed=sd, algo=algo, m=g.m)
                runs.append(r)
            os.unlink(path)
        workload = f"genrmf_a8_b16_cap1-10000 seeds 0..{len(seeds) - 1}"
    else:
        g = WL.config1(args.scale)
        path = os.path.join(tmp, f"rmat{args.scale}.dimacs")
        W.write_dimacs(path, g)
        r = _ref_cuda_once(binary, path, 1, g.m, args.ref_timeout)
        r.update(algo=1, m=g.m)
        runs.append(r)
        os.unlink(path)
        workload = f"rmat{args.scale}_ef16_cap1-100"
    os.rmdir(tmp)
    done = [r for r in runs if r.get("solve_s")]
    line = {"impl": "reference-cuda", "metric": METRIC, "unit": UNIT, "higher_is_better": True,
            "value": statistics.median(r["mteps"] for r in done) if done else None,
            "config": {"workload": workload, "layout": "rcsr", "timeout_s": args.ref_timeout},
            "binary": "maxflow-cuda (reference sources, nvcc -O3 sm_103a, WORKLOAD off)", "build_s": build_s,
            "runs": runs}
    print(json.dumps(line), flush=True)


def pinned_copy(g):
    """The graph's arrays copied into page-locked host memory (torch's pinned
    allocator); the graph itself when pinning is unavailable."""
    try:
        import numpy as np
        import torch

        import wbpr_gb300 as W

        def pin(a):
            t = torch.empty(a.size, dtype=torch.int32, pin_memory=True)
            out = t.numpy()
            out[:] = a
            return out, t

        (off, t0), (dst, t1), (cap, t2) = pin(g.off), pin(g.dst), pin(g.cap)
        gp = W.Graph(g.n, off, dst, cap, g.s, g.t)
        gp._pinned = (t0, t1, t2)  # keeps the page-locked buffers alive
        assert np.array_equal(gp.dst, g.dst)
        return gp
    except Exception:  # no torch, or no page-locked memory to be had
        return g


def run_ours(args) -> None:
    rank, world, local = dist_env()
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import wbpr_gb300 as W

    d = Dist(world)
    if W.device_count() < 1:
        raise RuntimeError("bench needs a CUDA device")
    w = dict(WORKLOAD, scale=args.scale)
    t0 = time.perf_counter()
    g = W.gen_rmat(w["scale"], w["edge_factor"], w["a"], w["b"], w["c"], w["cap_lo"], w["cap_hi"], w["seed"])
    gen_s = time.perf_counter() - t0
    tuning = dict(tile=args.tile, gr_alpha=args.gr_alpha, blocks_per_sm=args.blocks_per_sm,
                  heavy_degree=args.heavy_degree)
    dg = W.DeviceGraph(g, args.layout)
    for _ in range(args.warmup):
        dg.solve(args.algo, g.s, g.t, **tuning)
    d.barrier()
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0])
                          if world > 1 else 0)
    clocks.start()
    wall0 = time.perf_counter()
    res = [dg.solve(args.algo, g.s, g.t, **tuning) for _ in range(args.steps)]
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    d.barrier()
    flows = {r.flow for r in res}
    if len(flows) != 1:
        raise AssertionError(f"flow differs between steps: {flows}")
    flow = flows.pop()
    pin = load_pins().get("config1", {})
    pinned = args.scale == 22 and "flow" in pin
    if pinned and flow != pin["flow"]:
        raise AssertionError(f"flow {flow} != the oracle's pinned value {pin['flow']}")
    dev_s = sum(r.solve_ms for r in res) / 1e3
    dev_s_max = d.max(dev_s)
    value = world * args.steps * g.m / dev_s_max / 1e6
    rep = dg.verify()
    if not rep["ok"]:
        raise AssertionError(f"device certificate failed: {rep}")
    launch_ms = statistics.mean(r.launch_ms for r in res)
    alg = statistics.mean(r.alg_bytes for r in res)
    peak, peak_kind = hbm_peak()
    achieved = alg / (launch_ms * 1e-3) / 1e9
    prof = profile_traffic()
    traffic = prof.get("dram_bytes_per_launch") if prof else None
    # the input CSR crosses once (offsets, heads, capacities); either layout is built in HBM
    h2d = 8 * g.m + 4 * (g.n + 1)
    dg.close()
    # e2e through the C ABI from host buffers: the input CSR sits in pinned
    # host memory (set up once, outside the timed region); every step copies
    # it to the device, builds the residual graph there, solves, reads back.
    # One untimed step first, like the warm-up of the device-timed steps.
    e2e_steps = min(args.steps, args.e2e_steps)
    gp = pinned_copy(g)
    if e2e_steps > 0:
        with W.DeviceGraph(gp, args.layout) as dd:
            dd.solve(args.algo, g.s, g.t, **tuning)
    e2e_s = create_s = 0.0
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        with W.DeviceGraph(gp, args.layout) as dd:
            create_s += time.perf_counter() - t1
            r = dd.solve(args.algo, g.s, g.t, **tuning)
        e2e_s += time.perf_counter() - t1
        if r.flow != flow:
            raise AssertionError("e2e flow differs")
    e2e_s = d.max(e2e_s)
    e2e = None
    if e2e_steps > 0:
        e2e = {"value": world * e2e_steps * g.m / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 8 + 128, "steps": e2e_steps, "warmup": 1,
               "create_ms": create_s * 1e3 / e2e_steps, "ms_per_step": e2e_s * 1e3 / e2e_steps,
               "pinned": gp is not g,
               "path": "wbpr_graph_create (H2D of the input CSR from pinned host memory, residual graph "
                       "built on the device) + wbpr_solve + result read-back + wbpr_graph_destroy"}
    if rank == 0:
        cpu = cpu_baseline_once(args.sample_scale) if world == 1 and not args.no_cpu_baseline else None
        workload = "rmat22_ef16_cap1-100" if args.scale == 22 else f"rmat{args.scale}_ef16_cap1-100 (profiling size)"
        last = res[-1]
        # algorithmic bytes and device time of the launch's phases (last step)
        def ph(b, ms):
            return {"gb": b / 1e9, "ms": ms, "gbs": b / 1e9 / max(ms * 1e-3, 1e-12)}
        phases = {"push": ph(last.bytes_push, last.push_ms), "of_which_deep": ph(last.bytes_deep, last.deep_ms),
                  "relabel": ph(last.bytes_relabel, last.kernel_ms - last.push_ms),
                  "global_relabel": ph(last.bytes_gr, last.gr_ms)}
        extras = {}
        if not args.no_extras and world == 1:
            extras["batch"] = batch_record(args.batch_instances, 3, 3)
            extras["adjoint"] = adjoint_record(args.adjoint_grids, 3)
            extras["matching"] = matching_record(5, 3)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded R-MAT generator; the paper's SNAP graphs are not available)",
            "config": {"workload": workload, "n": g.n, "m": g.m, "s": g.s, "t": g.t,
                       "layout": args.layout, "algo": args.algo, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (2.1 GB residual graph); no flush"},
            "flow": flow, "flow_pinned": pinned,
            "solve_ms": {"mean": statistics.mean(r.solve_ms for r in res),
                         "min": min(r.solve_ms for r in res), "max": max(r.solve_ms for r in res)},
            "gr_ms": last.gr_ms, "gr_share": last.gr_ms / max(last.solve_ms, 1e-9), "rounds_ms": last.kernel_ms,
            "rounds": last.rounds,
            "global_relabels": last.global_relabels, "arcs_scanned": last.arcs_scanned,
            "pushes": last.pushes, "relabels": last.relabels, "stranded": last.stranded,
            "verified": True, "wall_s": wall, "gen_s": gen_s,
            "roofline": {"bound": "hbm", "kernel": "pr_persistent", "achieved": achieved, "peak": peak,
                         "peak_kind": f"{peak_kind} (copy bandwidth)", "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "alg_bytes_per_launch": alg, "launch_ms": launch_ms,
                         "definition": "achieved = algorithmic bytes of the pr_persistent launch (wbpr_result."
                                       "alg_bytes) / its CUDA-event time (launch_ms); frac = achieved / peak"},
            "phases": phases,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": 3 * args.steps,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    d.close()


# ---------------------------------------------------------------------------
# The other workloads (one JSON line each; `--config N`).  The default run is
# the R-MAT line above; these are measured on request.
def _line(metric, value, unit, hib, workload, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": hib,
         "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators)",
         "config": {"workload": workload}}
    d.update(extra)
    print(json.dumps(d), flush=True)


def _serial_ms(g) -> float:
    import oracle

    t0 = time.perf_counter()
    v, st = oracle.serial_maxflow(g.n, g.off, g.dst, g.cap, g.s, g.t)
    if st != 0:
        raise RuntimeError(f"serial status {st}")
    return (time.perf_counter() - t0) * 1e3, v


def config0(args):
    """GENRMF a=8, b=16 (1,024 vertices, 4,544 arcs), seeds 0..K-1: TC over
    RCSR (and VC beside it); each solve's certificate checked on the device."""
    import wbpr_gb300 as W

    from wbpr_gb300 import workloads as WL

    seeds = range(args.instances or 20)
    pin = load_pins().get("config0", {}).get("flows", [])
    tc, vc, flows = [], [], []
    for sd in seeds:
        g = WL.config0(sd)
        with W.DeviceGraph(g, "rcsr") as d:
            for _ in range(args.warmup):
                d.solve("tc", g.s, g.t)
            r = [d.solve("tc", g.s, g.t) for _ in range(args.steps)]
            if not d.verify()["ok"] or len({x.flow for x in r}) != 1:
                raise AssertionError("certificate failed")
            tc += [x.solve_ms for x in r]
            flows.append(r[0].flow)
            if sd < len(pin) and flows[-1] != pin[sd]:
                raise AssertionError(f"seed {sd}: flow {flows[-1]} != oracle {pin[sd]}")
            r = [d.solve("vc", g.s, g.t) for _ in range(args.steps)]
            if {x.flow for x in r} != {flows[-1]}:
                raise AssertionError("tc/vc differ")
            vc += [x.solve_ms for x in r]
    cpu = None
    if not args.no_cpu_baseline:
        ms, v = _serial_ms(W.gen_genrmf(8, 16, 1, 10000, 0))
        if v != flows[0]:
            raise AssertionError("serial flow differs")
        cpu = {"value": ms, "unit": "ms", "cores": 1, "kind": "port",
               "sample": "seed 0 instance: oracle restatement of maxflow-serial"}
    _line("max-flow solve ms (GENRMF 8x16, TC over RCSR)", statistics.median(tc), "ms", False,
          f"genrmf_a8_b16_cap1-10000 seeds 0..{len(seeds) - 1}", steps=args.steps, warmup=args.warmup,
          vc_ms_median=statistics.median(vc), tc_ms_p90=sorted(tc)[int(0.9 * (len(tc) - 1))],
          flows_first=flows[:5], flows_pinned=len(pin) >= len(seeds), verified=True, cpu_baseline=cpu)


def matching_record(steps: int, warmup: int, general_steps: int = 3) -> dict:
    """Config 2: the 2M x 2M unit-capacity matching, solved through
    wbpr_solve (which takes the matching kernel for this shape), against the
    general solver on the same handle (matching=-1, autotuned); the matching
    size checked against the oracle's pin and the device certificate."""
    import wbpr_gb300 as W

    from wbpr_gb300 import workloads as WL

    g = WL.config2()
    pin = load_pins().get("config2", {}).get("flow")
    with W.DeviceGraph(g, "bcsr") as d:
        for _ in range(warmup):
            d.solve("vc", g.s, g.t)
        r = [d.solve("vc", g.s, g.t) for _ in range(steps)]
        rep = d.verify()
        gen = [d.solve("vc", g.s, g.t, matching=-1, gr_alpha=0.5, bfs_alpha=4, gr_plateau=4)
               for _ in range(general_steps + 1)][1:]
    if not rep["ok"] or rep["label_violations"] or len({x.flow for x in r + gen}) != 1:
        raise AssertionError(f"certificate failed: {rep}")
    if pin is not None and r[0].flow != pin:
        raise AssertionError(f"matching {r[0].flow} != oracle {pin}")
    ms = statistics.median(x.solve_ms for x in r)
    gms = statistics.median(x.solve_ms for x in gen)
    last = r[-1]
    return {"workload": f"bipartite_L2M_R2M_zipf2.0 (n={g.n}, m={g.m})", "kernel": "pr_match",
            "path": "matching" if last.matching else "general", "solve_ms": ms, "value": g.m / ms / 1e3,
            "unit": "MTEPS", "launch_ms": last.launch_ms, "rounds": last.rounds,
            "global_relabels": last.global_relabels, "gr_ms": last.gr_ms, "matching": r[0].flow,
            "alg_bytes_per_launch": last.alg_bytes, "achieved_gbs": last.alg_bytes / 1e9 / (last.launch_ms * 1e-3),
            "matching_pinned": pin is not None, "verified": True, "general_solver_ms": gms,
            "speedup_vs_general": gms / ms, "steps": steps}


def config2(args):
    """Unit-capacity bipartite matching, 2M x 2M, Zipf(2.0) left degrees."""
    rec = matching_record(args.steps, args.warmup)
    _line("max-flow MTEPS (bipartite matching, unit capacity)", rec["value"], "MTEPS", True, rec["workload"],
          steps=args.steps, warmup=args.warmup, solve_ms=rec["solve_ms"], gr_ms=rec["gr_ms"], rounds=rec["rounds"],
          matching=rec["matching"], matching_pinned=rec["matching_pinned"], verified=True, path=rec["path"],
          general_solver_ms=rec["general_solver_ms"], speedup_vs_general=rec["speedup_vs_general"])


def load_pins() -> dict:
    """Exact maximum-flow values of the workloads at full size, from the CPU
    oracle (tests/golden/make_fullsize.py); {} when the file is absent."""
    p = os.path.join(ROOT, "tests", "golden", "fullsize.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def batch_record(count: int, steps: int, warmup: int, loop_sample: int = 96, union: bool = False) -> dict:
    """Config 3: `count` uneven instances in one persistent launch (CUDA graph
    replay, tuning from wbpr_batch_autotune), every flow checked against the
    oracle's pinned values, against a loop of the plain single-instance
    solver over a seeded sample of the same instances."""
    import numpy as np
    import wbpr_gb300 as W
    from wbpr_gb300 import workloads as WL

    gs = WL.config3(count)
    pin = load_pins().get("config3", {}).get("flows")
    with W.Batch(gs) as b:
        best, _ = b.autotune()
        for _ in range(warmup):
            b.solve(best)
        runs = [b.solve(best) for _ in range(steps)]
        flows = runs[0][0]
        if any(not np.array_equal(f, flows) for f, _ in runs):
            raise AssertionError("batch flows differ between steps")
        ims, _rounds = b.instance_stats()
    pinned = pin is not None and len(pin) >= count
    if pinned and not np.array_equal(flows, np.asarray(pin[:count], np.int64)):
        bad = int(np.flatnonzero(flows != np.asarray(pin[:count]))[0])
        raise AssertionError(f"instance {bad}: batch flow {flows[bad]} != oracle {pin[bad]}")
    ms = statistics.median(x[1] for x in runs)
    rec = {"instances": count, "batch_ms": ms, "instances_per_s": count / ms * 1e3,
           "inst_p50_ms": float(np.percentile(ims, 50)), "inst_p99_ms": float(np.percentile(ims, 99)),
           "tuning": {"tile": best.tile, "block": best.block, "gr_alpha": best.gr_alpha, "batch_cluster": best.batch_cluster},
           "flows_pinned": pinned, "n_total": int(sum(g.n for g in gs)), "m_total": int(sum(g.m for g in gs))}
    if union:
        # the same instances as one disjoint-union graph, all pairs in one solve
        u, src, snk = W.disjoint_union(gs)
        with W.DeviceGraph(u, "bcsr") as du:
            for _ in range(warmup):
                du.solve_pairs(src, snk)
            uruns = [du.solve_pairs(src, snk) for _ in range(steps)]
        for f, _ in uruns:
            if not np.array_equal(f, flows):
                raise AssertionError("union solve flows differ from the batch")
        ums = statistics.median(r.solve_ms for _, r in uruns)
        rec["disjoint_union"] = {"ms": ums, "instances_per_s": count / ums * 1e3, "rounds": uruns[-1][1].rounds,
                                 "global_relabels": uruns[-1][1].global_relabels}
    idx = np.random.default_rng(1).choice(count, min(count, loop_sample), replace=False)
    lat = []
    for i in idx:
        with W.DeviceGraph(gs[i], "bcsr") as d:
            d.solve("vc", gs[i].s, gs[i].t)
            r = d.solve("vc", gs[i].s, gs[i].t)
            if r.flow != flows[i]:
                raise AssertionError(f"instance {i}: batch {flows[i]} plain {r.flow}")
            lat.append(r.solve_ms)
    loop = len(lat) / sum(lat) * 1e3
    rec["looped_plain"] = {"instances_per_s": loop, "sample": len(lat), "p50_ms": float(np.percentile(lat, 50)),
                           "p99_ms": float(np.percentile(lat, 99))}
    rec["speedup_vs_loop"] = rec["instances_per_s"] / loop
    return rec


def adjoint_record(grids: int, warmup: int, fd_arcs: int = 0) -> dict:
    """Config 4: 512 x 512 grids, forward solve then both adjoint sides; each
    flow checked against the oracle's pinned value and each indicator's cut
    against the flow; `fd_arcs` arcs of the first grid checked by +-1
    finite-difference re-solves."""
    import numpy as np
    import wbpr_gb300 as W
    from wbpr_gb300 import workloads as WL

    pin = load_pins().get("config4", {}).get("flows")
    fwd, adj, flows = [], [], []
    fd_checked = 0
    for sd in range(grids):
        g = WL.config4(sd)
        with W.DeviceGraph(g, "bcsr") as d:
            for _ in range(warmup if sd == 0 else 0):
                d.solve("vc", g.s, g.t)
            r = d.solve("vc", g.s, g.t)
            i0, ms0 = d.mincut_adjoint(0)
            i1, ms1 = d.mincut_adjoint(1)
        if pin is not None and sd < len(pin) and r.flow != pin[sd]:
            raise AssertionError(f"grid {sd}: flow {r.flow} != oracle {pin[sd]}")
        cap = g.cap.astype(np.int64)
        if int((i0 * cap).sum()) != r.flow or int((i1 * cap).sum()) != r.flow:
            raise AssertionError("cut != flow")
        fwd.append(r.solve_ms)
        adj.append(ms0 + ms1)
        flows.append(r.flow)
        if sd == 0 and fd_arcs:
            # +-1 re-solves on one handle: only the capacities change
            rng = np.random.default_rng(0)
            fd = W.DeviceGraph(g, "bcsr")
            for e in rng.choice(g.m, min(g.m, fd_arcs), replace=False):
                up = g.cap.copy()
                up[e] += 1
                fd.set_capacities(up)
                dp = fd.solve("vc", g.s, g.t).flow - r.flow
                dm = 0
                if g.cap[e] > 0:
                    dn = g.cap.copy()
                    dn[e] -= 1
                    fd.set_capacities(dn)
                    dm = r.flow - fd.solve("vc", g.s, g.t).flow
                for ind in (i0, i1):
                    if not (dp <= ind[e] and (g.cap[e] == 0 or ind[e] <= dm)):
                        raise AssertionError(f"finite difference at arc {e}")
                fd_checked += 1
            fd.close()
    return {"grids": grids, "pct": 100.0 * sum(adj) / sum(fwd), "forward_ms_median": statistics.median(fwd),
            "adjoint_ms_median": statistics.median(adj), "grids_per_s": grids / (sum(fwd) + sum(adj)) * 1e3,
            "fd_arcs_checked": fd_checked, "flows_pinned": pin is not None and grids <= len(pin),
            "flows_first": flows[:3]}


def config3(args):
    """4,096 uneven instances in one persistent launch (CUDA graph replay,
    autotuned) against a loop of the plain solver over a sample.  Under
    torchrun the instances are sharded across the ranks by estimated work
    (wbpr_gb300.shard), one batched launch per rank, and the flows gathered
    on rank 0 over gloo; the total work is fixed, so the scaling is strong."""
    rank, world, local = dist_env()
    count = args.instances or 4096
    if world == 1:
        rec = batch_record(count, args.steps, args.warmup, union=True)
        best_ms = min(rec["batch_ms"], rec["disjoint_union"]["ms"])
        _line("batched max-flow instances/s (exact flows)", count / best_ms * 1e3, "instances/s", True,
              f"{count} instances: half GENRMF a,b log-uniform [4,32]x[4,64], half layered 8-64 x 16-512",
              steps=args.steps, warmup=args.warmup, best_ms=best_ms, **rec)
        return
    if "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    import wbpr_gb300 as W
    from wbpr_gb300 import shard, workloads as WL

    d = Dist(world)
    graphs = WL.config3(count)
    parts = shard.partition([shard.estimated_work(g) for g in graphs], world)
    mine = parts[rank]
    with W.Batch([graphs[i] for i in mine]) as b:
        best, _ = b.autotune()
        for _ in range(args.warmup):
            b.solve(best)
        d.barrier()
        runs = [b.solve(best) for _ in range(args.steps)]
        d.barrier()
    flows = runs[0][0]
    if any(not np.array_equal(f, flows) for f, _ in runs):
        raise AssertionError("batch flows differ between steps")
    ms = d.max(statistics.median(x[1] for x in runs))
    allf = shard.gather_flows(count, mine, flows, rank, world, d.dist)
    if rank == 0:
        pin = load_pins().get("config3", {}).get("flows")
        pinned = pin is not None and len(pin) >= count
        if pinned and not np.array_equal(allf, np.asarray(pin[:count], np.int64)):
            raise AssertionError("sharded batch flows differ from the oracle's")
        line = {"metric": "batched max-flow instances/s (exact flows)", "value": count / ms * 1e3,
                "unit": "instances/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic (seeded generators)",
                "config": {"workload": f"{count} instances: half GENRMF, half layered", "parallelism":
                           f"instances sharded by estimated work over {world} ranks; flows gathered on rank 0"},
                "flows_pinned": pinned, "shard_sizes": [len(p) for p in parts]}
        print(json.dumps(line), flush=True)
    d.close()


def config4(args):
    """512x512 graph-cut grids: forward solve, then both adjoint sides; the
    cut of each indicator must equal the flow, and a few arcs of the first
    grid are checked against +-1 re-solves."""
    rec = adjoint_record(args.instances or 32, args.warmup, args.fd_arcs)
    grids = rec["grids"]
    _line("adjoint ms as % of forward solve (512x512 grids)", rec["pct"], "%", False,
          f"{grids} grids 512x512, 4-connected, seeds 0..{grids - 1}", steps=grids, warmup=args.warmup,
          verified=True, **rec)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference", "reference-cuda"], default="ours")
    ap.add_argument("--layout", choices=["bcsr", "rcsr"], default="bcsr")
    ap.add_argument("--algo", choices=["vc", "tc"], default="vc")
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--gr-alpha", type=float, default=0.0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--heavy-degree", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-extras", action="store_true", help="skip the batch and adjoint sub-records")
    ap.add_argument("--batch-instances", type=int, default=4096, help="instances of the batch sub-record")
    ap.add_argument("--adjoint-grids", type=int, default=4, help="512x512 grids of the adjoint sub-record")
    ap.add_argument("--scale", type=int, default=22, help="R-MAT scale (22 is the benchmark; smaller "
                    "sizes are for profiling captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU sample (profiling)")
    ap.add_argument("--sample-scale", type=int, default=SAMPLE_SCALE,
                    help="R-MAT scale of the CPU samples (the baseline and the reference arm)")
    ap.add_argument("--config", type=int, choices=[0, 1, 2, 3, 4], default=1,
                    help="1: the R-MAT benchmark (default); 0: GENRMF 8x16; 2: bipartite matching; "
                    "3: batched instances; 4: grids with the adjoint")
    ap.add_argument("--instances", type=int, default=0, help="instances/seeds/grids for --config 0/3/4")
    ap.add_argument("--fd-arcs", type=int, default=6, help="--config 4: arcs of the first grid checked by "
                    "+-1 finite-difference re-solves")
    ap.add_argument("--ref-timeout", type=float, default=900.0, help="--impl reference-cuda: seconds per run")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.impl == "reference-cuda":
        run_reference_cuda(args)
    elif args.config != 1:
        {0: config0, 2: config2, 3: config3, 4: config4}[args.config](args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
