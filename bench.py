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
def _serial_sample(seed: int, scale: int = SAMPLE_SCALE):
    """One bounded CPU sample: the reference's serial solver (oracle port) on a
    small R-MAT (scale 11 by default) with the workload's parameters."""
    import oracle
    import wbpr_gb300 as W

    w = WORKLOAD
    g = W.gen_rmat(scale, w["edge_factor"], w["a"], w["b"], w["c"], w["cap_lo"], w["cap_hi"], seed)
    t0 = time.perf_counter()
    v, st = oracle.serial_maxflow(g.n, g.off, g.dst, g.cap, g.s, g.t)
    dt = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError(f"serial sample status {st}")
    return g.m, dt, v


def cpu_baseline_once(scale: int = SAMPLE_SCALE) -> dict:
    m, dt, _ = _serial_sample(WORKLOAD["seed"], scale)
    return {"value": m / dt / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"R-MAT scale {scale} (n={1 << scale}, m={m}) of the workload's generator, "
                      f"seed {WORKLOAD['seed']}: oracle restatement of maxflow-serial, {dt:.2f} s on 1 core"}


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        def step(k):
            t0 = time.perf_counter()
            outs = pool.starmap(_serial_sample, [(1000 + k * cores + i, args.sample_scale) for i in range(cores)])
            return sum(o[0] for o in outs), time.perf_counter() - t0
        for k in range(args.warmup):
            step(k)
        arcs, secs = 0, 0.0
        for k in range(args.steps):
            a, dt = step(args.warmup + k)
            arcs += a
            secs += dt
    value = arcs / secs / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT samples)",
        "config": {"workload": "rmat22_ef16_cap1-100 (bounded samples: scale-11 instances of the same "
                               "generator, one per host core per step)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} parallel scale-{args.sample_scale} R-MAT instances per step; the "
                                   "reference CPU solver maxflow-serial restated in oracle/oracle.c "
                                   "(reference sources are not on the GPU host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
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
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded R-MAT generator; the paper's SNAP graphs are not available)",
            "config": {"workload": workload, "n": g.n, "m": g.m, "s": g.s, "t": g.t,
                       "layout": args.layout, "algo": args.algo, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (2.1 GB residual graph); no flush"},
            "flow": flow,
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
                         "alg_bytes_per_launch": alg, "launch_ms": launch_ms},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": 3 * args.steps,
        }
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

    seeds = range(args.instances or 20)
    tc, vc, flows = [], [], []
    for sd in seeds:
        g = W.gen_genrmf(8, 16, 1, 10000, sd)
        with W.DeviceGraph(g, "rcsr") as d:
            for _ in range(args.warmup):
                d.solve("tc", g.s, g.t)
            r = [d.solve("tc", g.s, g.t) for _ in range(args.steps)]
            if not d.verify()["ok"] or len({x.flow for x in r}) != 1:
                raise AssertionError("certificate failed")
            tc += [x.solve_ms for x in r]
            flows.append(r[0].flow)
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
          flows_first=flows[:5], verified=True, cpu_baseline=cpu)


def config2(args):
    """Unit-capacity bipartite matching, 2M x 2M, Zipf(2.0) left degrees."""
    import wbpr_gb300 as W

    g = W.gen_bipartite(2000000, 2000000, 2.0, 4096, 1)
    with W.DeviceGraph(g, "bcsr") as d:
        # the library's own tuning search (wbpr_autotune), outside the timing;
        # unit-capacity matching gains from more frequent global relabels
        tu, _ = d.autotune("vc", g.s, g.t)
        kw = {"tile": tu.tile, "gr_alpha": tu.gr_alpha, "heavy_degree": tu.heavy_degree}
        for _ in range(args.warmup):
            d.solve("vc", g.s, g.t, **kw)
        r = [d.solve("vc", g.s, g.t, **kw) for _ in range(args.steps)]
        rep = d.verify()
    if not rep["ok"] or len({x.flow for x in r}) != 1:
        raise AssertionError(f"certificate failed: {rep}")
    ms = statistics.median(x.solve_ms for x in r)
    _line("max-flow MTEPS (bipartite matching, unit capacity)", g.m / ms / 1e3, "MTEPS", True,
          f"bipartite_L2M_R2M_zipf2.0 (n={g.n}, m={g.m})", steps=args.steps, warmup=args.warmup,
          solve_ms=ms, gr_ms=r[-1].gr_ms, rounds=r[-1].rounds, matching=r[0].flow, verified=True,
          tuning=kw)


def _config3_instances(count: int, seed: int = 7):
    import numpy as np
    import wbpr_gb300 as W

    rng = np.random.default_rng(seed)
    aw = np.arange(4, 33)
    aw_p = (1.0 / aw) / (1.0 / aw).sum()  # log-uniform over the integers
    bw = np.arange(4, 65)
    bw_p = (1.0 / bw) / (1.0 / bw).sum()
    out = []
    for i in range(count):
        if i % 2 == 0:
            out.append(W.gen_genrmf(int(rng.choice(aw, p=aw_p)), int(rng.choice(bw, p=bw_p)), 1, 10000, i))
        else:
            out.append(W.gen_layered(int(rng.integers(8, 65)), int(rng.integers(16, 513)), 3, 6, 1, 1000, i))
    return out


def config3(args):
    """4,096 uneven instances in one persistent launch (CUDA graph replay,
    autotuned) against a loop of the plain solver over a sample."""
    import numpy as np
    import wbpr_gb300 as W

    count = args.instances or 4096
    gs = _config3_instances(count)
    with W.Batch(gs) as b:
        best, _ = b.autotune()
        for _ in range(args.warmup):
            b.solve(best)
        runs = [b.solve(best) for _ in range(args.steps)]
        flows = runs[0][0]
        if any(not np.array_equal(f, flows) for f, _ in runs):
            raise AssertionError("batch flows differ between steps")
        ims, rounds = b.instance_stats()
    ms = statistics.median(x[1] for x in runs)
    # the same instances as one disjoint-union graph, all pairs in one solve
    u, src, snk = W.disjoint_union(gs)
    with W.DeviceGraph(u, "bcsr") as du:
        for _ in range(args.warmup):
            du.solve_pairs(src, snk)
        uruns = [du.solve_pairs(src, snk) for _ in range(args.steps)]
    for f, _ in uruns:
        if not np.array_equal(f, flows):
            raise AssertionError("union solve flows differ from the batch")
    ums = statistics.median(r.solve_ms for _, r in uruns)
    idx = np.random.default_rng(1).choice(count, min(count, 96), replace=False)
    lat = []
    for i in idx:
        with W.DeviceGraph(gs[i], "bcsr") as d:
            d.solve("vc", gs[i].s, gs[i].t)
            r = d.solve("vc", gs[i].s, gs[i].t)
            if r.flow != flows[i] or not d.verify()["ok"]:
                raise AssertionError(f"instance {i}: batch {flows[i]} plain {r.flow}")
            lat.append(r.solve_ms)
    loop = len(lat) / sum(lat) * 1e3
    best_ms = min(ms, ums)
    _line("batched max-flow instances/s (exact flows)", count / best_ms * 1e3, "instances/s", True,
          f"{count} instances: half GENRMF a,b log-uniform [4,32]x[4,64], half layered 8-64 x 16-512",
          steps=args.steps, warmup=args.warmup, batch_ms=best_ms,
          modes={"block_per_instance": {"ms": ms, "instances_per_s": count / ms * 1e3},
                 "disjoint_union": {"ms": ums, "instances_per_s": count / ums * 1e3,
                                    "rounds": uruns[-1][1].rounds, "global_relabels": uruns[-1][1].global_relabels}},
          tuning={"tile": best.tile, "block": best.block, "gr_alpha": best.gr_alpha},
          inst_p50_ms=float(np.percentile(ims, 50)), inst_p99_ms=float(np.percentile(ims, 99)),
          looped_plain={"instances_per_s": loop, "sample": len(lat), "p50_ms": float(np.percentile(lat, 50)),
                        "p99_ms": float(np.percentile(lat, 99))},
          speedup_vs_loop=count / best_ms * 1e3 / loop, n_total=int(sum(g.n for g in gs)),
          m_total=int(sum(g.m for g in gs)))


def config4(args):
    """512x512 graph-cut grids: forward solve, then both adjoint sides; the
    cut of each indicator must equal the flow, and a few arcs of the first
    grid are checked against +-1 re-solves."""
    import numpy as np
    import wbpr_gb300 as W

    grids = args.instances or 32
    fwd, adj, flows = [], [], []
    fd_checked = 0
    for sd in range(grids):
        g = W.gen_grid(512, 512, sd)
        with W.DeviceGraph(g, "bcsr") as d:
            for _ in range(args.warmup if sd == 0 else 0):
                d.solve("vc", g.s, g.t)
            r = d.solve("vc", g.s, g.t)
            i0, ms0 = d.mincut_adjoint(0)
            i1, ms1 = d.mincut_adjoint(1)
        cap = g.cap.astype(np.int64)
        if int((i0 * cap).sum()) != r.flow or int((i1 * cap).sum()) != r.flow:
            raise AssertionError("cut != flow")
        fwd.append(r.solve_ms)
        adj.append(ms0 + ms1)
        flows.append(r.flow)
        if sd == 0:
            # +-1 re-solves on one handle: only the capacities change
            rng = np.random.default_rng(0)
            fd = W.DeviceGraph(g, "bcsr")
            for e in rng.choice(g.m, min(g.m, args.fd_arcs), replace=False):
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
    pct = 100.0 * sum(adj) / sum(fwd)
    _line("adjoint ms as % of forward solve (512x512 grids)", pct, "%", False,
          f"{grids} grids 512x512, 4-connected, seeds 0..{grids - 1}", steps=grids, warmup=args.warmup,
          forward_ms_median=statistics.median(fwd), adjoint_ms_median=statistics.median(adj),
          grids_per_s=grids / (sum(fwd) + sum(adj)) * 1e3, fd_arcs_checked=fd_checked,
          flows_first=flows[:3], verified=True)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--layout", choices=["bcsr", "rcsr"], default="bcsr")
    ap.add_argument("--algo", choices=["vc", "tc"], default="vc")
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--gr-alpha", type=float, default=0.0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--heavy-degree", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=2)
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
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.config != 1:
        {0: config0, 2: config2, 3: config3, 4: config4}[args.config](args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
