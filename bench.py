"""Benchmark of the fv2d residual-and-update step on one GB300.

Workload (default): 2-D Navier-Stokes flow around a circular cylinder (D = 1, centred in a
40 x 20 box) on a ~1M-cell polygonal Voronoi mesh with jittered seeds graded from 0.005 at the
wall to 0.1 far away; Re = 100, Mach 0.2, Pr = 0.72, NO_SLIP_WALL cylinder, FREESTREAM box,
second order with the squeeze limiter, LOCAL time step, FP64 plain path.  The time step runs at
CFL 0.5: the reference scheme itself (checked with the bit-exact oracle) diverges at the cylinder
wall within 5-25 iterations for any CFL from 0.6 to 0.9 on this mesh; the work per iteration does
not depend on the CFL number.
One step = one SSP-RK3 iteration = 3 x num_cells cell-stage updates.  The solve's device arrays
(~1.4 GB) are larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--cells C]
                  [--only fp32|batched|serve|precision] [--no-fp32] [--no-batch] [--no-serve] [--no-cpu]

The JSON line: `value` (device-timed graph replay), `e2e` (the C ABI with page-locked host buffers,
H2D + step + D2H + residual norm each step; `pageable_value` with ordinary arrays), `roofline`
(dominant kernel against the measured HBM peak, plus `fp64_pipe` against the FP64 issue peak: per
kernel, and for the whole graph-replayed iteration in `fp64_pipe.iteration`),
`cpu_baseline` (the oracle port on one host core), and the FP32, c4 batch and c5 serving lines.
`roofline.fp64_pipe_frac` is the FP64 path's binding roof (the whole iteration's FP64-pipe
instructions over the FP64 issue peak); `step_8d_frac` (FP32 lines) is the whole step's algorithmic
bytes by the specification's formula B = N(40.67s+28) + F(9s+8 [+5s NS]) + 4(2F-Nb) per stage over
the measured HBM peak (`_euler_geometry`: without the NS face terms).  The FP32 engine and its
batches run one fused kernel per RK stage (`k_tstage`); the serving sample runs a persistent FP32
batch.
--impl reference times the reference's CPU solver step (the oracle port, a line-by-line
restatement proven bit-identical to the reference) on the host cores: one independent replica of
the same solve per core, a bounded sample of iterations.
Multi-GPU: replicas only (each rank advances its own copy of the solve; no collective on the path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

METRIC = "cell-stage updates/s"
WORKLOAD_CFL = 0.5
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def workload_case(pkg, cells):
    mg = pkg.meshgen
    u = mg.mach_speed(0.2)
    mu = 1.225 * u * 1.0 / 100.0           # Re = rho u D / mu = 100
    case = dict(mg.DEFAULT_CASE, eqn="NS", mu=mu, Pr=0.72, u=u, v=0.0, limiter="SQUEEZE", time_step_type="LOCAL",
                CFL=WORKLOAD_CFL, BC1="NO_SLIP_WALL", BC2="FREESTREAM", solution_poly_order=1)
    return case


def make_grid(pkg, cells, seed=0):
    return pkg.meshgen.voronoi_cylinder(cells, seed=seed)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"fv2d_bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "25"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        lines = open(self.path).read().splitlines()
        try:
            os.remove(self.path)
        except OSError:
            pass
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def bytes_per_launch(kernel, N, F, ninc, Nb, s, ns, squeeze, comp=False, store_r=True, order2=True, fval=False):
    """Algorithmic bytes of one launch (average over the three RK stages): every array element the
    kernel must touch, counted once.  s = state bytes (8 FP64, 4 FP32); ids 4 B; LSQ moments 8 B.
    comp: FP32 delta-form increments and compensated base state; store_r: residual kept (last stage);
    fval: the face pass stores its reconstructed face states and the squeeze reads them (FP64 single
    solve) instead of recomputing them from the previous stage's Q and limited G."""
    if kernel in ("k_gradient", "kb_gradient"):
        if not order2:
            return 0.0
        b = N * (4 * s + 8 * s)                  # Q read, G write
        if squeeze and fval:
            b += ninc * 4 * s                    # stored face state on the cell's side, per incidence
        elif squeeze:
            b += N * (4 * s + 8 * s)             # previous Q and limited G
        b += N * 4 + ninc * 8 + N * 24           # CSR offsets, (face, neighbour) pairs, Ixx/Iyy/Ixy
        b += ninc * 4 * s                        # per-incidence dxj, dyj, face-centre offset
        b += Nb * 2 * s                          # nx, ny on boundary faces
        return b
    if kernel in ("k_face", "kb_face"):
        geo = 7 + (3 if (ns and order2) else 0)  # nx ny area c1dx c1dy c2dx c2dy [+ lx ly dist]
        b = F * (8 + geo * s)                    # c1, c2, geometry
        b += N * (4 * s + (8 * s if order2 else 0))   # Q (and G) of every cell
        b += F * 4 * s                           # t written
        b += (F * s) / 3.0                       # spectral term, last stage only
        if squeeze and fval and order2:
            b += (2 * F - Nb) * 4 * s            # face states stored for the next squeeze
        return b
    if kernel in ("k_update", "kb_update"):
        b = N * 4 + ninc * 4 + F * 4 * s         # CSR, face contributions
        b += N * s                               # volume
        b += N * 4 * s                           # Qn read
        b += N * 4 * s                           # stage result written
        b += N * s                               # dt written (stage 1) or read (stages 2-3)
        b += (F * s + N * s) / 3.0               # spectral sum (last stage)
        if comp:
            b += N * 4 * s * (1 + 2 + 1) / 3.0   # increment D: write, read+write, read
            b += N * 4 * s * 2 / 3.0             # compensation term: read+write on the last stage
        else:
            b += N * 4 * s * 2.0 / 3.0           # Q1 / Q2 read on stages 2-3
        if store_r:
            b += (N * 4 * s) / 3.0               # residual stored on the last stage
        return b
    return 0.0


def bytes_8d(N, F, Nb, s, ns=False, squeeze=True, euler_geometry=False):
    """Algorithmic bytes of one RK stage of one solve by the benchmark specification's formula (a
    two-pass design, every array counted once per stage):
        B = N (40.67 s + 28) + F (g s + 8) + 4 (2F - Nb)
    per cell: stage state read 4s, Qn read on stages 2-3 (8/3)s, state written 4s, gradient written
    and read 16s, previous stage's state and limited gradient for the squeeze limiter 12s, dt s,
    volume s, LSQ moments 24 B (always FP64), CSR offset 4 B; per face: g = 9 geometry values
    (nx ny A d1x d1y d2x d2y dxj dyj) plus 5 for NS (mx my lx ly dist), cell ids 8 B; per incidence:
    the face id 4 B.  euler_geometry: count 9 geometry values for NS meshes too.
    s = state bytes (8 FP64, 4 FP32)."""
    per_cell = (4 + 8.0 / 3.0 + 4 + 16 + (12 if squeeze else 0) + 1 + 1) * s + 24 + 4
    g = 9 + (5 if (ns and not euler_geometry) else 0)
    return N * per_cell + F * (g * s + 8) + 4 * (2 * F - Nb)


def step_8d(solves, ms_per_iteration, peak):
    """Whole-step HBM fraction on the specification's algorithmic bytes: `solves` is a list of
    (N, F, Nb, s, ns, squeeze); one iteration is 3 stages of each.  Reported with the NS geometry term
    (the formula as specified) and with Euler geometry for every solve (the smaller byte count)."""
    out = {}
    for key, eg in (("", False), ("_euler_geometry", True)):
        b = 3.0 * sum(bytes_8d(N, F, Nb, s, ns, sq, euler_geometry=eg) for N, F, Nb, s, ns, sq in solves)
        ach = b / (ms_per_iteration * 1e-3) / 1e9
        cells = sum(x[0] for x in solves)
        out["bytes_per_cell_stage" + key] = round(b / (3.0 * cells), 1)
        out["achieved" + key] = round(ach, 1)
        out["frac" + key] = round(ach / peak, 4)
    return out


def add_step_8d(roof, solves, ms_per_iteration, peak):
    """Put the whole-step fraction on the specification's bytes into a roofline dict as scalars."""
    for k, v in step_8d(solves, ms_per_iteration, peak).items():
        roof["step_8d_" + k] = v


def roofline(kt, kbytes, peak):
    """Dominant kernel (largest total time) of the event-timed pass, its achieved GB/s on the
    algorithmic bytes, and every kernel's share of the stage time."""
    per = {}
    for k, nbytes in kbytes.items():
        ms, launches = kt.get(k, (0.0, 0))
        if launches:
            per[k] = dict(avg_ms=ms / launches, launches=launches, total_ms=ms, bytes=nbytes)
    tot = sum(v["total_ms"] for v in per.values()) or 1.0
    dom = max(per, key=lambda k: per[k]["total_ms"])
    d = per[dom]
    achieved = d["bytes"] / (d["avg_ms"] * 1e-3) / 1e9
    return dom, {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                 "frac": round(achieved / peak, 4), "traffic": None, "kernel": dom,
                 "kernel_avg_ms": round(d["avg_ms"], 4), "bytes_per_launch": int(d["bytes"]),
                 "share": {k: round(v["total_ms"] / tot, 3) for k, v in per.items()}}, per


def ncu_traffic(precision, kernel, N, F):
    """DRAM bytes of one launch of `kernel` from the committed ncu capture, scaled by units."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            t = json.load(fh)[precision][kernel]
        return int(t["bytes"] / t["units"] * (N if t["per"] == "cells" else F))
    except Exception:
        return None


def fp64_pipe(kernels, N, F, sm_mhz):
    """FP64 path: each kernel's FP64 thread-instructions per launch (per-unit count from the
    committed ncu capture x this mesh's units) over its live event-timed launch time, against the
    FP64 issue peak of 2 thread-instructions per SM per cycle at the sampled SM clock."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            t = json.load(fh)["fp64"]
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    except Exception:
        return None
    peak = 2.0 * sms * sm_mhz * 1e6 / 1e9
    out = {}
    for k, v in kernels.items():
        if k not in t or "fp64_inst" not in t[k]:
            continue
        inst = t[k]["fp64_inst"] / t[k]["units"] * (N if t[k]["per"] == "cells" else F)
        ach = inst / (v["avg_ms"] * 1e-3) / 1e9
        out[k] = {"achieved": round(ach, 1), "frac": round(ach / peak, 3), "inst_per_launch": int(inst)}
    if not out:
        return None
    dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
    return {"bound": "fp64_pipe", "kernel": dom, "achieved": out[dom]["achieved"], "peak": round(peak, 1),
            "unit": "G FP64 thread-inst/s", "frac": out[dom]["frac"], "sm_mhz": sm_mhz,
            "per_kernel": out}


def peaks():
    try:
        with open(PEAKS_FILE) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def cpu_baseline(pkg, orc, grid, case, iters, samples):
    """The oracle port on one host core: `samples` timed samples of `iters` iterations each after one
    warm-up iteration; the median sample's rate (the shared host's rate drifts from run to run)."""
    o = orc.Oracle("port", grid=grid, case=case)
    o.iterate(1)                                   # first iteration includes allocation warm-up
    ts = [o.time_iterations(iters) for _ in range(samples)]
    N = grid.num_cells
    rates = [3.0 * N * iters / t for t in ts]
    return statistics.median(rates), sum(ts), [round(r, 1) for r in rates]


def max_over_ranks(x: float, ws: int) -> float:
    """The slowest rank's value (MAX all-reduce over the host process group; identity at N=1)."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


REF_SAMPLE_S = 40.0           # bounded CPU sample per replica (seconds of work, estimated)
REF_CELL_STAGE_PER_S = 1.0e6  # single-core rate of the oracle port (about 1.1e6 measured on the GPU host), for sizing


def reference_iterations(steps: int, cells: int) -> int:
    """Iterations each CPU replica times: `steps`, capped to about REF_SAMPLE_S of work."""
    return max(1, min(steps, int(REF_SAMPLE_S * REF_CELL_STAGE_PER_S / (3.0 * cells))))


def run_reference_arm(args):
    """Oracle port on the host cores: one replica per core, same mesh and options, each timing a
    bounded sample of iterations (reference_iterations)."""
    import multiprocessing as mp

    ws, rank, _ = dist_env()
    if rank != 0:
        return
    pkg = entry.load_package()
    orc = entry.load_oracle()
    orc.build(ref_dir="/nonexistent")
    grid = make_grid(pkg, args.cells)
    case = workload_case(pkg, args.cells)
    cores = args.cpu_cores or os.cpu_count() or 1
    ctx = mp.get_context("fork")       # no CUDA in this process
    q = ctx.Queue()

    iters = reference_iterations(args.steps, grid.num_cells)

    def worker(i):
        o = orc.Oracle("port", grid=grid, case=case)
        o.iterate(args.warmup)             # warm-up iterations (allocation, first touch), untimed
        t = o.time_iterations(iters)
        q.put(t)

    t0 = time.time()
    procs = [ctx.Process(target=worker, args=(i,)) for i in range(cores)]
    for p in procs:
        p.start()
    ts = [q.get() for _ in procs]
    for p in procs:
        p.join()
    wall = time.time() - t0
    N = grid.num_cells
    per_core = [3.0 * N * iters / t for t in ts]
    value = sum(per_core)
    line = {"metric": METRIC, "value": value, "unit": "cell-stage/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * max(ts) / iters,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ns_cylinder_voronoi", "cells": N, "faces": grid.num_faces, "precision": "fp64",
                       "parallelism": f"{cores} independent CPU replicas"},
            "cpu_baseline": {"value": value, "unit": "cell-stage/s", "cores": cores, "kind": "port",
                             "sample": f"{iters} SSP-RK3 iterations of the {N}-cell solve per core "
                                       f"(of {args.steps} steps, capped to ~{REF_SAMPLE_S:.0f} s), after {args.warmup} warm-up iterations",
                             "single_core_value": statistics.median(per_core)},
            "e2e": {"value": value, "unit": "cell-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(wall, 1)}
    print(json.dumps(line), flush=True)


def single_kernel_bytes(N, F, ninc, Nb, s, comp, store_r=True):
    return {k: bytes_per_launch(k, N, F, ninc, Nb, s, True, True, comp=comp, store_r=store_r, fval=(s == 8))
            for k in ("k_gradient", "k_face", "k_update")}


def measure_fp32(pkg, grid, case, args, peak, peak_kind, N, F, ninc, Nb):
    """The same solve through the FP32 path: device-timed throughput and its dominant kernel."""
    import torch
    s = pkg.Solver(grid, case, precision=pkg.FP32)
    st = torch.cuda.ExternalStream(s.stream())
    s.step(args.warmup)
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        s.step(1)
    e1.record(st)
    e1.synchronize()
    s.synchronize()
    ms = e0.elapsed_time(e1)
    s.set_kernel_timing(True)
    s.step(args.steps)
    kt = s.kernel_times()
    s.close()
    # the FP32 engine runs one fused kernel per stage: its algorithmic bytes are the whole stage's
    ns = case["eqn"] == "NS"
    dom, roof, per = roofline(kt, {"k_tstage": bytes_8d(N, F, Nb, 4, ns, case["limiter"] == "SQUEEZE")}, peak)
    roof["peak_source"] = f"{peak_kind} hbm_gbs"
    roof["traffic"] = ncu_traffic("fp32", dom, N, F)
    add_step_8d(roof, [(N, F, Nb, 4, case["eqn"] == "NS", case["limiter"] == "SQUEEZE")], ms / args.steps, peak)
    return {"value": 3.0 * N * args.steps / (ms * 1e-3), "unit": "cell-stage/s", "ms_per_step": ms / args.steps,
            "roofline": roof,
            "kernels": {k: {"avg_ms": round(v["avg_ms"], 4), "gbs": round(v["bytes"] / (v["avg_ms"] * 1e-3) / 1e9, 1)}
                        for k, v in per.items()}}


def measure_batched(pkg, args, peak, peak_kind):
    """c4: 256 independent FP32 solves in one batch, tile shapes autotuned, graph-replayed iterations."""
    import torch
    from fv2d_gb300 import autotune, workloads
    t0 = time.time()
    specs = workloads.c4_specs(args.batch_solves, seed=args.seed)
    grids = workloads.grids_parallel(specs)
    t_gen = time.time() - t0
    tot_c = sum(g.num_cells for g in grids)
    tot_f = sum(g.num_faces for g in grids)
    b = pkg.Batch(tot_c + 16, tot_f + 16, len(grids) + 1, precision=pkg.FP32)
    t0 = time.time()
    for g, sp in zip(grids, specs):
        b.add(g, workloads.spec_case(sp))
    t_add = time.time() - t0
    if args.no_tune:
        b.set_tuning(256, (1, 2, 4), (16384, 131072))
        tuning = {"block": 256, "tile_mult": [1, 2, 4], "bucket_edges": [16384, 131072]}
    else:
        tuning = autotune.tune(b, iters=3, warmup=1)
    st = torch.cuda.ExternalStream(b.stream())
    b.step(args.warmup)
    b.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.step(args.steps)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    b.set_kernel_timing(True)
    b.step(max(3, args.steps // 4))
    kt = b.kernel_times()
    b.set_kernel_timing(False)
    # one fused kernel per stage (k_tstage_1..3), each moving a whole stage's algorithmic bytes
    stage_bytes = sum(bytes_8d(g.num_cells, g.num_faces, int((g.fc2 <= 0).sum()), 4, bool(sp["ns"]), True)
                      for g, sp in zip(grids, specs))
    kbytes = {k: stage_bytes for k in ("k_tstage_1", "k_tstage_2", "k_tstage_3")}
    dom, roof, per = roofline(kt, kbytes, peak)
    roof["peak_source"] = f"{peak_kind} hbm_gbs"
    roof["traffic"] = ncu_traffic("batch_fp32", dom, tot_c, tot_f)
    add_step_8d(roof, [(g.num_cells, g.num_faces, int((g.fc2 <= 0).sum()), 4, bool(sp["ns"]), True)
                       for g, sp in zip(grids, specs)], ms / args.steps, peak)
    norms = b.norms()
    finite = all(np.all(np.isfinite(v[0])) for v in norms.values())
    b.close()
    return {"value": 3.0 * tot_c * args.steps / (ms * 1e-3), "unit": "cell-stage/s", "ms_per_step": ms / args.steps,
            "solves": len(grids), "cells": tot_c, "faces": tot_f, "ns_solves": sum(sp["ns"] for sp in specs),
            "roofline": roof, "tuning": {k: tuning.get(k) for k in ("block", "tile_mult", "bucket_edges", "full_grid")},
            "kernels": {k: {"avg_ms": round(v["avg_ms"], 4), "gbs": round(v["bytes"] / (v["avg_ms"] * 1e-3) / 1e9, 1)}
                        for k, v in per.items()},
            "finite": finite, "mesh_gen_s": round(t_gen, 1), "admit_s": round(t_add, 1),
            "workload": "256 bump-channel Voronoi solves, cells log-uniform 2k-200k, FP32, graph-replayed iterations"}


def measure_serving(pkg, args):
    """c5 sample: a Poisson stream through continuous batching (FP32) for `serve_seconds` and, as the
    baseline, the same stream one request at a time through the plain FP64 path for
    `serve_baseline_seconds` (default: the same)."""
    from fv2d_gb300 import serve, workloads
    t0 = time.time()
    pool = serve.MeshPool(lo=5e3, hi=2e6, n=args.pool_meshes, seed=args.seed)
    pool.prebuild()
    t_pool = time.time() - t0
    stream = workloads.c5_stream(rate=args.serve_rate, duration=args.serve_seconds, seed=args.seed, lo=5e3, hi=2e6)
    budget = args.serve_budget_gb * 1e9
    cells, faces, solves, bound = serve.capacity_from_budget(pool, budget)
    b = pkg.Batch(cells, faces, solves, precision=pkg.FP32)
    b.set_grid_mode(False)   # persistent stage kernels: the autotuner's choice for FP32 batches (c4)
    peak, _ = peaks()

    def stage_bytes(g, spec):
        return bytes_8d(g.num_cells, g.num_faces, int((g.fc2 <= 0).sum()), 4, bool(spec["ns"]), True)

    out = serve.serve(b, stream, pool, duration=args.serve_seconds, target=1e-6, max_iters=args.serve_max_iters,
                      check_every=25, stall_iters=args.serve_stall_iters, stage_bytes=stage_bytes)
    if out.get("bytes_per_s"):
        out["step_8d_achieved"] = round(out["bytes_per_s"] / 1e9, 1)
        out["step_8d_frac"] = round(out["bytes_per_s"] / 1e9 / peak, 4)
    usage = b.usage()
    b.close()
    base_s = args.serve_baseline_seconds if args.serve_baseline_seconds > 0 else args.serve_seconds
    base = serve.serve_one_at_a_time(stream, pool, duration=base_s, precision=pkg.FP64, target=1e-6,
                                     max_iters=args.serve_max_iters, check_every=25, stall_iters=args.serve_stall_iters)
    return {"batched_fp32": out, "baseline_fp64_one_at_a_time": base,
            "stream": {"rate_per_s": args.serve_rate, "seconds": args.serve_seconds, "requests": len(stream),
                       "cells": "log-uniform 5k-2M (snapped to a pool of %d meshes)" % args.pool_meshes},
            "arena": {"budget_gb": args.serve_budget_gb, "cells": cells, "faces": faces, "bytes": usage["bytes"],
                      "bound": bound},
            "pool_gen_s": round(t_pool, 1)}


def measure_precision(pkg, args):
    """c3: FP32 against FP64 (bit-exact) on the 4M-cell Euler bump channel (Mach drawn from the seed,
    squeeze, LOCAL dt), run to a 1e-6 residual drop or an iteration cap: second order with the
    squeeze limiter (which stalls near a 5 % drop, so it runs to the cap) and first order (which
    converges).  Density / pressure L2 and Linf differences and the wall-force difference."""
    from fv2d_gb300 import precision, workloads
    t0 = time.time()
    grid, case, mach = workloads.c3_case(cells=args.prec_cells, seed=args.seed)
    t_mesh = time.time() - t0
    out = {"workload": "c3 bump channel, Euler", "cells": grid.num_cells, "faces": grid.num_faces,
           "mach": round(mach, 4), "seed": args.seed, "mesh_gen_s": round(t_mesh, 1)}
    out["second_order_squeeze"] = precision.compare(grid, case, drop=1e-6, max_iters=args.prec_max_iters,
                                                    check_every=100)
    first = dict(case, solution_poly_order=0, limiter="NONE")
    out["first_order"] = precision.compare(grid, first, drop=1e-6, max_iters=args.prec_max_iters_first,
                                           check_every=1000 if args.prec_max_iters_first > 50000 else 200)
    return out


def run_partial(args):
    """One measurement alone: --only fp32 | batched | serve | precision."""
    import torch
    pkg = entry.load_package()
    pkg.build.build()
    torch.cuda.set_device(0)
    peak, peak_kind = peaks()
    if args.only == "serve":
        out = measure_serving(pkg, args)
    elif args.only == "precision":
        out = measure_precision(pkg, args)
    elif args.only == "fp32":
        grid, case = make_grid(pkg, args.cells), workload_case(pkg, args.cells)
        N, F = grid.num_cells, grid.num_faces
        Nb = int((grid.fc2 <= 0).sum())
        out = measure_fp32(pkg, grid, case, args, peak, peak_kind, N, F, 2 * F - Nb, Nb)
    else:
        out = measure_batched(pkg, args, peak, peak_kind)
    print(json.dumps({"only": args.only, **out}), flush=True)


def run_gpu_arm(args):
    import torch

    ws, rank, local = dist_env()
    pkg = entry.load_package()
    pkg.build.build()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    t_mesh = time.time()
    grid, case = make_grid(pkg, args.cells), workload_case(pkg, args.cells)
    t_mesh = time.time() - t_mesh
    prec = pkg.FP64 if args.precision == "fp64" else pkg.FP32
    N, F = grid.num_cells, grid.num_faces
    Nb = int((grid.fc2 <= 0).sum())
    ninc = 2 * F - Nb
    s_bytes = 8 if prec == pkg.FP64 else 4

    solver = pkg.Solver(grid, case, precision=prec)
    stream = torch.cuda.ExternalStream(solver.stream())
    solver.step(args.warmup)
    solver.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = Clocks(local)
    # ---- device-resident timed region (CUDA graph replay of whole iterations)
    barrier()
    torch.cuda.synchronize()
    solver.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        solver.step(1)
    e1.record(stream)
    e1.synchronize()
    solver.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    barrier()
    ms = max_over_ranks(ms, ws)
    value = ws * 3.0 * N * args.steps / (ms * 1e-3)

    # ---- per-kernel timing pass (events around every launch, eager launches)
    solver.set_kernel_timing(True)
    solver.step(args.steps)
    kt = solver.kernel_times()
    solver.set_kernel_timing(False)
    peak, peak_kind = peaks()
    dom, roof, per = roofline(kt, single_kernel_bytes(N, F, ninc, Nb, s_bytes, prec == pkg.FP32), peak)
    roof["peak_source"] = f"{peak_kind} hbm_gbs"
    roof["traffic"] = ncu_traffic(args.precision, dom, N, F)
    if prec == pkg.FP64:   # this path is bound by the FP64 pipe, not HBM
        fp = fp64_pipe(per, N, F, clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0)
        if fp:
            # the whole step: every stage kernel's FP64 pipe slots per iteration (three launches of
            # each) over the graph-replayed iteration time
            it_inst = 3 * sum(v["inst_per_launch"] for v in fp["per_kernel"].values())
            it_ach = it_inst / (ms / args.steps * 1e-3) / 1e9
            fp["iteration"] = {"inst": it_inst, "ms": round(ms / args.steps, 4), "achieved": round(it_ach, 1),
                               "frac": round(it_ach / fp["peak"], 3)}
            roof["fp64_pipe_iteration_frac"] = fp["iteration"]["frac"]
        roof["fp64_pipe"] = fp
        if fp:
            roof["fp64_pipe_frac"] = fp["frac"]
            roof["fp64_pipe_kernel"] = fp["kernel"]
    add_step_8d(roof, [(N, F, Nb, s_bytes, True, True)], ms / args.steps, peak)
    gpu_launches = 3 * 3 * args.steps

    # ---- end to end through the C ABI with host buffers: upload Qbar, one iteration, download
    # the step's input and output live in page-locked host memory (the library DMAs them directly)
    q = torch.empty(4 * N, dtype=torch.float64, pin_memory=True).numpy()
    solver.get_state(q)
    norm = np.zeros(4)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solver.load_state(q)
        solver.step(1)
        solver.get_state(q)
        norm = solver.residual_norm()
    t_e2e = max_over_ranks(time.perf_counter() - t0, ws)
    # the same with ordinary (pageable) host arrays: staged through the library's pinned buffer
    qp = np.array(q)
    kp = max(3, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(kp):
        solver.load_state(qp)
        solver.step(1)
        solver.get_state(qp)
        norm = solver.residual_norm()
    t_pg = max_over_ranks(time.perf_counter() - t0, ws)
    e2e = {"value": ws * 3.0 * N * args.steps / t_e2e, "unit": "cell-stage/s",
           "h2d_bytes_per_step": 4 * 8 * N, "d2h_bytes_per_step": 4 * 8 * N + 4 * 8, "host_buffers": "pinned",
           "pageable_value": ws * 3.0 * N * kp / t_pg}
    dev_bytes = solver.device_bytes()
    solver.close()

    fp32 = None
    if rank == 0 and prec == pkg.FP64 and not args.no_fp32:
        fp32 = measure_fp32(pkg, grid, case, args, peak, peak_kind, N, F, ninc, Nb)
    batched = None
    if rank == 0 and not args.no_batch:
        batched = measure_batched(pkg, args, peak, peak_kind)
        batched["vs_fp64_plain"] = round(batched["value"] / value * ws, 2)

    serving = None
    if rank == 0 and not args.no_serve:
        serving = measure_serving(pkg, args)

    # ---- CPU baseline (oracle port, 1 core, bounded sample)
    cpu = None
    if rank == 0 and not args.no_cpu:
        orc = entry.load_oracle()
        orc.build(ref_dir="/nonexistent")
        cv, ct, rates = cpu_baseline(pkg, orc, grid, case, args.cpu_iters, args.cpu_samples)
        cpu = {"value": cv, "unit": "cell-stage/s", "cores": 1, "kind": "port",
               "sample": f"median of {args.cpu_samples} samples of {args.cpu_iters} SSP-RK3 iterations of the same "
                         f"{N}-cell solve ({ct:.1f} s in all), after 1 warm-up iteration",
               "samples": rates}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-stage/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if prec == pkg.FP64 else "f32", "data": "synthetic",
                "config": {"workload": "ns_cylinder_voronoi", "cells": N, "faces": F, "boundary_faces": Nb,
                           "max_sides": max(grid.sides_histogram()), "precision": args.precision,
                           "re": 100, "mach": 0.2, "limiter": "SQUEEZE", "dt": "LOCAL", "cfl": WORKLOAD_CFL,
                           "l2": "working set > L2 (no flush)", "parallelism": f"{ws} replicas" if ws > 1 else "single GPU",
                           "mesh_gen_s": round(t_mesh, 1)},
                "clocks": clk, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
                "kernels": {k: {"avg_ms": round(v["avg_ms"], 4), "launches": v["launches"],
                                "bytes_per_launch": int(v["bytes"]),
                                "gbs": round(v["bytes"] / (v["avg_ms"] * 1e-3) / 1e9, 1)} for k, v in per.items()},
                "fp32": fp32, "batched": batched, "serving": serving,
                "residual_norm": [float(x) for x in norm], "device_bytes": dev_bytes}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--cpu-iters", type=int, default=2)
    ap.add_argument("--cpu-samples", type=int, default=5)
    ap.add_argument("--cpu-cores", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-solves", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "fp32", "batched", "serve", "precision"])
    ap.add_argument("--prec-cells", type=int, default=4_000_000)
    ap.add_argument("--prec-max-iters", type=int, default=4000)
    ap.add_argument("--prec-max-iters-first", type=int, default=20000)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=30.0)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-baseline-seconds", type=float, default=0.0,
                    help="length of the one-at-a-time FP64 baseline stream (0: --serve-seconds)")
    ap.add_argument("--serve-budget-gb", type=float, default=8.0)
    ap.add_argument("--serve-max-iters", type=int, default=2000)
    ap.add_argument("--serve-stall-iters", type=int, default=250,
                    help="retire a served solve whose residual has not dropped 1%% in this many iterations (0: off)")
    ap.add_argument("--pool-meshes", type=int, default=12)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.only != "all":
        run_partial(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
