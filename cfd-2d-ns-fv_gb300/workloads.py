"""The benchmark workloads: seeded synthetic meshes and flow conditions.

c1  128x64 quadrilateral bump channel, Euler, squeeze, GLOBAL dt at CFL 0.8 (the reference's own
    CPU-runnable case).
c2  NS cylinder on a ~1M-cell polygonal Voronoi mesh (Re 100, Mach 0.2, LOCAL dt).
c3  precision study: Euler bump channel on a Voronoi mesh, transonic Mach drawn in 0.6-0.85.
c4  256 independent bump-channel Voronoi solves, cells log-uniform in 2k-200k, bump 4-12 %,
    Mach 0.3-0.8, flow angle -3..3 degrees, Euler or NS with probability 1/2 (Re uniform in
    1e3-1e4 on the channel height), FP32.
c5  a Poisson stream of c4-like requests widened to 5k-2M cells.
Mesh generation runs in a process pool started with the spawn method (safe next to CUDA).
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import multiprocessing as mp
import os

import numpy as np

from . import meshgen as mg


def c1_case():
    grid = mg.channel_bump_quads(128, 64)
    case = dict(mg.DEFAULT_CASE, eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8,
                BC1="SLIP_WALL", BC2="FREESTREAM", u=mg.mach_speed(0.5), v=0.0, nmax=2000)
    return grid, case


def c2_case(cells=1_000_000, seed=0, cfl=0.5):
    grid = mg.voronoi_cylinder(cells, seed=seed)
    u = mg.mach_speed(0.2)
    case = dict(mg.DEFAULT_CASE, eqn="NS", mu=1.225 * u * 1.0 / 100.0, Pr=0.72, u=u, v=0.0, limiter="SQUEEZE",
                time_step_type="LOCAL", CFL=cfl, BC1="NO_SLIP_WALL", BC2="FREESTREAM")
    return grid, case


def c3_case(cells=4_000_000, seed=0, mach=None):
    rng = np.random.default_rng(seed)
    m = float(mach) if mach is not None else float(rng.uniform(0.6, 0.85))
    grid = mg.voronoi_bump_channel(cells, seed=seed)
    case = dict(mg.DEFAULT_CASE, eqn="EULER", limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.8,
                BC1="SLIP_WALL", BC2="FREESTREAM", u=mg.mach_speed(m), v=0.0)
    return grid, case, m


def solve_spec(rng, lo, hi):
    """One c4/c5 solve: mesh parameters and flow conditions."""
    cells = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    spec = dict(cells=cells, seed=int(rng.integers(1 << 30)), thickness=float(rng.uniform(0.04, 0.12)),
                mach=float(rng.uniform(0.3, 0.8)), angle=float(rng.uniform(-3.0, 3.0)),
                ns=bool(rng.random() < 0.5), re=float(rng.uniform(1e3, 1e4)))
    return spec


def spec_case(spec):
    U = mg.mach_speed(spec["mach"])
    a = math.radians(spec["angle"])
    c = dict(mg.DEFAULT_CASE, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.8, u=U * math.cos(a),
             v=U * math.sin(a), BC2="FREESTREAM")
    if spec["ns"]:
        c.update(eqn="NS", mu=1.225 * U * 1.0 / spec["re"], Pr=0.72, BC1="NO_SLIP_WALL")
    else:
        c.update(eqn="EULER", BC1="SLIP_WALL")
    return c


def spec_grid(spec):
    return mg.voronoi_bump_channel(spec["cells"], seed=spec["seed"], thickness=spec["thickness"])


def _grid_worker(spec):
    return spec_grid(spec)


def grids_parallel(specs, workers=None):
    """Generate meshes for many specs in a spawn-started process pool (largest first)."""
    workers = workers or max(1, min(len(specs), (os.cpu_count() or 2)))
    order = sorted(range(len(specs)), key=lambda i: -specs[i]["cells"])
    out = [None] * len(specs)
    if workers == 1:
        for i in order:
            out[i] = spec_grid(specs[i])
        return out
    try:   # spawned workers re-register this package through the repository's loader
        import importlib
        loader = importlib.import_module("__graft_entry__").load_package
    except Exception:
        loader = None
    if loader is None:
        for i in order:
            out[i] = spec_grid(specs[i])
        return out
    ctx = mp.get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=ctx, initializer=loader) as ex:
        futs = {ex.submit(_grid_worker, specs[i]): i for i in order}
        for f in cf.as_completed(futs):
            out[futs[f]] = f.result()
    return out


def c4_specs(n_solves=256, seed=0, lo=2e3, hi=2e5):
    rng = np.random.default_rng(seed)
    return [solve_spec(rng, lo, hi) for _ in range(n_solves)]


def c5_stream(rate=50.0, duration=600.0, seed=0, lo=5e3, hi=2e6):
    """Poisson arrivals: list of (arrival time s, spec)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            return out
        out.append((t, solve_spec(rng, lo, hi)))
