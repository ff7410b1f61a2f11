"""Generate the golden fixtures of tests/golden/ from the REFERENCE's own solver.

Runs the reference harness (oracle/_ref/libfv2d_ref.so, the reference's unmodified sources built
by oracle/Makefile) on small cases and stores, per case:
  - the mesh (grid_file.in arrays) and the input.in options,
  - per RK stage: SHA-256 of the exact FP64 bytes of the residual, Q*, Qbar and dt (file order,
    SoA), and for small meshes the arrays themselves,
  - SHA-256 of the reference geometry arrays.
Long-horizon cases (files named long_*.npz) store, instead of every stage, the SHA-256 of Qbar and
the residual after whole SSP-RK3 iterations (ssp_rk3() called as main.cpp:121-133 calls it) at a
list of checkpoints.
The GPU parity tests replay the same mesh and options and must reproduce these bytes.
Run where the reference tree exists (FV2D_REFERENCE, default /root/reference):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

REF_TREE = os.environ.get("FV2D_REFERENCE", "/root/reference")
REF_GRIDS = os.path.join(REF_TREE, "grids")
FULL_ARRAYS_MAX_CELLS = 200
GEOM_NAMES = ["area", "nx", "ny", "fcx", "fcy", "c1dx", "c1dy", "c2dx", "c2dy", "dxj", "dyj", "dist", "lx", "ly",
              "mx", "my", "vol", "ccx", "ccy", "Ixx", "Iyy", "Ixy", "delta"]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def cases(mg):
    m05 = mg.mach_speed(0.5)
    ch16 = mg.channel_bump_quads(16, 8)
    ch128 = mg.channel_bump_quads(128, 64)
    simple = mg.read_grid(os.path.join(REF_GRIDS, "simple_grid.in"), "simple_grid")
    airfoil = mg.read_grid(os.path.join(REF_GRIDS, "grid_file.in"), "airfoil")
    # a Voronoi bump channel with 4-6-sided cells (the reference's reader takes at most 6 sides)
    vor = mg.voronoi_bump_channel(3000, seed=3, jitter=0.15)
    m07 = mg.mach_speed(0.7)
    ns = dict(eqn="NS", mu=0.5, Pr=0.72)
    return [
        ("ch16_euler_sq_global", ch16, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8,
                                            BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), 12, None),
        ("ch16_ns_none_local_noslip", ch16, dict(ns, limiter="NONE", time_step_type="LOCAL", CFL=0.9,
                                                 BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=m05), 12, None),
        ("ch16_ns_sq_local_extrap", ch16, dict(ns, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.9,
                                               BC1="NO_SLIP_WALL", BC2="EXTRAPOLATION", u=m05), 12, None),
        ("ch16_ns_sq_slip", ch16, dict(ns, limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.5,
                                       BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), 9, None),
        ("ch16_euler_order0", ch16, dict(eqn="EULER", solution_poly_order=0, limiter="NONE",
                                         time_step_type="GLOBAL", CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM",
                                         u=m05), 9, None),
        ("ch16_euler_minmod_extrap", ch16, dict(eqn="EULER", limiter="MINMOD", time_step_type="LOCAL", CFL=0.7,
                                                BC1="EXTRAPOLATION", BC2="FREESTREAM", u=m05, v=20.0), 9, None),
        ("ch16_euler_sq_restart", ch16, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.8,
                                             BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), 9, 12345),
        ("simple_euler_sq", simple, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8,
                                         BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), 9, None),
        ("airfoil_ns_sq_local", airfoil, dict(ns, mu=0.04168601, limiter="SQUEEZE", time_step_type="LOCAL",
                                              CFL=1.0, BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=170.147), 6, None),
        ("airfoil_euler_sq_global", airfoil, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL",
                                                  CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM", u=170.147), 6, None),
        ("channel128_euler_sq_global", ch128, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL",
                                                   CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), 15, None),
        ("vor3k_euler_sq_global", vor, dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8,
                                            BC1="SLIP_WALL", BC2="FREESTREAM", u=m07), 12, None),
        ("vor3k_ns_sq_local_noslip", vor, dict(ns, mu=0.05, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.9,
                                               BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=m07), 12, None),
        # flux_solver = ROE: the reference's res() computes no inviscid flux (res.cpp:62-69)
        ("ch16_ns_roe_sq_local", ch16, dict(ns, flux_solver="ROE", limiter="SQUEEZE", time_step_type="LOCAL",
                                            CFL=0.5, BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=m05), 9, None),
        ("ch16_euler_roe_order0", ch16, dict(eqn="EULER", flux_solver="ROE", solution_poly_order=0,
                                             limiter="NONE", time_step_type="GLOBAL", CFL=0.1, BC1="SLIP_WALL",
                                             BC2="FREESTREAM", u=m05), 9, None),
    ]


def long_cases(mg):
    """(name, grid, options, iteration checkpoints): whole runs of the driver loop."""
    m05 = mg.mach_speed(0.5)
    # the plain FP64 method as the benchmark configuration states it: 128x64 quads of a 3 x 1 channel
    # with a 10 %-thick circular-arc bump, Euler, second order, squeeze, GLOBAL dt at CFL 0.8,
    # Mach 0.5, slip walls and freestream inlet/outlet, 2000 iterations
    return [
        ("long_c1_channel128_euler_sq_global", mg.channel_bump_quads(128, 64),
         dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM",
              u=m05, nmax=2000), [1, 10, 100, 500, 2000]),
    ]


def stable(case):
    """The case as stored: the grid path (a temporary file) reduced to its name, so that
    regenerating the fixtures reproduces their bytes."""
    return dict(case, grid_file=os.path.basename(case["grid_file"]))


def restart_state(grid, case, seed):
    """A seeded perturbation of the freestream state (restart-path input)."""
    rng = np.random.default_rng(seed)
    n = grid.num_cells
    rho = case["rho"] * (1 + 0.05 * rng.standard_normal(n))
    u = case["u"] * (1 + 0.05 * rng.standard_normal(n))
    v = 10.0 * rng.standard_normal(n)
    P = case["P"] * (1 + 0.05 * rng.standard_normal(n))
    E = P / (case["gamma"] - 1) + 0.5 * rho * (u * u + v * v)
    return np.concatenate([rho, rho * u, rho * v, E])


def main():
    pkg = entry.load_package()
    orc = entry.load_oracle()
    orc.build(ref_dir=REF_TREE)
    assert orc.available("ref"), "reference harness not built"
    mg = pkg.meshgen
    tmp = tempfile.mkdtemp()
    manifest = {}
    for name, grid, opts, nstages, restart_seed in cases(mg):
        gpath = os.path.join(tmp, name + ".grid")
        mg.write_grid(gpath, grid)
        ipath = os.path.join(tmp, name + ".in")
        case = mg.write_input(ipath, grid_file=gpath, **opts)
        ref = orc.Oracle("ref", ipath)
        out = dict(x=grid.x, y=grid.y, fp1=grid.fp1, fp2=grid.fp2, fc1=grid.fc1, fc2=grid.fc2,
                   num_cells=np.int64(grid.num_cells), case_json=np.array(json.dumps(stable(case))),
                   nstages=np.int64(nstages))
        if restart_seed is not None:
            q0 = restart_state(grid, case, restart_seed)
            ref.set_state(q0)
            out["restart_state"] = q0
        geo = {g: sha(ref.geom(g)) for g in GEOM_NAMES}
        full = grid.num_cells <= FULL_ARRAYS_MAX_CELLS
        hashes = []
        for s in range(nstages):
            ref.stage()
            rec = {"res": sha(ref.get(orc.RES)), "qbar": sha(ref.get(orc.QBAR)), "dt": sha(ref.get(orc.DT))}
            if s % 3 != 2:
                rec["qstar"] = sha(ref.get(orc.QSTAR))
            hashes.append(rec)
            if full:
                out[f"res_{s}"] = ref.get(orc.RES)
                out[f"qbar_{s}"] = ref.get(orc.QBAR)
                if s % 3 != 2:
                    out[f"qstar_{s}"] = ref.get(orc.QSTAR)
        out["final_qbar"] = ref.get(orc.QBAR)
        out["final_res"] = ref.get(orc.RES)
        out["stage_hashes"] = np.array(json.dumps(hashes))
        out["geom_hashes"] = np.array(json.dumps(geo))
        out["sizes"] = np.array(ref.sizes(), dtype=np.int64)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        manifest[name] = dict(cells=grid.num_cells, faces=grid.num_faces, stages=nstages, options=opts)
        print(name, grid.num_cells, "cells", nstages, "stages")
    for name, grid, opts, checkpoints in long_cases(mg):
        gpath = os.path.join(tmp, name + ".grid")
        mg.write_grid(gpath, grid)
        ipath = os.path.join(tmp, name + ".in")
        case = mg.write_input(ipath, grid_file=gpath, **opts)
        ref = orc.Oracle("ref", ipath)
        recs, done = [], 0
        for n in checkpoints:
            ref.iterate(n - done)
            done = n
            recs.append({"iter": n, "qbar": sha(ref.get(orc.QBAR)), "res": sha(ref.get(orc.RES))})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), x=grid.x, y=grid.y, fp1=grid.fp1, fp2=grid.fp2,
                            fc1=grid.fc1, fc2=grid.fc2, num_cells=np.int64(grid.num_cells),
                            case_json=np.array(json.dumps(stable(case))), iter_hashes=np.array(json.dumps(recs)))
        manifest[name] = dict(cells=grid.num_cells, faces=grid.num_faces, iterations=checkpoints, options=opts)
        print(name, grid.num_cells, "cells", checkpoints[-1], "iterations")
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
