"""Generate the golden output files of the command-line driver from the REFERENCE program.

Builds the reference program (oracle/_ref/fv2d_ref: the reference's src/base/main.cpp and solver
sources, unmodified, by oracle/Makefile) and runs it on small cases in a scratch directory, exactly
as a user would (input.in and grid_file.in in the working directory).  Stored per case
(tests/golden/cli/<case>.npz): the grid file and input.in texts, and every file the run leaves
under sol/ and mesh/ - its bytes for small meshes, and for all its length and the SHA-256 of its
bytes less the undefined last-row tau fields of tec_surf files (tests/cli_check.py).  A case
with `restart` runs twice (`inputs` holds one input.in text per run): to `nmax` / 2 with
restart = 0, then to `nmax` with restart = 1 from the restart file the first run wrote.  The GPU
test runs lib/fv2d_gpu the same way and compares the files.
Run here (where the reference tree exists):  python tests/golden/make_cli_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
import cli_check  # noqa: E402

REF = "/root/reference"
REF_PROG = os.path.join(ROOT, "oracle", "_ref", "fv2d_ref")
FULL_BYTES_MAX_CELLS = 200


def cases(mg):
    m05 = mg.mach_speed(0.5)
    ch16 = mg.channel_bump_quads(16, 8)
    airfoil = mg.read_grid(os.path.join(REF, "grids", "grid_file.in"), "airfoil")
    vor = mg.voronoi_bump_channel(400, seed=3, jitter=0.05)     # 4-6 sided cells (the reference reads <= 6)
    ns = dict(eqn="NS", mu=0.5, Pr=0.72)
    io = dict(nmax=12, monitor_step=3, output_step=6)
    return [
        ("ch16_euler_sq_global", ch16, dict(io, eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8,
                                            BC1="SLIP_WALL", BC2="FREESTREAM", u=m05), False),
        ("ch16_ns_sq_local_noslip", ch16, dict(io, **ns, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.9,
                                               BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=m05), False),
        ("ch16_euler_order0_restart", ch16, dict(io, eqn="EULER", solution_poly_order=0, limiter="NONE",
                                                 time_step_type="LOCAL", CFL=0.8, BC1="SLIP_WALL",
                                                 BC2="FREESTREAM", u=m05), True),
        ("vorbump_ns_none_local", vor, dict(io, **dict(ns, mu=0.05), limiter="NONE", time_step_type="LOCAL", CFL=0.5,
                                           BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=m05), False),
        ("airfoil_ns_sq_local", airfoil, dict(nmax=6, monitor_step=2, output_step=3, **dict(ns, mu=0.04168601),
                                              limiter="SQUEEZE", time_step_type="LOCAL", CFL=1.0,
                                              BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=170.147), False),
    ]


def collect(work):
    files = {}
    for sub in ("sol", "mesh"):
        for name in sorted(os.listdir(os.path.join(work, sub))):
            with open(os.path.join(work, sub, name), "rb") as fh:
                files[f"{sub}/{name}"] = fh.read()
    return files


def run(prog, work):
    r = subprocess.run([prog], cwd=work, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"{prog} failed in {work}: {r.stderr[-2000:]}")


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "refprog"], check=True)
    pkg = entry.load_package()
    mg = pkg.meshgen
    for name, grid, opts, restart in cases(mg):
        work = tempfile.mkdtemp(prefix=f"cli_{name}_")
        mg.write_grid(os.path.join(work, "grid_file.in"), grid)
        phases = [dict(opts, nmax=opts["nmax"] // 2), dict(opts, restart=1)] if restart else [opts]
        inputs = []
        for ph in phases:
            mg.write_input(os.path.join(work, "input.in"), grid_file="grid_file.in", **ph)
            with open(os.path.join(work, "input.in")) as fh:
                inputs.append(fh.read())
            run(REF_PROG, work)
        files = collect(work)
        with open(os.path.join(work, "grid_file.in")) as fh:
            grid_txt = fh.read()
        out = dict(grid_file=np.array(grid_txt), inputs=np.array(inputs), cells=np.int64(grid.num_cells))
        full = grid.num_cells <= FULL_BYTES_MAX_CELLS
        names = sorted(files)
        out["names"] = np.array(names)
        out["sha256"] = np.array([cli_check.digest(n, files[n]) for n in names])
        out["length"] = np.array([len(files[n]) for n in names], dtype=np.int64)
        if full:
            for i, n in enumerate(names):
                out[f"file_{i}"] = np.frombuffer(files[n], dtype=np.uint8)
        os.makedirs(os.path.join(HERE, "cli"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "cli", f"{name}.npz"), **out)
        print(name, grid.num_cells, "cells:", ", ".join(names))


if __name__ == "__main__":
    main()
