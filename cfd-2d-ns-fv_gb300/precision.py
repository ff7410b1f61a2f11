"""Precision study: the FP32 path against the FP64 path (the bit-exact oracle-equivalent) run to a
residual drop, with density / pressure L2 and Linf errors and the integrated wall-force error.

Wall force = sum over BC1 (wall) faces of P_face * n * A, with P_face from the wall face's
reconstructed state (cell value + limited gradient . (face centre - cell centroid)), evaluated on
the FP64 geometry.  This is the physical wall force, not save()'s CL/CD (which truncates
coordinates to int, src/base/save_sol.cpp:28-32).
"""
from __future__ import annotations

import time

import numpy as np

from . import fv2d


def primitives(q, gamma):
    n = q.size // 4
    rho, ru, rv, E = q[:n], q[n:2 * n], q[2 * n:3 * n], q[3 * n:]
    u, v = ru / rho, rv / rho
    P = (E - 0.5 * rho * (u * u + v * v)) * (gamma - 1)
    return rho, P


def wall_force(solver, grid, gamma):
    """Integrated pressure force on the BC1 faces (file code 0)."""
    nc = grid.num_cells
    q = solver.get_state()
    g = solver.get(fv2d.F_QBAR_GRAD)
    wall = np.nonzero(grid.fc2 == 0)[0]
    c1 = grid.fc1[wall] - 1
    d1x, d1y = solver.get(fv2d.GEOM["c1dx"])[wall], solver.get(fv2d.GEOM["c1dy"])[wall]
    nx, ny, A = (solver.get(fv2d.GEOM[k])[wall] for k in ("nx", "ny", "area"))
    face = [q[j * nc + c1] + g[j * nc + c1] * d1x + g[(4 + j) * nc + c1] * d1y for j in range(4)]
    rho, ru, rv, E = face
    P = (E - 0.5 * (ru * ru + rv * rv) / rho) * (gamma - 1)
    return np.array([np.sum(P * nx * A), np.sum(P * ny * A)])


def run_to_drop(grid, case, precision, drop=1e-6, max_iters=20000, check_every=50):
    s = fv2d.Solver(grid, case, precision=precision)
    s.step(1)
    r0 = s.residual_norm()
    it = 1
    hist = [(it, r0.tolist())]
    t0 = time.perf_counter()
    converged = False
    while it < max_iters:
        s.step(check_every)
        it += check_every
        r = s.residual_norm()
        hist.append((it, r.tolist()))
        if np.all(r <= drop * r0):
            converged = True
            break
        if not np.all(np.isfinite(r)):
            break
    return s, dict(iterations=it, converged=converged, seconds=time.perf_counter() - t0,
                   drop=(r / r0).tolist(), history=hist)


def compare(grid, case, drop=1e-6, max_iters=20000, check_every=50):
    """Run both precisions to the residual drop (or the iteration cap) and compare."""
    gamma = case["gamma"]
    s64, info64 = run_to_drop(grid, case, fv2d.FP64, drop, max_iters, check_every)
    s32, info32 = run_to_drop(grid, case, fv2d.FP32, drop, max_iters, check_every)
    q64, q32 = s64.get_state(), s32.get_state()
    rho64, P64 = primitives(q64, gamma)
    rho32, P32 = primitives(q32, gamma)
    f64, f32 = wall_force(s64, grid, gamma), wall_force(s32, grid, gamma)
    out = dict(
        cells=grid.num_cells, faces=grid.num_faces,
        rho_l2=float(np.linalg.norm(rho32 - rho64) / np.linalg.norm(rho64)),
        rho_linf=float(np.max(np.abs(rho32 - rho64)) / np.max(np.abs(rho64))),
        P_l2=float(np.linalg.norm(P32 - P64) / np.linalg.norm(P64)),
        P_linf=float(np.max(np.abs(P32 - P64)) / np.max(np.abs(P64))),
        wall_force_fp64=f64.tolist(), wall_force_fp32=f32.tolist(),
        wall_force_rel_err=float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
        fp64=dict((k, v) for k, v in info64.items() if k != "history"),
        fp32=dict((k, v) for k, v in info32.items() if k != "history"),
    )
    s64.close()
    s32.close()
    return out
