"""Synthetic meshes in the fv2d ``grid_file.in`` format, plus input.in writing.

The grid format is the one ``readmesh`` reads (src/base/readmesh.cpp:31-85)::

    np nf nc
    x y                      (np lines)
    p1 p2                    (nf lines, 1-based point ids)
    c1 c2                    (nf lines, 1-based cell ids; c2 = 0 -> BC1, c2 = -1 -> BC2)

Face orientation follows readmesh.cpp:129-134: the normal is (dy, -dx)/|d| for d = p2 - p1 and
points out of c1, i.e. c1 lies to the left of p1 -> p2.

Every generator writes its boundary faces first (BC1 faces, then BC2 faces) and puts the BC1
wall points first.  Two reference behaviours depend on that ordering: the NS geometry indexes
BC_faces[] by face id (readmesh.cpp:373,394), and the NO_SLIP_WALL gradient ghost reads cell
number `face id` (src/solver/cell_gradient.cpp:63-66).  The surface output assumes wall faces and
wall points come first (src/base/save_sol.cpp:23-24,227).
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

BC_CODES = {"FREESTREAM": -1, "SLIP_WALL": -2, "EXTRAPOLATION": -3, "NO_SLIP_WALL": -4}


@dataclasses.dataclass
class Grid:
    """A mesh in file conventions (1-based ids, c2 = 0 / -1 for BC1 / BC2)."""

    x: np.ndarray          # float64 [np]
    y: np.ndarray          # float64 [np]
    fp1: np.ndarray        # int32 [nf]
    fp2: np.ndarray        # int32 [nf]
    fc1: np.ndarray        # int32 [nf]
    fc2: np.ndarray        # int32 [nf]
    num_cells: int
    name: str = "grid"

    @property
    def num_points(self) -> int:
        return int(self.x.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.fp1.shape[0])

    def sides_histogram(self) -> dict:
        cnt = np.bincount(self.fc1 - 1, minlength=self.num_cells)
        inter = self.fc2 > 0
        cnt += np.bincount(self.fc2[inter] - 1, minlength=self.num_cells)
        vals, counts = np.unique(cnt, return_counts=True)
        return {int(v): int(c) for v, c in zip(vals, counts)}


def write_grid(path: str, g: Grid) -> None:
    """Write ``g`` in the grid_file.in format (17 significant digits, so the file round-trips)."""
    with open(path, "w") as fh:
        fh.write(f"{g.num_points} {g.num_faces} {g.num_cells}\n")
        np.savetxt(fh, np.column_stack([g.x, g.y]), fmt="%.17g")
        np.savetxt(fh, np.column_stack([g.fp1, g.fp2]), fmt="%d")
        np.savetxt(fh, np.column_stack([g.fc1, g.fc2]), fmt="%d")


def read_grid(path: str, name: str | None = None) -> Grid:
    """Read a grid_file.in (whitespace separated, as readmesh's ``>>`` reads it)."""
    with open(path) as fh:
        tok = fh.read().split()
    npt, nf, nc = int(tok[0]), int(tok[1]), int(tok[2])
    o = 3
    xy = np.array(tok[o:o + 2 * npt], dtype=np.float64).reshape(npt, 2)
    o += 2 * npt
    fp = np.array(tok[o:o + 2 * nf], dtype=np.int64).reshape(nf, 2)
    o += 2 * nf
    fc = np.array(tok[o:o + 2 * nf], dtype=np.int64).reshape(nf, 2)
    return Grid(xy[:, 0].copy(), xy[:, 1].copy(), fp[:, 0].astype(np.int32), fp[:, 1].astype(np.int32),
                fc[:, 0].astype(np.int32), fc[:, 1].astype(np.int32), nc, name or os.path.basename(path))


# --------------------------------------------------------------------------- input.in
DEFAULT_CASE = dict(
    nmax=100, monitor_step=50, output_step=1000, solution_poly_order=1, restart=0,
    grid_file="grid_file.in", eqn="EULER", flux_solver="RUSANOV",
    gamma=1.4, R=287.0, mu=0.0, Pr=0.72, P=101325.0, rho=1.225, u=170.147, v=0.0,
    time_scheme="SSP_RK3", time_step_type="GLOBAL", CFL=0.8, limiter="SQUEEZE", length=1.0,
    BC1="SLIP_WALL", BC2="FREESTREAM",
)


def write_input(path: str, **kw) -> dict:
    """Write an input.in with the reference's 9 sections (read_inputs.cpp:20-208)."""
    c = dict(DEFAULT_CASE)
    c.update(kw)
    r = lambda v: repr(float(v))  # noqa: E731  (round-trip exact decimal)
    txt = f"""[case]
    nmax = {int(c['nmax'])}
    monitor_step = {int(c['monitor_step'])}
    output_step = {int(c['output_step'])}
    solution_poly_order = {int(c['solution_poly_order'])}
    restart = {int(c['restart'])}

[grid]
    grid_file = {c['grid_file']}

[equations]
    eqn = {c['eqn']}
    flux_solver = {c['flux_solver']}

[fluid]
    gamma = {r(c['gamma'])}
    R = {r(c['R'])}
    mu = {r(c['mu'])}
    Pr = {r(c['Pr'])}

[init]
    P = {r(c['P'])}
    rho = {r(c['rho'])}
    u = {r(c['u'])}
    v = {r(c['v'])}

[time]
    time_scheme = {c['time_scheme']}
    time_step_type = {c['time_step_type']}
    CFL = {r(c['CFL'])}

[limiter]
    limiter = {c['limiter']}

[report]
    length = {r(c['length'])}

[BC]
    BC1 = {c['BC1']}
    BC2 = {c['BC2']}
"""
    with open(path, "w") as fh:
        fh.write(txt)
    return c


def mach_speed(mach: float, gamma: float = 1.4, P: float = 101325.0, rho: float = 1.225) -> float:
    return mach * math.sqrt(gamma * P / rho)


# --------------------------------------------------------------------------- structured channel
def bump_wall(x: np.ndarray, x0: float = 1.0, x1: float = 2.0, thickness: float = 0.1) -> np.ndarray:
    """Lower wall of a channel with a circular-arc bump of the given thickness over [x0, x1]."""
    half = 0.5 * (x1 - x0)
    rad = (half * half + thickness * thickness) / (2.0 * thickness)
    xc = 0.5 * (x0 + x1)
    yc = thickness - rad
    y = np.zeros_like(x)
    m = (x > x0) & (x < x1)
    y[m] = yc + np.sqrt(rad * rad - (x[m] - xc) ** 2)
    return y


def channel_bump_quads(nx: int = 128, ny: int = 64, length: float = 3.0, height: float = 1.0,
                       thickness: float = 0.1) -> Grid:
    """Quadrilateral channel [0, length] x [wall, height] with a circular-arc bump over [1, 2].

    Nodes are uniform in x and uniform in y between the lower wall and the top.  BC1 (file code 0)
    is the lower wall (x order) then the upper wall; BC2 (file code -1) is the inlet then the
    outlet.  Cells are numbered row by row (cell (i, j) -> j*nx + i + 1).
    """
    xs = np.linspace(0.0, length, nx + 1)
    yw = bump_wall(xs, 1.0, 2.0, thickness) if thickness > 0 else np.zeros_like(xs)
    t = np.arange(ny + 1, dtype=np.float64) / ny
    X = np.broadcast_to(xs[None, :], (ny + 1, nx + 1))
    Y = yw[None, :] + (height - yw[None, :]) * t[:, None]
    # point numbering: bottom wall row first (j = 0), then rows upwards: pid(i, j) = j*(nx+1) + i
    x = X.reshape(-1).astype(np.float64)
    y = Y.reshape(-1).astype(np.float64)
    pid = lambda i, j: j * (nx + 1) + i + 1  # noqa: E731
    cid = lambda i, j: j * nx + i + 1        # noqa: E731
    P1, P2, C1, C2 = [], [], [], []

    def add(p1, p2, c1, c2):
        P1.append(p1); P2.append(p2); C1.append(c1); C2.append(c2)

    i = np.arange(nx)
    j = np.arange(ny)
    # BC1: lower wall (left to right, c1 above), then upper wall (right to left, c1 below)
    add(pid(i, 0), pid(i + 1, 0), cid(i, 0), np.zeros(nx, int))
    add(pid(i + 1, ny), pid(i, ny), cid(i, ny - 1), np.zeros(nx, int))
    # BC2: inlet (downwards), outlet (upwards)
    add(pid(0, j + 1), pid(0, j), cid(0, j), -np.ones(ny, int))
    add(pid(nx, j), pid(nx, j + 1), cid(nx - 1, j), -np.ones(ny, int))
    # interior vertical faces at node columns 1..nx-1 (c1 = left cell)
    ii, jj = np.meshgrid(np.arange(1, nx), j, indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    add(pid(ii, jj), pid(ii, jj + 1), cid(ii - 1, jj), cid(ii, jj))
    # interior horizontal faces at node rows 1..ny-1 (c1 = lower cell)
    ii, jj = np.meshgrid(i, np.arange(1, ny), indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    add(pid(ii + 1, jj), pid(ii, jj), cid(ii, jj - 1), cid(ii, jj))
    cat = lambda L: np.concatenate([np.asarray(a).reshape(-1) for a in L]).astype(np.int32)  # noqa: E731
    return Grid(x, y, cat(P1), cat(P2), cat(C1), cat(C2), nx * ny, f"channel_bump_{nx}x{ny}")
