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


def _native():
    """The library's C++ grid reader/writer when it is built (host code; no GPU needed)."""
    from . import build as _b
    if not os.path.exists(_b.LIB):
        return None
    from . import fv2d
    return fv2d


def write_grid(path: str, g: Grid) -> None:
    """Write ``g`` in the grid_file.in format (17 significant digits, so the file round-trips).
    Uses the library's C++ writer when it is built (same bytes, ~10x faster than numpy)."""
    nat = _native()
    if nat is not None:
        nat.write_grid(path, g)
        return
    with open(path, "w") as fh:
        fh.write(f"{g.num_points} {g.num_faces} {g.num_cells}\n")
        np.savetxt(fh, np.column_stack([g.x, g.y]), fmt="%.17g")
        np.savetxt(fh, np.column_stack([g.fp1, g.fp2]), fmt="%d")
        np.savetxt(fh, np.column_stack([g.fc1, g.fc2]), fmt="%d")


def read_grid(path: str, name: str | None = None) -> Grid:
    """Read a grid_file.in (whitespace separated, as readmesh's ``>>`` reads it); the library's C++
    parser when it is built."""
    nat = _native()
    if nat is not None:
        x, y, fp1, fp2, fc1, fc2, nc = nat.read_grid(path)
        return Grid(x, y, fp1, fp2, fc1, fc2, nc, name or os.path.basename(path))
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


# --------------------------------------------------------------------------- Voronoi meshes
def _voronoi_grid(seeds: np.ndarray, ghosts: np.ndarray, ghost_code: np.ndarray, name: str,
                  vertex_map=None, wall_angle_center=None) -> Grid:
    """Polygonal mesh from the Voronoi diagram of ``seeds`` closed by mirror ``ghosts``.

    A ridge between two seeds is an interior face; a ridge between a seed and a ghost is a
    boundary face with the ghost's file code (0 -> BC1, -1 -> BC2); ghost-ghost ridges are dropped.
    ``vertex_map`` maps Voronoi vertices (and seeds) into the physical domain.  BC1 faces are
    written first (ordered by angle about ``wall_angle_center`` when given), then BC2 faces, then
    interior faces; BC1 wall points come first.
    """
    from scipy.spatial import Voronoi

    n = seeds.shape[0]
    pts = np.concatenate([seeds, ghosts])
    vor = Voronoi(pts)
    rp = vor.ridge_points.astype(np.int64)
    rv = np.asarray(vor.ridge_vertices, dtype=np.int64)
    a_in, b_in = rp[:, 0] < n, rp[:, 1] < n
    keep = a_in | b_in
    rp, rv = rp[keep], rv[keep]
    a_in, b_in = a_in[keep], b_in[keep]
    if np.any(rv < 0):
        raise RuntimeError(f"{name}: an interior cell is unbounded (ghost layer too thin)")
    V = vor.vertices.copy()
    # merge (near-)coincident vertices left by co-circular seeds: drop zero-length ridges
    seglen = np.hypot(*(V[rv[:, 1]] - V[rv[:, 0]]).T)
    scale = np.median(seglen)
    short = seglen < 1e-9 * scale
    if np.any(short):
        parent = np.arange(V.shape[0])

        def find(u):
            while parent[u] != u:
                parent[u] = parent[parent[u]]
                u = parent[u]
            return u

        for u, w in rv[short]:
            ru, rw = find(u), find(w)
            if ru != rw:
                parent[max(ru, rw)] = min(ru, rw)
        root = np.array([find(u) for u in range(V.shape[0])])
        rv = root[rv]
        ok = rv[:, 0] != rv[:, 1]
        rp, rv, a_in, b_in = rp[ok], rv[ok], a_in[ok], b_in[ok]
    if vertex_map is not None:
        V = vertex_map(V)
        seeds_m = vertex_map(seeds)
    else:
        seeds_m = seeds
    interior = a_in & b_in
    c_in = np.where(a_in, rp[:, 0], rp[:, 1])                 # the seed side of a boundary ridge
    c_gh = np.where(a_in, rp[:, 1], rp[:, 0]) - n
    code = np.where(interior, 1, ghost_code[np.clip(c_gh, 0, None)])
    c1 = np.where(interior, np.minimum(rp[:, 0], rp[:, 1]), c_in)
    c2 = np.where(interior, np.maximum(rp[:, 0], rp[:, 1]), -1)
    # orientation: c1 on the left of p1 -> p2
    p1, p2 = rv[:, 0].copy(), rv[:, 1].copy()
    A, B, S = V[p1], V[p2], seeds_m[c1]
    cross = (B[:, 0] - A[:, 0]) * (S[:, 1] - A[:, 1]) - (B[:, 1] - A[:, 1]) * (S[:, 0] - A[:, 0])
    flip = cross < 0
    p1[flip], p2[flip] = p2[flip], p1[flip]
    # face order: BC1, BC2, interior
    is_bc1 = (~interior) & (code == 0)
    is_bc2 = (~interior) & (code == -1)
    key = np.zeros(len(p1))
    if wall_angle_center is not None:
        mid = 0.5 * (V[p1] + V[p2])
        key = np.arctan2(mid[:, 1] - wall_angle_center[1], mid[:, 0] - wall_angle_center[0])
    o1 = np.nonzero(is_bc1)[0]
    o1 = o1[np.argsort(key[o1], kind="stable")]
    order = np.concatenate([o1, np.nonzero(is_bc2)[0], np.nonzero(interior)[0]])
    p1, p2, c1, c2 = p1[order], p2[order], c1[order], c2[order]
    file_c2 = np.where(c2 >= 0, c2 + 1, 0)
    nb1 = len(o1)
    file_c2[nb1:nb1 + int(is_bc2.sum())] = -1
    file_c2[:nb1] = 0
    # every cell must be a closed polygon: each of its vertices used by exactly two of its faces
    cnt = np.bincount(c1, minlength=n) + np.bincount(c2[c2 >= 0], minlength=n)
    if cnt.min() < 3:
        raise RuntimeError(f"{name}: a cell has fewer than 3 faces")
    inc_c = np.concatenate([c1, c1, c2[c2 >= 0], c2[c2 >= 0]])
    inc_v = np.concatenate([p1, p2, p1[c2 >= 0], p2[c2 >= 0]])
    pair = np.unique(inc_c * np.int64(V.shape[0]) + inc_v, return_counts=True)[1]
    if np.any(pair != 2):
        raise RuntimeError(f"{name}: open cell polygon after vertex merging")
    # cell numbering: the cells next to BC1 faces first, in BC1 face order, then the others in seed
    # order.  With one wall face per wall cell this makes cell number k the owner of wall face k,
    # which is the cell the reference's NO_SLIP_WALL gradient ghost reads (cell_gradient.cpp:63-66).
    first_wall = np.unique(c1[:nb1], return_index=True)[1]
    wall_cells = c1[:nb1][np.sort(first_wall)]
    rest = np.setdiff1d(np.arange(n), wall_cells, assume_unique=False)
    cell_new = np.empty(n, np.int64)
    cell_new[np.concatenate([wall_cells, rest])] = np.arange(n)
    c1 = cell_new[c1]
    file_c2 = np.where(file_c2 > 0, cell_new[np.maximum(file_c2 - 1, 0)] + 1, file_c2)
    # compact points; BC1 wall points first (in face order), then the rest by first use
    used_order = np.concatenate([np.stack([p1[:nb1], p2[:nb1]], 1).reshape(-1), np.stack([p1, p2], 1).reshape(-1)])
    _, first = np.unique(used_order, return_index=True)
    uniq = used_order[np.sort(first)]
    remap = -np.ones(V.shape[0], np.int64)
    remap[uniq] = np.arange(len(uniq))
    X = V[uniq]
    return Grid(X[:, 0].copy(), X[:, 1].copy(), (remap[p1] + 1).astype(np.int32), (remap[p2] + 1).astype(np.int32),
                (c1 + 1).astype(np.int32), file_c2.astype(np.int32), n, name)


def _mirror_box(p: np.ndarray, h: np.ndarray, x0, x1, y0, y1, band=4.0):
    """Mirror images of points within ``band*h`` of the edges (and corners) of a box."""
    out = []
    nearL, nearR = p[:, 0] - x0 < band * h, x1 - p[:, 0] < band * h
    nearB, nearT = p[:, 1] - y0 < band * h, y1 - p[:, 1] < band * h
    for m, fx, fy in ((nearL, 1, 0), (nearR, 2, 0), (nearB, 0, 1), (nearT, 0, 2),
                      (nearL & nearB, 1, 1), (nearL & nearT, 1, 2), (nearR & nearB, 2, 1), (nearR & nearT, 2, 2)):
        q = p[m].copy()
        if fx == 1: q[:, 0] = 2 * x0 - q[:, 0]
        if fx == 2: q[:, 0] = 2 * x1 - q[:, 0]
        if fy == 1: q[:, 1] = 2 * y0 - q[:, 1]
        if fy == 2: q[:, 1] = 2 * y1 - q[:, 1]
        out.append(q)
    return np.concatenate(out) if out else np.zeros((0, 2))


def _ring_seeds(h_of_r, r_wall, r_max, rng, jitter_max):
    """Jittered rings about the origin with radial and tangential spacing h(r).  The first ring
    (next to the wall) is regular, so each of its cells owns exactly one wall face."""
    rings = []
    jitter = 0.0
    r = r_wall + 0.5 * h_of_r(r_wall)
    k = 0
    while r < r_max:
        h = h_of_r(r)
        m = max(8, int(round(2 * np.pi * r / h)))
        th = (np.arange(m) + 0.5 * (k & 1)) * (2 * np.pi / m)
        rr = np.full(m, r)
        if jitter > 0:
            th = th + rng.uniform(-jitter, jitter, m) * (2 * np.pi / m)
            rr = rr + rng.uniform(-jitter, jitter, m) * h
        rings.append(np.stack([rr * np.cos(th), rr * np.sin(th), np.full(m, h)], 1))
        jitter = jitter_max                      # the ring next to the wall is not jittered
        r += h
        k += 1
    return np.concatenate(rings)


def voronoi_cylinder(target_cells: int = 1_000_000, seed: int = 0, box=(40.0, 20.0), diameter: float = 1.0,
                     h_wall: float = 0.005, h_far: float = 0.1, jitter: float = 0.2) -> Grid:
    """Polygonal Voronoi mesh of a box with a circular cylinder at its centre.

    Seeds lie on jittered rings (seeded RNG) whose spacing grows linearly from ``h_wall`` at the
    cylinder to ``h_far`` far away; the growth rate is calibrated so the mesh has about
    ``target_cells`` cells.  Cylinder faces (mirror seeds inside the cylinder) are BC1, box faces
    are BC2.  Cells have 3-9 sides.
    """
    W, H = box
    R = 0.5 * diameter
    x0, x1, y0, y1 = -W / 2, W / 2, -H / 2, H / 2
    r_max = float(np.hypot(W / 2, H / 2)) + h_far

    def count(g):
        hr = lambda r: min(h_far, h_wall + g * (r - R))  # noqa: E731
        r, k, tot = R + 0.5 * h_wall, 0, 0.0
        while r < r_max:
            h = hr(r)
            m = max(8, int(round(2 * np.pi * r / h)))
            # fraction of the ring inside the box
            if r <= min(W, H) / 2:
                frac = 1.0
            else:
                t = np.linspace(0, 2 * np.pi, 256, endpoint=False)
                frac = np.mean((np.abs(r * np.cos(t)) < W / 2) & (np.abs(r * np.sin(t)) < H / 2))
            tot += m * frac
            r += h
            k += 1
        return tot

    lo, hi = 1e-5, 1.0
    for _ in range(40):
        mid = np.sqrt(lo * hi)
        if count(mid) > target_cells:
            lo = mid
        else:
            hi = mid
    g = np.sqrt(lo * hi)
    rng = np.random.default_rng(seed)
    hr = lambda r: min(h_far, h_wall + g * (r - R))  # noqa: E731
    s = _ring_seeds(hr, R, r_max, rng, jitter)
    h = s[:, 2]
    inside = (s[:, 0] > x0 + 0.3 * h) & (s[:, 0] < x1 - 0.3 * h) & (s[:, 1] > y0 + 0.3 * h) & (s[:, 1] < y1 - 0.3 * h)
    s = s[inside]
    p, h = s[:, :2], s[:, 2]
    rad = np.hypot(p[:, 0], p[:, 1])
    near = rad < R + 4 * h
    cyl_ghost = p[near] * ((2 * R - rad[near]) / rad[near])[:, None]
    box_ghost = _mirror_box(p, h, x0, x1, y0, y1)
    ghosts = np.concatenate([cyl_ghost, box_ghost])
    code = np.concatenate([np.zeros(len(cyl_ghost), np.int64), -np.ones(len(box_ghost), np.int64)])
    return _voronoi_grid(p, ghosts, code, f"voronoi_cylinder_{len(p)}", wall_angle_center=(0.0, 0.0))


def voronoi_bump_channel(target_cells: int = 4_000_000, seed: int = 0, length: float = 4.0, height: float = 1.0,
                         thickness: float = 0.1, bump=(1.5, 2.5), jitter: float = 0.25) -> Grid:
    """Polygonal Voronoi mesh of a channel with a circular-arc bump on the lower wall.

    Seeds form a jittered hexagonal lattice (seeded RNG) in the straight channel
    [0, length] x [0, height], closed by mirror seeds across its four sides; Voronoi vertices are
    then mapped to the bumped channel by y -> yw(x) + (height - yw(x)) y / height.  Lower and upper
    walls are BC1 (written bottom first), inlet and outlet are BC2.
    """
    area = length * height
    hx = np.sqrt(area / target_cells / (np.sqrt(3) / 2))
    hy = hx * np.sqrt(3) / 2
    ny = max(2, int(round(height / hy)))
    hy = height / ny
    nx = max(2, int(round(length / hx)))
    hx = length / nx
    rng = np.random.default_rng(seed)
    j = np.arange(ny)
    i = np.arange(nx)
    X = (i[None, :] + 0.5 + 0.5 * ((j[:, None] & 1) - 0.5)) * hx
    Y = np.broadcast_to((j[:, None] + 0.5) * hy, X.shape)
    p = np.stack([X.reshape(-1), Y.reshape(-1)], 1)
    p = p + rng.uniform(-jitter, jitter, p.shape) * np.array([hx, hy])
    p[:, 0] = np.clip(p[:, 0], 0.05 * hx, length - 0.05 * hx)
    hh = np.full(len(p), max(hx, hy))
    gL = p[p[:, 0] < 4 * hh[0]] * np.array([-1, 1])
    gR = p[p[:, 0] > length - 4 * hh[0]] * np.array([-1, 1]) + np.array([2 * length, 0])
    gB = p[p[:, 1] < 4 * hh[0]] * np.array([1, -1])
    gT = p[p[:, 1] > height - 4 * hh[0]] * np.array([1, -1]) + np.array([0, 2 * height])
    corners = []
    for cx, sx in ((0.0, -1), (length, -1)):
        for cy, sy in ((0.0, -1), (height, -1)):
            m = (np.abs(p[:, 0] - cx) < 4 * hh[0]) & (np.abs(p[:, 1] - cy) < 4 * hh[0])
            corners.append(np.stack([2 * cx - p[m, 0], 2 * cy - p[m, 1]], 1))
    ghosts = np.concatenate([gB, gT, gL, gR] + corners)
    code = np.concatenate([np.zeros(len(gB) + len(gT), np.int64),
                           -np.ones(len(gL) + len(gR) + sum(len(c) for c in corners), np.int64)])

    def vmap(v):
        yw = bump_wall(v[:, 0], bump[0], bump[1], thickness) if thickness > 0 else np.zeros(len(v))
        return np.stack([v[:, 0], yw + (height - yw) * v[:, 1] / height], 1)

    return _voronoi_grid(p, ghosts, code, f"voronoi_bump_{len(p)}", vertex_map=vmap)
