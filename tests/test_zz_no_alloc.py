"""fv2d_residual_noalloc: the first-order residual for callers that cannot allocate device memory
(their inputs and outputs live in memory they already own; the call's face scratch is a static
device array).  Checked through the C ABI against the existing entry point (a solver handle's
first stage, fv2d_stage) on two calls in a row, to the FP64 parity tolerance; the device's free
memory is the same before and after a call that follows the first; a mesh of exactly the face
limit runs."""
import ctypes

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

TOL = 1e-12
BC = {"FREESTREAM": -1, "SLIP_WALL": -2, "EXTRAPOLATION": -3, "NO_SLIP_WALL": -4}


class NoallocMesh(ctypes.Structure):
    _fields_ = [("num_cells", ctypes.c_int), ("num_faces", ctypes.c_int),
                ("face_cell1", ctypes.c_void_p), ("face_cell2", ctypes.c_void_p),
                ("face_nx", ctypes.c_void_p), ("face_ny", ctypes.c_void_p), ("face_area", ctypes.c_void_p),
                ("cell_face_offsets", ctypes.c_void_p), ("cell_faces", ctypes.c_void_p),
                ("cell_vol", ctypes.c_void_p)]


def device_mesh(pkg, torch, grid, case):
    """Mesh arrays in the reference's numbering, placed in device memory the caller owns."""
    hm = pkg.HostMesh(grid, pkg.case_from_dict(case))
    nf, nc = grid.num_faces, grid.num_cells
    fc1 = (grid.fc1 - 1).astype(np.int32)
    fc2 = np.where(grid.fc2 > 0, grid.fc2 - 1,
                   np.where(grid.fc2 == 0, BC[case["BC1"]], BC[case["BC2"]])).astype(np.int32)
    f = np.arange(nf, dtype=np.int64)
    inter = fc2 >= 0
    cells = np.concatenate([fc1, fc2[inter]]).astype(np.int64)
    ent = np.concatenate([f << 1, (f[inter] << 1) | 1])
    order = np.lexsort((ent >> 1, cells))          # per cell, ascending face id
    off = np.zeros(nc + 1, np.int64)
    np.add.at(off, cells + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    arrays = dict(fc1=dev(fc1), fc2=dev(fc2), nx=dev(hm.geom("nx")), ny=dev(hm.geom("ny")),
                  area=dev(hm.geom("area")), off=dev(off), inc=dev(ent[order].astype(np.int32)),
                  vol=dev(hm.geom("vol")))
    m = NoallocMesh(nc, nf, *[arrays[k].data_ptr() for k in ("fc1", "fc2", "nx", "ny", "area", "off", "inc", "vol")])
    return m, arrays


def perturbed_state(case, n, seed):
    rng = np.random.default_rng(seed)
    rho = case["rho"] * (1 + 0.05 * rng.standard_normal(n))
    u = case["u"] * (1 + 0.05 * rng.standard_normal(n))
    v = 10.0 * rng.standard_normal(n)
    P = case["P"] * (1 + 0.05 * rng.standard_normal(n))
    E = P / (case["gamma"] - 1) + 0.5 * rho * (u * u + v * v)
    return np.concatenate([rho, rho * u, rho * v, E])


def residual_existing(pkg, grid, case, q):
    """The existing entry point: a handle's first stage (res() of the state) with the residual kept."""
    s = pkg.Solver(grid, case, precision=pkg.FP64)
    s.set_store_residual(True)
    s.set_state(q)
    s.stage()
    r = s.get(2)
    s.close()
    return r


def test_residual_noalloc_matches_existing_entry_point_twice(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.library()
    fn = lib.fv2d_residual_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(NoallocMesh), ctypes.POINTER(pkg.Case), ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    grid = pkg.meshgen.voronoi_bump_channel(20000, seed=11)
    assert grid.num_faces <= 262144
    base = dict(pkg.meshgen.DEFAULT_CASE, solution_poly_order=0, limiter="NONE", u=pkg.meshgen.mach_speed(0.6))
    cases = [dict(base, eqn="EULER", BC1="SLIP_WALL", BC2="FREESTREAM"),
             dict(base, eqn="NS", mu=0.01, BC1="NO_SLIP_WALL", BC2="EXTRAPOLATION", v=15.0)]
    r_dev = torch.empty(4 * grid.num_cells, dtype=torch.float64, device="cuda")
    for call, case in enumerate(cases):          # two calls in a row, sharing the static scratch
        m, keep = device_mesh(pkg, torch, grid, case)
        q = perturbed_state(case, grid.num_cells, seed=100 + call)
        q_dev = torch.from_numpy(q).cuda()
        r_dev.fill_(float("nan"))
        cs = pkg.case_from_dict(case)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = fn(ctypes.byref(m), ctypes.byref(cs), q_dev.data_ptr(), r_dev.data_ptr(), None)
        assert rc == 0, lib.fv2d_last_error(None)
        torch.cuda.synchronize()
        if call > 0:   # the first call may place the library's code and scratch (lazy module loading)
            assert torch.cuda.mem_get_info()[0] == free0, "a call after the first took device memory"
        r = r_dev.cpu().numpy()
        ref = residual_existing(pkg, grid, case, q)
        assert np.all(np.isfinite(r))
        assert max_rel(r, ref, floor=1e-30) <= TOL, f"call {call}: max rel {max_rel(r, ref, floor=1e-30):.3e}"


def split_quads(pkg, grid, k):
    """`grid` with its first k quadrilateral cells each cut into two triangles along a diagonal: k
    more cells and k more (interior) faces, appended after the existing ones.  The new face's c1 is
    the triangle on its left (the face normal points out of c1), as the grid format requires."""
    fp1, fp2 = grid.fp1.astype(np.int64).copy(), grid.fp2.astype(np.int64).copy()
    fc1, fc2 = grid.fc1.astype(np.int64).copy(), grid.fc2.astype(np.int64).copy()
    x, y = grid.x, grid.y
    faces_of = {}
    for f in range(grid.num_faces):
        for c in (fc1[f], fc2[f]):
            if c > 0:
                faces_of.setdefault(int(c), []).append(f)
    nf, nc = grid.num_faces, grid.num_cells
    new_faces = []
    for c in range(1, k + 1):
        fs = faces_of[c]
        assert len(fs) == 4
        adj = {}
        for f in fs:
            adj.setdefault(fp1[f], []).append(fp2[f])
            adj.setdefault(fp2[f], []).append(fp1[f])
        loop = [fp1[fs[0]], fp2[fs[0]]]
        while len(loop) < 4:
            a, b = adj[loop[-1]]
            loop.append(a if a != loop[-2] else b)
        p0, p1, p2, p3 = loop
        nc += 1
        for f in fs:   # the edges of triangle (p2, p3, p0) move to the new cell
            if {fp1[f], fp2[f]} in ({p2, p3}, {p3, p0}):
                if fc1[f] == c:
                    fc1[f] = nc
                else:
                    fc2[f] = nc
        dx, dy = x[p2 - 1] - x[p0 - 1], y[p2 - 1] - y[p0 - 1]
        left_is_t1 = dx * (y[p1 - 1] - y[p0 - 1]) - dy * (x[p1 - 1] - x[p0 - 1]) > 0
        new_faces.append((p0, p2, c if left_is_t1 else nc, nc if left_is_t1 else c))
    a = np.array(new_faces, dtype=np.int64)
    cat = lambda u, v: np.concatenate([u, v]).astype(np.int32)  # noqa: E731
    return pkg.meshgen.Grid(x, y, cat(fp1, a[:, 0]), cat(fp2, a[:, 1]), cat(fc1, a[:, 2]), cat(fc2, a[:, 3]), nc,
                            f"{grid.name}_split{k}")


def test_residual_noalloc_at_the_face_limit(pkg):
    """A mesh of exactly FV2D_NOALLOC_MAX_FACES faces: the last face's contribution lands in the
    scratch array's last entries and the residual equals the existing entry point's."""
    torch = pytest.importorskip("torch")
    lib = pkg.library()
    fn = lib.fv2d_residual_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(NoallocMesh), ctypes.POINTER(pkg.Case), ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    base = pkg.meshgen.channel_bump_quads(512, 255)                # 261,887 faces
    grid = split_quads(pkg, base, 262144 - base.num_faces)
    assert grid.num_faces == 262144
    case = dict(pkg.meshgen.DEFAULT_CASE, solution_poly_order=0, limiter="NONE", eqn="EULER", BC1="SLIP_WALL",
                BC2="FREESTREAM", u=pkg.meshgen.mach_speed(0.5), v=10.0)
    m, keep = device_mesh(pkg, torch, grid, case)
    q = perturbed_state(case, grid.num_cells, seed=7)
    q_dev = torch.from_numpy(q).cuda()
    r_dev = torch.full((4 * grid.num_cells,), float("nan"), dtype=torch.float64, device="cuda")
    cs = pkg.case_from_dict(case)
    rc = fn(ctypes.byref(m), ctypes.byref(cs), q_dev.data_ptr(), r_dev.data_ptr(), None)
    assert rc == 0, lib.fv2d_last_error(None)
    torch.cuda.synchronize()
    r = r_dev.cpu().numpy()
    ref = residual_existing(pkg, grid, case, q)
    assert np.all(np.isfinite(r))
    assert max_rel(r, ref, floor=1e-30) <= TOL


def test_residual_noalloc_rejects_oversized_mesh(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.library()
    fn = lib.fv2d_residual_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(NoallocMesh), ctypes.POINTER(pkg.Case), ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    m = NoallocMesh(4, 262145, p, p, p, p, p, p, p, p)
    cs = pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE))
    rc = fn(ctypes.byref(m), ctypes.byref(cs), p, p, None)
    assert rc == 1
    assert b"exceeds the static scratch limit" in lib.fv2d_last_error(None)
