"""fv2d_residual_noalloc: the first-order residual for callers that cannot allocate device memory
(their inputs and outputs live in memory they already own; the call's face scratch is a static
device array).  Checked through the C ABI against the existing entry point (a solver handle's
first stage, fv2d_stage) on two calls in a row, to the FP64 parity tolerance."""
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
        rc = fn(ctypes.byref(m), ctypes.byref(cs), q_dev.data_ptr(), r_dev.data_ptr(), None)
        assert rc == 0, lib.fv2d_last_error(None)
        torch.cuda.synchronize()
        r = r_dev.cpu().numpy()
        ref = residual_existing(pkg, grid, case, q)
        assert np.all(np.isfinite(r))
        assert max_rel(r, ref, floor=1e-30) <= TOL, f"call {call}: max rel {max_rel(r, ref, floor=1e-30):.3e}"


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
