"""Python binding of the C ABI (include/fv2d_gpu.h) over ctypes.

``Solver`` mirrors the reference's solver interface: ``step()`` is ``ssp_rk3()`` applied n times
(src/solver/ssp_rk3.cpp:18), ``stage()`` one residual evaluation plus its RK combination
(src/solver/res.cpp:21), ``set_state`` the restart path (src/base/main.cpp:82-106).  The library
must be built (``build.build()``); nothing here falls back to a CPU implementation: if the native
library or a GPU is missing the calls fail with ``Fv2dError``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

FP64, FP32 = 0, 1
OK = 0
ERRORS = {1: "ERR_ARG", 2: "ERR_IO", 3: "ERR_MESH", 4: "ERR_CASE", 5: "ERR_CUDA", 6: "ERR_NOMEM", 7: "ERR_STATE",
          8: "ERR_NODEV"}
F_QBAR, F_QSTAR, F_RES, F_DT, F_QBAR_GRAD, F_QSTAR_GRAD = range(6)
GEOM = dict(area=20, nx=21, ny=22, fcx=23, fcy=24, c1dx=25, c1dy=26, c2dx=27, c2dy=28, dxj=29, dyj=30, dist=31,
            lx=32, ly=33, mx=34, my=35, vol=40, ccx=41, ccy=42, Ixx=43, Iyy=44, Ixy=45, delta=46, bccx=50, bccy=51)
BC = {"FREESTREAM": -1, "SLIP_WALL": -2, "EXTRAPOLATION": -3, "NO_SLIP_WALL": -4}
EXPORTS = [
    "fv2d_read_inputs", "fv2d_read_grid", "fv2d_write_grid", "fv2d_free", "fv2d_mesh_build", "fv2d_mesh_free", "fv2d_mesh_sizes",
    "fv2d_mesh_get", "fv2d_mesh_permutation", "fv2d_mesh_tiles", "fv2d_create", "fv2d_create_from_files", "fv2d_destroy",
    "fv2d_step", "fv2d_stage", "fv2d_set_state", "fv2d_load_state", "fv2d_get_state", "fv2d_get_field", "fv2d_residual_norm",
    "fv2d_sizes", "fv2d_save", "fv2d_post", "fv2d_write_history_headers", "fv2d_write_mesh_files",
    "fv2d_read_restart", "fv2d_write_restart", "fv2d_synchronize", "fv2d_set_store_residual", "fv2d_set_graphs", "fv2d_set_kernel_timing",
    "fv2d_kernel_times", "fv2d_stream", "fv2d_device_bytes", "fv2d_last_error", "fv2d_residual_noalloc",
    "fv2d_batch_create", "fv2d_batch_destroy", "fv2d_batch_footprint", "fv2d_batch_add", "fv2d_batch_add_mesh",
    "fv2d_batch_remove",
    "fv2d_batch_step", "fv2d_batch_norms", "fv2d_batch_get_state", "fv2d_batch_synchronize", "fv2d_batch_set_tuning",
    "fv2d_batch_get_tuning", "fv2d_batch_set_grid_mode", "fv2d_batch_usage", "fv2d_batch_set_kernel_timing", "fv2d_batch_kernel_times",
    "fv2d_batch_stream",
]


class Fv2dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Case(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("nmax", ctypes.c_int), ("monitor_step", ctypes.c_int),
                ("output_step", ctypes.c_int), ("restart", ctypes.c_int), ("eqn", ctypes.c_int),
                ("flux_solver", ctypes.c_int), ("limiter", ctypes.c_int), ("time_type", ctypes.c_int),
                ("time_scheme", ctypes.c_int), ("bc1", ctypes.c_int), ("bc2", ctypes.c_int),
                ("cfl", ctypes.c_double), ("gamma", ctypes.c_double), ("R", ctypes.c_double),
                ("mu", ctypes.c_double), ("Pr", ctypes.c_double), ("P", ctypes.c_double),
                ("rho", ctypes.c_double), ("u", ctypes.c_double), ("v", ctypes.c_double),
                ("length", ctypes.c_double), ("grid_file", ctypes.c_char * 4096)]


class MeshDesc(ctypes.Structure):
    _fields_ = [("num_points", ctypes.c_int), ("num_faces", ctypes.c_int), ("num_cells", ctypes.c_int),
                ("x", ctypes.POINTER(ctypes.c_double)), ("y", ctypes.POINTER(ctypes.c_double)),
                ("face_point1", ctypes.POINTER(ctypes.c_int)), ("face_point2", ctypes.POINTER(ctypes.c_int)),
                ("face_cell1", ctypes.POINTER(ctypes.c_int)), ("face_cell2", ctypes.POINTER(ctypes.c_int))]


_LIB = None


def library():
    """Load the native library (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(_build.LIB):
            raise Fv2dError(8, f"native library not built: {_build.LIB} (run build())")
        lib = ctypes.CDLL(_build.LIB)
        vp, ip, dp, cp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_char_p
        pvp = ctypes.POINTER(ctypes.c_void_p)
        sig = {
            "fv2d_read_inputs": (ctypes.c_int, [cp, ctypes.POINTER(Case)]),
            "fv2d_free": (None, [vp]),
            "fv2d_read_grid": (ctypes.c_int, [cp, ip, ip, ip, ctypes.POINTER(dp), ctypes.POINTER(dp), ctypes.POINTER(ip),
                                              ctypes.POINTER(ip), ctypes.POINTER(ip), ctypes.POINTER(ip)]),
            "fv2d_write_grid": (ctypes.c_int, [cp, ctypes.POINTER(MeshDesc)]),
            "fv2d_mesh_build": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Case), pvp]),
            "fv2d_mesh_free": (None, [vp]),
            "fv2d_mesh_sizes": (ctypes.c_int, [vp, ip]),
            "fv2d_mesh_get": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "fv2d_mesh_permutation": (ctypes.c_int, [vp, ctypes.c_int, ip]),
            "fv2d_mesh_tiles": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong)]),
            "fv2d_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Case), ctypes.c_int, pvp]),
            "fv2d_create_from_files": (ctypes.c_int, [cp, ctypes.c_int, pvp]),
            "fv2d_destroy": (None, [vp]),
            "fv2d_step": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_stage": (ctypes.c_int, [vp]),
            "fv2d_set_state": (ctypes.c_int, [vp, dp]),
            "fv2d_load_state": (ctypes.c_int, [vp, dp]),
            "fv2d_get_state": (ctypes.c_int, [vp, dp]),
            "fv2d_get_field": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "fv2d_residual_norm": (ctypes.c_int, [vp, dp]),
            "fv2d_sizes": (ctypes.c_int, [vp, ip]),
            "fv2d_save": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_post": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_write_history_headers": (ctypes.c_int, [vp]),
            "fv2d_write_mesh_files": (ctypes.c_int, [vp]),
            "fv2d_read_restart": (ctypes.c_int, [cp, ctypes.c_int, ip, dp]),
            "fv2d_write_restart": (ctypes.c_int, [vp, cp, ctypes.c_int, ctypes.c_int]),
            "fv2d_synchronize": (ctypes.c_int, [vp]),
            "fv2d_set_store_residual": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_set_graphs": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_set_kernel_timing": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_kernel_times": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int, dp, ip, ctypes.c_int, ip]),
            "fv2d_stream": (vp, [vp]),
            "fv2d_device_bytes": (ctypes.c_longlong, [vp]),
            "fv2d_last_error": (ctypes.c_char_p, [vp]),
            "fv2d_batch_create": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, pvp]),
            "fv2d_batch_destroy": (None, [vp]),
            "fv2d_batch_footprint": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
            "fv2d_batch_add": (ctypes.c_int, [vp, ctypes.POINTER(MeshDesc), ctypes.POINTER(Case), ip]),
            "fv2d_batch_add_mesh": (ctypes.c_int, [vp, vp, ctypes.POINTER(Case), ip]),
            "fv2d_batch_remove": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_batch_step": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_batch_norms": (ctypes.c_int, [vp, ip, dp, ip, ctypes.c_int, ip]),
            "fv2d_batch_get_state": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "fv2d_batch_synchronize": (ctypes.c_int, [vp]),
            "fv2d_batch_set_tuning": (ctypes.c_int, [vp, ctypes.c_int, ip, ip]),
            "fv2d_batch_get_tuning": (ctypes.c_int, [vp, ip, ip, ip]),
            "fv2d_batch_set_grid_mode": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_batch_usage": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong)]),
            "fv2d_batch_set_kernel_timing": (ctypes.c_int, [vp, ctypes.c_int]),
            "fv2d_batch_kernel_times": (ctypes.c_int, [vp, dp, ip]),
            "fv2d_batch_stream": (vp, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def _check(rc, h=None):
    if rc != OK:
        msg = library().fv2d_last_error(h)
        raise Fv2dError(rc, msg.decode() if msg else "")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def read_inputs(path: str) -> Case:
    cs = Case()
    _check(library().fv2d_read_inputs(path.encode(), ctypes.byref(cs)))
    return cs


def read_grid(path: str):
    """Parse a grid_file.in (C++ parser): (x, y, face_point1, face_point2, face_cell1, face_cell2,
    num_cells), ids 1-based as in the file."""
    lib = library()
    npt, nf, nc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    px, py = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)()
    pi = [ctypes.POINTER(ctypes.c_int)() for _ in range(4)]
    _check(lib.fv2d_read_grid(path.encode(), ctypes.byref(npt), ctypes.byref(nf), ctypes.byref(nc), ctypes.byref(px),
                              ctypes.byref(py), *[ctypes.byref(p) for p in pi]))
    try:
        x = np.ctypeslib.as_array(px, shape=(npt.value,)).copy()
        y = np.ctypeslib.as_array(py, shape=(npt.value,)).copy()
        ids = [np.ctypeslib.as_array(p, shape=(nf.value,)).copy() for p in pi]
    finally:
        for p in [px, py] + pi:
            lib.fv2d_free(ctypes.cast(p, ctypes.c_void_p))
    return (x, y, *ids, nc.value)


def write_grid(path: str, grid):
    """Write `grid` (x, y, fp1, fp2, fc1, fc2 1-based, num_cells) as a grid_file.in (C++ writer,
    17 significant digits)."""
    d = _Desc(grid)
    _check(library().fv2d_write_grid(path.encode(), ctypes.byref(d.desc)))


def read_restart(path: str, num_cells: int):
    """(iteration, q[4, num_cells]) from a restart_sol.dat-format file."""
    q = np.zeros(4 * num_cells, np.float64)
    ndx = ctypes.c_int()
    _check(library().fv2d_read_restart(path.encode(), int(num_cells), ctypes.byref(ndx), _dp(q)))
    return ndx.value, q.reshape(4, num_cells)


def case_from_dict(c: dict) -> Case:
    """Case from the keys of meshgen.write_input (string options as input.in spells them)."""
    lim = {"NONE": 0, "MINMOD": 1, "SQUEEZE": 2}[c["limiter"]]
    cs = Case()
    cs.order = int(c["solution_poly_order"]) + 1
    cs.nmax = int(c.get("nmax", 0)); cs.monitor_step = int(c.get("monitor_step", 0))
    cs.output_step = int(c.get("output_step", 0)); cs.restart = int(c.get("restart", 0))
    cs.eqn = 1 if c["eqn"] == "EULER" else 2
    cs.flux_solver = 1 if c.get("flux_solver", "RUSANOV") == "RUSANOV" else 2
    cs.limiter = lim
    cs.time_type = 1 if c["time_step_type"] == "GLOBAL" else 2
    cs.time_scheme = 2
    cs.bc1, cs.bc2 = BC[c["BC1"]], BC[c["BC2"]]
    cs.cfl = float(c["CFL"])
    for k in ("gamma", "R", "mu", "Pr", "P", "rho", "u", "v"):
        setattr(cs, k, float(c[k]))
    cs.length = float(c.get("length", 1.0))
    cs.grid_file = str(c.get("grid_file", "")).encode()[:4095]
    return cs


class _Desc:
    """Keeps the numpy arrays of a mesh descriptor alive."""

    def __init__(self, grid):
        self.x = np.ascontiguousarray(grid.x, dtype=np.float64)
        self.y = np.ascontiguousarray(grid.y, dtype=np.float64)
        self.ints = [np.ascontiguousarray(a, dtype=np.int32) for a in (grid.fp1, grid.fp2, grid.fc1, grid.fc2)]
        self.desc = MeshDesc(grid.num_points, grid.num_faces, grid.num_cells, _dp(self.x), _dp(self.y),
                             *[_ip(a) for a in self.ints])


class HostMesh:
    """Host-only mesh build (connectivity, geometry, renumbering); needs no GPU."""

    def __init__(self, grid, case: Case):
        lib = library()
        self._d = _Desc(grid)
        h = ctypes.c_void_p()
        _check(lib.fv2d_mesh_build(ctypes.byref(self._d.desc), ctypes.byref(case), ctypes.byref(h)))
        self.h = h
        s = np.zeros(8, np.int32)
        _check(lib.fv2d_mesh_sizes(self.h, _ip(s)))
        self.sizes = [int(v) for v in s]
        self.np, self.nf, self.nc = self.sizes[:3]

    def geom(self, name: str) -> np.ndarray:
        fid = GEOM[name]
        n = self.nf if fid < 40 else self.nc if fid < 50 else self.sizes[6]
        out = np.empty(n, np.float64)
        _check(library().fv2d_mesh_get(self.h, fid, _dp(out)))
        return out

    def tiles(self) -> dict:
        """The FP32 engine's tile layout of this mesh (checked; host only)."""
        o = (ctypes.c_longlong * 8)()
        _check(library().fv2d_mesh_tiles(self.h, o))
        keys = ("tiles", "record_words", "records", "csr_words", "halo_ids", "flux_records", "ring1", "ring2")
        return dict(zip(keys, [int(v) for v in o]))

    def permutation(self, kind: int) -> np.ndarray:
        out = np.empty(self.nc if kind == 0 else self.nf, np.int32)
        _check(library().fv2d_mesh_permutation(self.h, kind, _ip(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            library().fv2d_mesh_free(self.h)
            self.h = None

    __del__ = close


class Solver:
    """One resident solve on the GPU (a handle of the C ABI)."""

    def __init__(self, grid=None, case: Case | dict | None = None, precision: int = FP64, input_file: str | None = None):
        lib = library()
        h = ctypes.c_void_p()
        if input_file is not None:
            _check(lib.fv2d_create_from_files(input_file.encode(), precision, ctypes.byref(h)))
        else:
            if isinstance(case, dict):
                case = case_from_dict(case)
            d = _Desc(grid)
            _check(lib.fv2d_create(ctypes.byref(d.desc), ctypes.byref(case), precision, ctypes.byref(h)))
        self.h = h
        self.precision = precision
        s = self.sizes()
        self.np, self.nf, self.nc = s[:3]

    def close(self):
        if getattr(self, "h", None):
            library().fv2d_destroy(self.h)
            self.h = None

    __del__ = close

    def sizes(self):
        s = np.zeros(8, np.int32)
        _check(library().fv2d_sizes(self.h, _ip(s)), self.h)
        return [int(v) for v in s]

    def step(self, iterations: int = 1):
        _check(library().fv2d_step(self.h, iterations), self.h)

    def stage(self, n: int = 1):
        for _ in range(n):
            _check(library().fv2d_stage(self.h), self.h)

    def synchronize(self):
        _check(library().fv2d_synchronize(self.h), self.h)

    def set_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.size == 4 * self.nc
        _check(library().fv2d_set_state(self.h, _dp(q)), self.h)

    def load_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.size == 4 * self.nc
        _check(library().fv2d_load_state(self.h, _dp(q)), self.h)

    def get_state(self, out=None):
        out = np.empty(4 * self.nc, np.float64) if out is None else out
        _check(library().fv2d_get_state(self.h, _dp(out)), self.h)
        return out

    def get(self, field: int):
        n = {F_QBAR: 4, F_QSTAR: 4, F_RES: 4, F_DT: 1, F_QBAR_GRAD: 8, F_QSTAR_GRAD: 8}.get(field)
        if n is None:
            n = 1
            length = self.nf if field < 40 else self.nc
        else:
            length = n * self.nc
        out = np.empty(length, np.float64)
        _check(library().fv2d_get_field(self.h, field, _dp(out)), self.h)
        return out

    def residual_norm(self):
        out = np.zeros(4, np.float64)
        _check(library().fv2d_residual_norm(self.h, _dp(out)), self.h)
        return out

    def save(self, ndx: int):
        """Monitor / Tecplot output of iteration `ndx` under ./sol (the reference's save())."""
        _check(library().fv2d_save(self.h, int(ndx)), self.h)

    def post(self, ndx: int):
        """./sol/restart_sol.dat for iteration `ndx` (the reference's post())."""
        _check(library().fv2d_post(self.h, int(ndx)), self.h)

    def write_restart(self, path: str, ndx: int, digits: int = 17):
        """Checkpoint Qbar in the restart-file layout (17 digits: exact round trip)."""
        _check(library().fv2d_write_restart(self.h, path.encode(), int(ndx), int(digits)), self.h)

    def write_history_headers(self):
        _check(library().fv2d_write_history_headers(self.h), self.h)

    def write_mesh_files(self):
        """./mesh/cell_data.dat and ./mesh/face_data.dat."""
        _check(library().fv2d_write_mesh_files(self.h), self.h)

    def set_store_residual(self, every: bool):
        _check(library().fv2d_set_store_residual(self.h, int(every)), self.h)

    def set_graphs(self, enable: bool):
        _check(library().fv2d_set_graphs(self.h, int(enable)), self.h)

    def set_kernel_timing(self, enable: bool):
        _check(library().fv2d_set_kernel_timing(self.h, int(enable)), self.h)

    def kernel_times(self):
        names = ctypes.create_string_buffer(512)
        ms = np.zeros(16, np.float64)
        ln = np.zeros(16, np.int32)
        n = ctypes.c_int()
        _check(library().fv2d_kernel_times(self.h, names, 512, _dp(ms), _ip(ln), 16, ctypes.byref(n)), self.h)
        keys = names.value.decode().split(",")
        return {k: (float(ms[i]), int(ln[i])) for i, k in enumerate(keys[: n.value])}

    def stream(self) -> int:
        return int(library().fv2d_stream(self.h) or 0)

    def device_bytes(self) -> int:
        return int(library().fv2d_device_bytes(self.h))


class Batch:
    """Many independent solves advanced together on one GPU (C ABI fv2d_batch_*)."""

    def __init__(self, max_cells: int, max_faces: int, max_solves: int, precision: int = FP32):
        lib = library()
        h = ctypes.c_void_p()
        _check(lib.fv2d_batch_create(max_cells, max_faces, max_solves, precision, ctypes.byref(h)))
        self.h = h
        self.precision = precision
        self.cells = {}

    def close(self):
        if getattr(self, "h", None):
            library().fv2d_batch_destroy(self.h)
            self.h = None

    __del__ = close

    @staticmethod
    def footprint(grid, precision: int = FP32) -> int:
        d = _Desc(grid)
        out = ctypes.c_longlong()
        _check(library().fv2d_batch_footprint(ctypes.byref(d.desc), precision, ctypes.byref(out)))
        return int(out.value)

    def add(self, grid, case) -> int:
        if isinstance(case, dict):
            case = case_from_dict(case)
        d = _Desc(grid)
        sid = ctypes.c_int()
        _check(library().fv2d_batch_add(self.h, ctypes.byref(d.desc), ctypes.byref(case), ctypes.byref(sid)))
        self.cells[sid.value] = grid.num_cells
        return sid.value

    def add_mesh(self, host_mesh, case) -> int:
        """Admit a solve on a prebuilt HostMesh (built with the same BC codes as `case`)."""
        if isinstance(case, dict):
            case = case_from_dict(case)
        sid = ctypes.c_int()
        _check(library().fv2d_batch_add_mesh(self.h, host_mesh.h, ctypes.byref(case), ctypes.byref(sid)))
        self.cells[sid.value] = host_mesh.nc
        return sid.value

    def remove(self, sid: int):
        _check(library().fv2d_batch_remove(self.h, sid))
        self.cells.pop(sid, None)

    def step(self, iterations: int = 1):
        _check(library().fv2d_batch_step(self.h, iterations))

    def synchronize(self):
        _check(library().fv2d_batch_synchronize(self.h))

    def norms(self):
        """{solve id: (norms[4], iterations)} for every active solve."""
        mx = max(1, len(self.cells))
        ids = np.zeros(mx, np.int32)
        nr = np.zeros(4 * mx, np.float64)
        it = np.zeros(mx, np.int32)
        n = ctypes.c_int()
        _check(library().fv2d_batch_norms(self.h, _ip(ids), _dp(nr), _ip(it), mx, ctypes.byref(n)))
        return {int(ids[i]): (nr[4 * i:4 * i + 4].copy(), int(it[i])) for i in range(n.value)}

    def get_state(self, sid: int):
        out = np.empty(4 * self.cells[sid], np.float64)
        _check(library().fv2d_batch_get_state(self.h, sid, _dp(out)))
        return out

    def set_tuning(self, block: int, tile_mult=(1, 2, 4), bucket_edges=(16384, 131072)):
        tm = np.asarray(tile_mult, np.int32)
        be = np.asarray(bucket_edges, np.int32)
        _check(library().fv2d_batch_set_tuning(self.h, block, _ip(tm), _ip(be)))

    def set_grid_mode(self, full_grid: bool):
        _check(library().fv2d_batch_set_grid_mode(self.h, int(full_grid)))

    def get_tuning(self):
        b = ctypes.c_int()
        tm = np.zeros(3, np.int32)
        be = np.zeros(2, np.int32)
        _check(library().fv2d_batch_get_tuning(self.h, ctypes.byref(b), _ip(tm), _ip(be)))
        return int(b.value), tuple(int(x) for x in tm), tuple(int(x) for x in be)

    def usage(self):
        """Arena use.  FP64: cells, faces, incidences; FP32 (tile layout): cells, face records and
        csr words, reported under the same keys."""
        o = (ctypes.c_longlong * 8)()
        _check(library().fv2d_batch_usage(self.h, o))
        keys = ("cells_used", "cells_cap", "faces_used", "faces_cap", "incs_used", "incs_cap", "active", "bytes")
        return dict(zip(keys, [int(v) for v in o]))

    def set_kernel_timing(self, enable: bool):
        _check(library().fv2d_batch_set_kernel_timing(self.h, int(enable)))

    def kernel_times(self):
        ms = np.zeros(3, np.float64)
        ln = np.zeros(3, np.int32)
        _check(library().fv2d_batch_kernel_times(self.h, _dp(ms), _ip(ln)))
        names = (("kb_gradient", "kb_face", "kb_update") if self.precision == FP64
                 else ("k_tstage_1", "k_tstage_2", "k_tstage_3"))   # FP32: the fused kernel of each RK stage
        return {k: (float(ms[i]), int(ln[i])) for i, k in enumerate(names)}

    def stream(self) -> int:
        return int(library().fv2d_batch_stream(self.h) or 0)
