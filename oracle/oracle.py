"""ctypes binding of the two CPU checkers -- TEST INFRASTRUCTURE ONLY.

``Oracle("port", ...)`` loads oracle/build/libfv2d_oracle.so (the CPU restatement);
``Oracle("ref", ...)`` loads oracle/_ref/libfv2d_ref.so (the reference's own sources, only
available where the reference tree was present at build time).  Only tests, the smoke check and
the CPU-baseline leg of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "build", "libfv2d_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfv2d_ref.so")

# field ids (fv2d_oracle.h)
QBAR, QSTAR, RES, DT, QBAR_GRAD, QSTAR_GRAD, QF1, QF2, VNC, QBAR_PRIM = range(10)
GEOM_FACE = dict(area=20, nx=21, ny=22, fcx=23, fcy=24, c1dx=25, c1dy=26, c2dx=27, c2dy=28,
                 dxj=29, dyj=30, dist=31, lx=32, ly=33, mx=34, my=35)
GEOM_CELL = dict(vol=40, ccx=41, ccy=42, Ixx=43, Iyy=44, Ixy=45, delta=46)
GEOM_BC = dict(bccx=50, bccy=51)
I_FC1, I_FC2, I_FP1, I_FP2, I_CFC, I_BCF = range(6)


class FvoCase(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("eqn", ctypes.c_int), ("flux_solver", ctypes.c_int),
                ("limiter", ctypes.c_int), ("time_type", ctypes.c_int), ("time_scheme", ctypes.c_int),
                ("bc1", ctypes.c_int), ("bc2", ctypes.c_int), ("cfl", ctypes.c_double),
                ("gamma", ctypes.c_double), ("R", ctypes.c_double), ("mu", ctypes.c_double),
                ("Pr", ctypes.c_double), ("P", ctypes.c_double), ("rho", ctypes.c_double),
                ("u", ctypes.c_double), ("v", ctypes.c_double)]


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Compile the checkers (make -C oracle); the reference part only where its tree exists."""
    env = dict(os.environ)
    if ref_dir:
        env["REF"] = ref_dir
    out = subprocess.run(["make", "-C", HERE, "all"], env=env, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_LIBS: dict = {}


def _lib(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path = PORT_LIB if kind == "port" else REF_LIB
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = ctypes.CDLL(path)
    p = "fvo_" if kind == "port" else "fvr_"
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    fns = {
        "open": (vp, [ctypes.c_char_p]),
        "close": (None, [vp]),
        "sizes": (None, [vp, ip]),
        "stage": (None, [vp]),
        "iterate": (None, [vp, ctypes.c_int]),
        "get": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "get_int": (ctypes.c_int, [vp, ctypes.c_int, ip]),
        "set_state": (None, [vp, dp]),
        "time_iterations": (ctypes.c_double, [vp, ctypes.c_int]),
    }
    if kind == "port":
        fns["open_arrays"] = (vp, [ctypes.POINTER(FvoCase), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   dp, dp, ip, ip, ip, ip])
    table = {}
    for name, (res, args) in fns.items():
        f = getattr(lib, p + name)
        f.restype = res
        f.argtypes = args
        table[name] = f
    _LIBS[kind] = table
    return table


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def case_struct(c: dict) -> FvoCase:
    lim = {"NONE": 0, "MINMOD": 1, "SQUEEZE": 2}[c["limiter"]]
    codes = {"FREESTREAM": -1, "SLIP_WALL": -2, "EXTRAPOLATION": -3, "NO_SLIP_WALL": -4}
    flux = 1 if c.get("flux_solver", "RUSANOV") == "RUSANOV" else 2
    return FvoCase(int(c["solution_poly_order"]) + 1, 1 if c["eqn"] == "EULER" else 2, flux, lim,
                   1 if c["time_step_type"] == "GLOBAL" else 2, 2, codes[c["BC1"]], codes[c["BC2"]],
                   float(c["CFL"]), float(c["gamma"]), float(c["R"]), float(c["mu"]), float(c["Pr"]),
                   float(c["P"]), float(c["rho"]), float(c["u"]), float(c["v"]))


class Oracle:
    """One solver instance of either checker."""

    def __init__(self, kind: str, input_file: str | None = None, grid=None, case: dict | None = None):
        self.kind = kind
        self.f = _lib(kind)
        if input_file is not None:
            self.h = self.f["open"](input_file.encode())
        else:
            assert kind == "port" and grid is not None and case is not None
            cs = case_struct(case)
            self._keep = [np.ascontiguousarray(a) for a in
                          (grid.x, grid.y, grid.fp1, grid.fp2, grid.fc1, grid.fc2)]
            x, y = (np.ascontiguousarray(a, dtype=np.float64) for a in (grid.x, grid.y))
            ints = [np.ascontiguousarray(a, dtype=np.int32) for a in (grid.fp1, grid.fp2, grid.fc1, grid.fc2)]
            self._keep = [x, y] + ints
            self.h = self.f["open_arrays"](ctypes.byref(cs), grid.num_points, grid.num_faces, grid.num_cells,
                                           _dp(x), _dp(y), *[_ip(a) for a in ints])
        if not self.h:
            raise RuntimeError(f"oracle ({kind}) failed to open the case")
        s = self.sizes()
        self.np, self.nf, self.nc = s[0], s[1], s[2]

    def close(self):
        if getattr(self, "h", None):
            self.f["close"](self.h)
            self.h = None

    __del__ = close

    def sizes(self):
        out = np.zeros(8, np.int32)
        self.f["sizes"](self.h, _ip(out))
        return [int(v) for v in out]

    def stage(self, n: int = 1):
        for _ in range(n):
            self.f["stage"](self.h)

    def iterate(self, n: int = 1):
        self.f["iterate"](self.h, n)

    def time_iterations(self, n: int) -> float:
        return float(self.f["time_iterations"](self.h, n))

    def _len(self, field: int) -> int:
        if field in (QBAR, QSTAR, RES, QBAR_PRIM):
            return 4 * self.nc
        if field in (QBAR_GRAD, QSTAR_GRAD):
            return 8 * self.nc
        if field == DT:
            return self.nc
        if field in (QF1, QF2):
            return 4 * self.nf
        if field == VNC:
            return 2 * self.nf
        if 20 <= field < 40:
            return self.nf
        if 40 <= field < 50:
            return self.nc
        return self.sizes()[6]

    def get(self, field: int) -> np.ndarray:
        out = np.empty(self._len(field), np.float64)
        n = self.f["get"](self.h, field, _dp(out))
        if n < 0:
            raise KeyError(field)
        return out[:n]

    def geom(self, name: str) -> np.ndarray:
        fid = GEOM_FACE.get(name) or GEOM_CELL.get(name) or GEOM_BC.get(name)
        return self.get(fid)

    def get_int(self, field: int) -> np.ndarray:
        n = {I_FC1: self.nf, I_FC2: self.nf, I_FP1: self.nf, I_FP2: self.nf, I_CFC: self.nc,
             I_BCF: self.sizes()[6]}[field]
        out = np.empty(n, np.int32)
        self.f["get_int"](self.h, field, _ip(out))
        return out

    def set_state(self, q: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.size == 4 * self.nc
        self.f["set_state"](self.h, _dp(q))
