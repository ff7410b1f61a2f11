"""The FP64 engine's shared-reciprocal division (two Markstein corrections) must round exactly
like IEEE division: checked bit for bit on device-generated operands, including mantissas near
all-ones / near powers of two, signed operands and signed-zero dividends."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def helper(tmp_path_factory, pkg):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("divcheck") / "libdivcheck.so")
    cmd = [nvcc, "-std=c++17", "-O3", "-fmad=false", "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
           "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "cfd-2d-ns-fv_gb300", "csrc"),
           os.path.join(HERE, "gpu_helpers", "div_check.cu"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = ctypes.CDLL(out)
    lib.div_check.restype = ctypes.c_int
    lib.div_check.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_double)]
    return lib


@pytest.mark.parametrize("elo,ehi,ma,mb", [
    (-60, 60, 0, 0),      # random mantissas, wide exponents
    (-30, 30, 0, 1),      # divisor mantissa near all ones
    (-30, 30, 1, 1),
    (-30, 30, 2, 0),      # dividend near a power of two
    (-30, 30, 0, 2),      # divisor near a power of two
    (-20, 20, 1, 2),
    (-3, 20, 0, 0),       # the solver's range (densities, momenta, energies, volumes)
    (-30, 30, 3, 0),      # signed-zero dividend: +-0 / b keeps the sign rule of IEEE division
])
def test_shared_reciprocal_division_is_correctly_rounded(helper, elo, ehi, ma, mb):
    bad = ctypes.c_ulonglong()
    ex = (ctypes.c_double * 4)()
    n = 1 << 26
    for seed in (1, 2):
        rc = helper.div_check(n, seed * 7919 + elo * 31 + ma * 3 + mb, elo, ehi, ma, mb, ctypes.byref(bad), ex)
        assert rc == 0
        assert bad.value == 0, f"{bad.value} mismatches, e.g. a={ex[0]!r} b={ex[1]!r} got {ex[2]!r} want {ex[3]!r}"
