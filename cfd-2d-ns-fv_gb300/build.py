"""Build recipe of the native library (no cmake): nvcc for sm_103a, g++ for the host mesh code.

Outputs (git-ignored, built in place on each machine):
    lib/libfv2d_gb300.so   the C-ABI library (include/fv2d_gpu.h)
    lib/fv2d_gpu           the fv2d-compatible command-line driver
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libfv2d_gb300.so")
CLI = os.path.join(LIBDIR, "fv2d_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _units():
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + ARCH
    host = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
    return [
        # (source, object, command prefix)
        ("fv2d_host.cpp", host),
        ("fv2d_tiles.cpp", host),
        ("fv2d_output.cpp", host),
        ("fv2d_api.cu", [nvcc] + common),
        # the FP64 engine must not contract a*b+c: bit-identical with the reference
        ("fv2d_fp64.cu", [nvcc] + common + ["-fmad=false"]),
        # the FP32 engine: a single solve and a batch run the same fused stage kernels, so FMA
        # contraction is allowed (both round alike); divisions and square roots use the
        # approximate (few-ulp) forms
        # FP32 engine: approximate division and square root, denormals flushed to zero (the flow's
        # FP32 values are far above FP32's normal range; norms are summed in FP64)
        ("fv2d_tiled.cu", [nvcc] + common + ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
        ("fv2d_noalloc.cu", [nvcc] + common + ["-fmad=false"]),
    ]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "fv2d_gpu.h"))
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src, cmd in _units():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(cmd + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for warn in ex.map(run, jobs):
            if verbose and warn.strip():
                print(warn)
    if force or jobs or _stale(LIB, objs):
        run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    cli_src = os.path.join(CSRC, "fv2d_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + headers)):
        run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", INCLUDE, cli_src, "-o", CLI, "-L", LIBDIR,
             "-lfv2d_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
