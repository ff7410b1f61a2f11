"""The solution output files (mesh/cell_data.dat, mesh/face_data.dat, sol/output.dat,
sol/res_history.dat, sol/tec_sol*.dat, sol/tec_surf*.dat, sol/restart_sol.dat) against the files the
REFERENCE program wrote on the same cases (tests/golden/cli/*.npz, made by make_cli_golden.py).

CPU: the library's host writers driven by the oracle port (tests/cpu_helpers/cli_oracle.cpp); and the
     reference's own src/base/main.cpp linked with the reference-signature shim
     (shim/ssp_rk3_gpu.cpp) over the oracle-backed ABI stub (oracle/abi_oracle_stub.cpp), built by
     `make -C oracle shim` where the reference tree exists.
GPU: the shipped command-line driver lib/fv2d_gpu (FP64), whose state comes from the GPU engine.
Both must reproduce every byte but the undefined last-row tau fields of tec_surf (cli_check.masked).
"""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

import cli_check
from conftest import ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, "golden", "cli", "*.npz")))
CSRC = os.path.join(ROOT, "cfd-2d-ns-fv_gb300", "csrc")


def test_cases_present():
    names = [os.path.basename(c) for c in CASES]
    assert "ch16_euler_order0_restart.npz" in names and len(names) >= 5


def test_mask_only_drops_last_row_tau():
    data = b"TITLE\n1 2 3 4 5 6 7 8\n9 10 11 12 13 14 15 16\n"
    assert cli_check.masked("sol/tec_surf_6.dat", data) == b"TITLE\n1 2 3 4 5 6 7 8\n9 10 11 12 13 14\n"
    assert cli_check.masked("sol/tec_sol_6.dat", data) == data


@pytest.fixture(scope="module")
def oracle_cli(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("cli") / "cli_oracle")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
           "-I", os.path.join(ROOT, "oracle"), os.path.join(HERE, "cpu_helpers", "cli_oracle.cpp"),
           os.path.join(CSRC, "fv2d_host.cpp"), os.path.join(CSRC, "fv2d_output.cpp"),
           os.path.join(ROOT, "oracle", "fv2d_oracle.cpp"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    return out


@pytest.mark.parametrize("case", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_writers_match_reference_files(oracle_cli, case, tmp_path):
    assert cli_check.run_case([oracle_cli], case, str(tmp_path)) == []


@pytest.fixture(scope="module")
def shim_program():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "shim"], check=True, capture_output=True)
    prog = os.path.join(ROOT, "oracle", "_ref", "fv2d_ref_shim_oracle")
    if not os.path.exists(prog):
        pytest.skip("reference tree not present: the reference main cannot be built here")
    return prog


@pytest.mark.parametrize("case", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_reference_main_through_shim(shim_program, case, tmp_path):
    assert cli_check.run_case([shim_program], case, str(tmp_path)) == []


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_cli_matches_reference_files(pkg, case, tmp_path):
    prog = pkg.build.CLI
    assert os.path.exists(prog), "lib/fv2d_gpu not built"
    assert cli_check.run_case([prog], case, str(tmp_path)) == []


def test_reference_main_links_against_gpu_library(pkg, shim_program):
    """The link-time swap: the reference's main.cpp + shim resolve every symbol in libfv2d_gb300.so."""
    assert os.path.exists(pkg.build.LIB)
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "shim"], check=True, capture_output=True)
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "fv2d_ref_shim_gpu"))


@pytest.fixture(scope="module")
def oracle_cli_sanitized(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("cli_san") / "cli_oracle_san")
    cmd = [cxx, "-O1", "-g", "-std=c++17", "-ffp-contract=off", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", os.path.join(ROOT, "oracle"),
           os.path.join(HERE, "cpu_helpers", "cli_oracle.cpp"), os.path.join(CSRC, "fv2d_host.cpp"),
           os.path.join(CSRC, "fv2d_output.cpp"), os.path.join(ROOT, "oracle", "fv2d_oracle.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime unavailable: " + r.stderr[-300:])
    return out


@pytest.mark.parametrize("case", [c for c in CASES if "airfoil" not in c], ids=lambda p: os.path.basename(p)[:-4])
def test_host_code_clean_under_asan_ubsan(oracle_cli_sanitized, case, tmp_path):
    """The library's host code (input/grid parsing, connectivity, geometry, renumbering, output
    writers) has no memory errors or undefined behaviour on the golden cases (ASan + UBSan)."""
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1")
    assert cli_check.run_case([oracle_cli_sanitized], case, str(tmp_path), env=env) == []


@pytest.mark.gpu
def test_gpu_cli_fp32_tracks_fp64(pkg, tmp_path):
    """lib/fv2d_gpu --fp32 writes the same files from the FP32 engine; its restart state stays within
    FP32 round-off of the FP64 run on each quantity's scale (the restart file's 6 significant digits
    bound the comparison)."""
    case = next(c for c in CASES if os.path.basename(c).startswith("ch16_euler_sq_global"))
    prog = pkg.build.CLI
    states = {}
    for flag in ("", "--fp32"):
        work = tmp_path / (flag.strip("-") or "fp64")
        argv = [prog] + ([flag] if flag else [])
        grid_txt, inputs, files = cli_check.load_case(case)
        os.makedirs(work, exist_ok=True)
        (work / "grid_file.in").write_text(grid_txt)
        (work / "input.in").write_text(inputs[0])
        r = subprocess.run(argv, cwd=work, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-500:]
        got = sorted(f"{s}/{n}" for s in ("sol", "mesh") for n in os.listdir(work / s))
        assert got == sorted(files)
        rows = (work / "sol" / "restart_sol.dat").read_text().split("\n")[1:]
        states[flag] = np.array([[float(x) for x in ln.split()] for ln in rows if ln.strip()])
    a, b = states[""], states["--fp32"]
    assert a.shape == b.shape
    # error on each quantity's own scale: density, momentum (both components together), energy
    mom = np.max(np.abs(a[:, 1:3]))
    scale = np.array([np.max(np.abs(a[:, 0])), mom, mom, np.max(np.abs(a[:, 3]))])
    assert np.max(np.abs(b - a) / scale) < 2e-5
