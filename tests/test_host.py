"""Host side of the library (no GPU): C-ABI exports, input.in and grid parsing, connectivity, BC
tagging, geometry (bit-exact against the reference) and the renumbering."""
import ctypes
import hashlib
import json
import os
import re
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, bits_equal, golden_names

CASES = golden_names()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def header_functions():
    txt = open(os.path.join(ROOT, "include", "fv2d_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fv2d_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.build.LIB)
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(pkg.fv2d.EXPORTS) == names


def test_create_without_gpu_fails_loudly(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = pkg.meshgen.channel_bump_quads(8, 4)
    with pytest.raises(pkg.Fv2dError) as e:
        pkg.Solver(g, dict(pkg.meshgen.DEFAULT_CASE))
    assert e.value.code == 8


def load(name, pkg):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    grid = pkg.meshgen.Grid(z["x"], z["y"], z["fp1"], z["fp2"], z["fc1"], z["fc2"], int(z["num_cells"]), name)
    return z, grid, json.loads(str(z["case_json"]))


@pytest.mark.parametrize("name", CASES)
def test_geometry_bit_exact_vs_reference(name, pkg):
    z, grid, case = load(name, pkg)
    hm = pkg.HostMesh(grid, pkg.case_from_dict(case))
    geo = json.loads(str(z["geom_hashes"]))
    interleaved = name.startswith("simple")
    for g, h in geo.items():
        if interleaved and g in ("dist", "lx", "ly"):
            continue
        assert sha(hm.geom(g)) == h, g
    assert hm.sizes[:7] == [int(v) for v in z["sizes"][:7]]


def test_geometry_matches_oracle_on_polygons(pkg, orc):
    g = pkg.meshgen.voronoi_cylinder(5000, seed=2, box=(6.0, 3.0), h_wall=0.01, h_far=0.08)
    case = dict(pkg.meshgen.DEFAULT_CASE, eqn="NS", mu=0.01, BC1="NO_SLIP_WALL", BC2="FREESTREAM")
    hm = pkg.HostMesh(g, pkg.case_from_dict(case))
    port = orc.Oracle("port", grid=g, case=case)
    for name in ("area", "nx", "ny", "c1dx", "c1dy", "c2dx", "c2dy", "dxj", "dyj", "dist", "lx", "ly", "mx", "my",
                 "vol", "ccx", "ccy", "Ixx", "Iyy", "Ixy", "delta", "bccx", "bccy"):
        assert bits_equal(hm.geom(name), port.geom(name)), name
    assert hm.sizes[7] == max(g.sides_histogram())


def test_renumbering_is_a_permutation(pkg):
    g = pkg.meshgen.voronoi_bump_channel(4000, seed=1)
    hm = pkg.HostMesh(g, pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE)))
    for kind, n in ((0, g.num_cells), (1, g.num_faces)):
        p = hm.permutation(kind)
        assert np.array_equal(np.sort(p), np.arange(n))
    # Hilbert order keeps neighbours close: the median |new c1 - new c2| is small
    inv = np.empty(g.num_cells, np.int64)
    inv[hm.permutation(0)] = np.arange(g.num_cells)
    inter = g.fc2 > 0
    gap = np.abs(inv[g.fc1[inter] - 1] - inv[g.fc2[inter] - 1])
    assert np.median(gap) < 0.01 * g.num_cells


def test_read_inputs_matches_reference_parser(pkg, orc, tmp_path):
    p = str(tmp_path / "input.in")
    c = pkg.meshgen.write_input(p, eqn="NS", mu=0.04168601, limiter="NONE", time_step_type="LOCAL", CFL=1.0,
                                BC1="NO_SLIP_WALL", BC2="FREESTREAM", nmax=10000, monitor_step=50, output_step=1000,
                                grid_file="../../grids/grid_file.in")
    cs = pkg.read_inputs(p)
    assert (cs.order, cs.nmax, cs.monitor_step, cs.output_step, cs.restart) == (2, 10000, 50, 1000, 0)
    assert (cs.eqn, cs.flux_solver, cs.limiter, cs.time_type, cs.time_scheme) == (2, 1, 0, 2, 2)
    assert (cs.bc1, cs.bc2) == (-4, -1)
    assert cs.grid_file.decode() == "../../grids/grid_file.in"
    for k in ("gamma", "R", "mu", "Pr", "P", "rho", "u", "v"):
        assert getattr(cs, k) == float(c[k]), k
    assert cs.cfl == 1.0 and cs.length == 1.0


def test_read_inputs_section_order_free_and_errors(pkg, tmp_path):
    # sections may come in any order (read_inputs loops over 9 tokens); values map to codes
    p = tmp_path / "a.in"
    p.write_text("[BC]\n BC1 = SLIP_WALL\n BC2 = EXTRAPOLATION\n[limiter]\n limiter = MINMOD\n"
                 "[case]\n nmax = 5\n monitor_step = 1\n output_step = 2\n solution_poly_order = 0\n restart = 1\n"
                 "[grid]\n grid_file = g.in\n[equations]\n eqn = EULER\n flux_solver = ROE\n"
                 "[fluid]\n gamma = 1.3\n R = 200\n mu = 0\n Pr = 0.7\n[init]\n P = 1e5\n rho = 1\n u = 10\n v = 1\n"
                 "[time]\n time_scheme = SSP_RK2\n time_step_type = GLOBAL\n CFL = 0.5\n[report]\n length = 2\n")
    cs = pkg.read_inputs(str(p))
    assert (cs.bc1, cs.bc2, cs.limiter, cs.order, cs.restart, cs.flux_solver, cs.time_scheme) == (-2, -3, 1, 1, 1, 2, 1)
    with pytest.raises(pkg.Fv2dError) as e:
        pkg.read_inputs(str(tmp_path / "missing.in"))
    assert e.value.code == 2
    bad = tmp_path / "bad.in"
    bad.write_text("[case]\n nmax = abc\n")
    with pytest.raises(pkg.Fv2dError):
        pkg.read_inputs(str(bad))


def test_grid_reader_roundtrip(pkg, tmp_path):
    g = pkg.meshgen.voronoi_bump_channel(2000, seed=4)
    path = str(tmp_path / "g.in")
    pkg.meshgen.write_grid(path, g)
    lib = pkg.library()
    n = [ctypes.c_int() for _ in range(3)]
    ptrs = [ctypes.POINTER(ctypes.c_double)() for _ in range(2)] + [ctypes.POINTER(ctypes.c_int)() for _ in range(4)]
    lib.fv2d_read_grid.argtypes = None
    rc = lib.fv2d_read_grid(path.encode(), *[ctypes.byref(v) for v in n], *[ctypes.byref(p) for p in ptrs])
    assert rc == 0
    npt, nf, nc = (v.value for v in n)
    assert (npt, nf, nc) == (g.num_points, g.num_faces, g.num_cells)
    x = np.ctypeslib.as_array(ptrs[0], (npt,)).copy()
    fc2 = np.ctypeslib.as_array(ptrs[5], (nf,)).copy()
    assert bits_equal(x, g.x) and np.array_equal(fc2, g.fc2)
    for p in ptrs:
        lib.fv2d_free(ctypes.cast(p, ctypes.c_void_p))


def test_mesh_errors(pkg):
    g = pkg.meshgen.channel_bump_quads(8, 4)
    case = pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE))
    bad = pkg.meshgen.Grid(g.x, g.y, g.fp1, g.fp2, g.fc1.copy(), g.fc2, g.num_cells)
    bad.fc1[3] = g.num_cells + 5
    with pytest.raises(pkg.Fv2dError) as e:
        pkg.HostMesh(bad, case)
    assert e.value.code == 3
    # NO_SLIP_WALL faces must have ids below the cell count (the reference gradient reads cell `face id`)
    late = pkg.meshgen.Grid(g.x, g.y, g.fp1[::-1].copy(), g.fp2[::-1].copy(), g.fc1[::-1].copy(), g.fc2[::-1].copy(),
                            g.num_cells)
    ns = pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE, eqn="NS", BC1="NO_SLIP_WALL"))
    with pytest.raises(pkg.Fv2dError) as e:
        pkg.HostMesh(late, ns)
    assert e.value.code == 3
    for opts in (dict(solution_poly_order=2), dict(time_step_type="LOCAL", CFL=-1.0)):
        c = pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE, **opts))
        with pytest.raises(pkg.Fv2dError) as e:
            pkg.HostMesh(g, c)
        assert e.value.code == 4
    # ROE is accepted and run as the reference runs it (no inviscid flux routine, res.cpp:62-69)
    pkg.HostMesh(g, pkg.case_from_dict(dict(pkg.meshgen.DEFAULT_CASE, flux_solver="ROE"))).close()


def test_fp64_engine_is_built_without_fma_contraction():
    src = open(os.path.join(ROOT, "cfd-2d-ns-fv_gb300", "build.py")).read()
    assert re.search(r'"fv2d_fp64\.cu".*-fmad=false', src)


def test_fp64_division_by_three(tmp_path):
    """The face kernel's FP64 a/3 (one residual correction of RN(a RN(1/3))) equals IEEE a / 3 on
    random operands of every exponent and on quotients next to rounding midpoints."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "div3_check")
    here = os.path.dirname(os.path.abspath(__file__))
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(here, "cpu_helpers", "div3_check.cpp"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert "0 mismatches" in r.stdout


def test_parallel_host_copy(tmp_path):
    """The pooled host copy used by the staged host<->device transfers copies every byte."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = next((d for d in ("/usr/local/cuda/include",) if os.path.exists(os.path.join(d, "cuda_runtime.h"))), None)
    if cuda_inc is None:
        pytest.skip("no CUDA headers")
    exe = str(tmp_path / "copypool_check")
    here = os.path.dirname(os.path.abspath(__file__))
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", cuda_inc, "-I",
                    os.path.join(ROOT, "cfd-2d-ns-fv_gb300", "csrc"), os.path.join(here, "cpu_helpers", "copypool_check.cpp"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout


def test_native_grid_writer_and_reader(pkg, tmp_path):
    """fv2d_write_grid writes the same bytes as the numpy writer, and fv2d_read_grid returns the same
    doubles and ids (17-digit round trip)."""
    mg = pkg.meshgen
    g = mg.voronoi_bump_channel(3000, seed=11)
    a, b = str(tmp_path / "native.in"), str(tmp_path / "numpy.in")
    pkg.fv2d.write_grid(a, g)
    with open(b, "w") as fh:
        fh.write(f"{g.num_points} {g.num_faces} {g.num_cells}\n")
        np.savetxt(fh, np.column_stack([g.x, g.y]), fmt="%.17g")
        np.savetxt(fh, np.column_stack([g.fp1, g.fp2]), fmt="%d")
        np.savetxt(fh, np.column_stack([g.fc1, g.fc2]), fmt="%d")
    assert open(a, "rb").read() == open(b, "rb").read()
    x, y, fp1, fp2, fc1, fc2, nc = pkg.fv2d.read_grid(a)
    assert nc == g.num_cells
    assert bits_equal(x, g.x) and bits_equal(y, g.y)
    for u, v in ((fp1, g.fp1), (fp2, g.fp2), (fc1, g.fc1), (fc2, g.fc2)):
        np.testing.assert_array_equal(u, v)
    with pytest.raises(pkg.Fv2dError):
        pkg.fv2d.read_grid(str(tmp_path / "missing.in"))


def golden_grid(pkg, name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return pkg.meshgen.Grid(z["x"], z["y"], z["fp1"], z["fp2"], z["fc1"], z["fc2"], int(z["num_cells"]), name)


@pytest.mark.parametrize("kind", ["voronoi", "cylinder", "quads", "wheels", "airfoil", "tiny"])
def test_tile_layout_checks(pkg, kind):
    """The FP32 engine's tile layout: built and checked on the host (every index its stage kernels
    derive stays in range), with the duplication the design expects on Voronoi meshes."""
    from conftest import wheels_grid
    mg = pkg.meshgen
    g = {"voronoi": lambda: mg.voronoi_bump_channel(60000, seed=2),
         "cylinder": lambda: mg.voronoi_cylinder(12000, seed=0, box=(8.0, 4.0), h_wall=0.01, h_far=0.08),
         "quads": lambda: mg.channel_bump_quads(128, 64),
         "wheels": lambda: wheels_grid(pkg),
         "airfoil": lambda: golden_grid(pkg, "airfoil_ns_sq_local"),
         "tiny": lambda: mg.channel_bump_quads(4, 2)}[kind]()
    case = dict(mg.DEFAULT_CASE, eqn="NS", BC1="NO_SLIP_WALL", BC2="FREESTREAM")
    hm = pkg.HostMesh(g, pkg.case_from_dict(case))
    t = hm.tiles()
    assert t["tiles"] >= 1
    assert g.num_faces <= t["flux_records"] <= 2 * g.num_faces
    if kind == "voronoi":
        # compact 256-cell Hilbert blocks: 1.103 flux records per face, 0.317 ring-1 and 0.319 ring-2
        # cells per cell on this mesh (Morton blocks gave about 1.108, 0.34 and 0.36 on a similar
        # one); the bounds leave a small margin over the measured values
        assert t["flux_records"] < 1.115 * g.num_faces
        assert t["ring1"] < 0.335 * g.num_cells
        assert t["ring1"] + t["ring2"] < 0.68 * g.num_cells
    hm.close()
