"""FP64 GPU path against the reference (golden fixtures, replayed byte for byte) and against the
oracle port on meshes the reference cannot read (7-9-sided cells).  All calls go through the
C ABI (ctypes)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_names, bits_equal, max_rel, wheels_grid

pytestmark = pytest.mark.gpu

CASES = golden_names()
LONG = golden_names(long=True)
TOL = 1e-12   # relative, per value: the FP64 path's parity bar (it is expected to be bit-exact)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def load(name, pkg):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    grid = pkg.meshgen.Grid(z["x"], z["y"], z["fp1"], z["fp2"], z["fc1"], z["fc2"], int(z["num_cells"]), name)
    return z, grid, json.loads(str(z["case_json"]))


def rel(a, b):
    return max_rel(a, b, floor=1e-30)


@pytest.mark.parametrize("name", CASES)
def test_fp64_reproduces_reference_every_stage(name, pkg, orc):
    z, grid, case = load(name, pkg)
    gpu = pkg.Solver(grid, case, precision=pkg.FP64)
    gpu.set_store_residual(True)
    port = orc.Oracle("port", grid=grid, case=case)
    if "restart_state" in z:
        gpu.set_state(z["restart_state"])
        port.set_state(z["restart_state"])
    hashes = json.loads(str(z["stage_hashes"]))
    for s, rec in enumerate(hashes):
        gpu.stage()
        port.stage()
        R, Q, dt = gpu.get(2), gpu.get(0), gpu.get(3)
        # within tolerance of the oracle (which itself reproduces the reference's bytes)
        assert rel(R, port.get(orc.RES)) <= TOL, f"stage {s}: residual"
        assert rel(Q, port.get(orc.QBAR)) <= TOL, f"stage {s}: Qbar"
        assert rel(dt, port.get(orc.DT)) <= TOL, f"stage {s}: dt"
        # and the reference's exact bytes
        assert sha(R) == rec["res"], f"stage {s}: residual not bit-identical (max rel {rel(R, port.get(orc.RES)):.2e})"
        assert sha(Q) == rec["qbar"], f"stage {s}: Qbar not bit-identical"
        assert sha(dt) == rec["dt"], f"stage {s}: dt not bit-identical"
        if "qstar" in rec:
            assert sha(gpu.get(1)) == rec["qstar"], f"stage {s}: Q* not bit-identical"
    assert bits_equal(gpu.get_state(), z["final_qbar"])
    gpu.close()


@pytest.mark.parametrize("name", LONG)
def test_fp64_full_run_reproduces_reference(name, pkg):
    """The plain FP64 method run as the reference's driver runs it (ssp_rk3() once per iteration,
    main.cpp:121-133; here fv2d_step, i.e. graph-replayed iterations): Qbar and the residual after
    1, 10, 100, 500 and 2000 iterations are the reference's exact bytes."""
    z, grid, case = load(name, pkg)
    gpu = pkg.Solver(grid, case, precision=pkg.FP64)
    done = 0
    for rec in json.loads(str(z["iter_hashes"])):
        gpu.step(rec["iter"] - done)
        done = rec["iter"]
        assert sha(gpu.get_state()) == rec["qbar"], f"Qbar not bit-identical after iteration {done}"
        assert sha(gpu.get(2)) == rec["res"], f"residual not bit-identical after iteration {done}"
    gpu.close()


def test_fp64_long_run_cylinder_vs_oracle(pkg, orc):
    """300 iterations of the benchmark's flow (NS cylinder of diameter 1, Re 100, Mach 0.2, Pr 0.72,
    no-slip cylinder, freestream box, squeeze, LOCAL dt at CFL 0.5) on a 12k-cell Voronoi mesh of an
    8 x 4 box with 4-8-sided cells, bit for bit against the oracle at iterations 1, 30 and 300: past
    the start-up transient, where the limiter's warp-shared quotient path is taken or left per warp
    as the flow settles."""
    mg = pkg.meshgen
    g = mg.voronoi_cylinder(12000, seed=0, box=(8.0, 4.0), h_wall=0.01, h_far=0.08)
    u = mg.mach_speed(0.2)
    case = dict(mg.DEFAULT_CASE, eqn="NS", mu=1.225 * u * 1.0 / 100.0, Pr=0.72, u=u, v=0.0, limiter="SQUEEZE",
                time_step_type="LOCAL", CFL=0.5, BC1="NO_SLIP_WALL", BC2="FREESTREAM", solution_poly_order=1)
    gpu = pkg.Solver(g, case, precision=pkg.FP64)
    port = orc.Oracle("port", grid=g, case=case)
    done = 0
    for n in (1, 30, 300):
        gpu.step(n - done)
        port.iterate(n - done)
        done = n
        assert bits_equal(gpu.get_state(), port.get(orc.QBAR)), f"Qbar after iteration {n}"
        assert bits_equal(gpu.get(2), port.get(orc.RES)), f"residual after iteration {n}"
        assert bits_equal(gpu.get(3), port.get(orc.DT)), f"dt after iteration {n}"
        assert bits_equal(gpu.get(4), port.get(orc.QBAR_GRAD)), f"Qbar gradient after iteration {n}"
    assert np.all(np.isfinite(gpu.get_state()))
    gpu.close()


@pytest.mark.parametrize("opts", [
    dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM"),
    dict(eqn="NS", mu=0.02, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.9, BC1="NO_SLIP_WALL", BC2="FREESTREAM"),
    dict(eqn="NS", mu=0.02, limiter="NONE", time_step_type="GLOBAL", CFL=0.5, BC1="NO_SLIP_WALL", BC2="EXTRAPOLATION"),
], ids=["euler_sq_global", "ns_sq_local", "ns_none_extrap"])
def test_fp64_polygonal_cells_vs_oracle(opts, pkg, orc):
    """Cylinder Voronoi mesh with 7-9-sided cells (beyond the reference's 6 face slots)."""
    g = pkg.meshgen.voronoi_cylinder(12000, seed=7, box=(8.0, 4.0), h_wall=0.01, h_far=0.08)
    assert max(g.sides_histogram()) >= 7
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.4), v=5.0, **opts)
    gpu = pkg.Solver(g, case, precision=pkg.FP64)
    gpu.set_store_residual(True)
    port = orc.Oracle("port", grid=g, case=case)
    for s in range(12):
        gpu.stage()
        port.stage()
        assert bits_equal(gpu.get(2), port.get(orc.RES)), f"stage {s}: residual"
        assert bits_equal(gpu.get(0), port.get(orc.QBAR)), f"stage {s}: Qbar"
        # the gradient kernel's own output (limited LSQ gradient of this stage's input) and dt
        if s % 3 == 0:
            assert bits_equal(gpu.get(4), port.get(orc.QBAR_GRAD)), f"stage {s}: Qbar gradient"
        else:
            assert bits_equal(gpu.get(5), port.get(orc.QSTAR_GRAD)), f"stage {s}: Q* gradient"
        assert bits_equal(gpu.get(3), port.get(orc.DT)), f"stage {s}: dt"
    gpu.close()


@pytest.mark.parametrize("opts", [
    dict(eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8, BC1="SLIP_WALL", BC2="FREESTREAM"),
    dict(eqn="NS", mu=0.02, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.5, BC1="NO_SLIP_WALL", BC2="FREESTREAM"),
], ids=["euler_sq_global", "ns_sq_local"])
def test_fp64_cells_beyond_16_faces_vs_oracle(opts, pkg, orc):
    """20-faced cells: the limiter's multi-chunk flag masks, and warps mixing them with 4-faced cells
    (the warp-shared limiter quotients are taken by whole warps only)."""
    g = wheels_grid(pkg)
    assert max(g.sides_histogram()) == 20
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.4), v=5.0, **opts)
    gpu = pkg.Solver(g, case, precision=pkg.FP64)
    gpu.set_store_residual(True)
    port = orc.Oracle("port", grid=g, case=case)
    for s in range(12):
        gpu.stage()
        port.stage()
        assert bits_equal(gpu.get(2), port.get(orc.RES)), f"stage {s}: residual"
        assert bits_equal(gpu.get(0), port.get(orc.QBAR)), f"stage {s}: Qbar"
        if s % 3 == 0:
            assert bits_equal(gpu.get(4), port.get(orc.QBAR_GRAD)), f"stage {s}: Qbar gradient"
        else:
            assert bits_equal(gpu.get(5), port.get(orc.QSTAR_GRAD)), f"stage {s}: Q* gradient"
        assert bits_equal(gpu.get(3), port.get(orc.DT)), f"stage {s}: dt"
    gpu.close()


def test_graph_replay_equals_eager(pkg):
    g = pkg.meshgen.voronoi_bump_channel(20000, seed=2)
    case = dict(pkg.meshgen.DEFAULT_CASE, eqn="NS", mu=0.01, limiter="SQUEEZE", time_step_type="LOCAL",
                BC1="NO_SLIP_WALL", BC2="FREESTREAM", u=pkg.meshgen.mach_speed(0.6))
    a = pkg.Solver(g, case)
    b = pkg.Solver(g, case)
    b.set_graphs(False)
    a.step(7)
    b.step(7)
    assert bits_equal(a.get_state(), b.get_state())
    assert bits_equal(a.get(2), b.get(2))
    np.testing.assert_array_equal(a.residual_norm(), b.residual_norm())


def test_pinned_and_pageable_transfers_agree(pkg):
    """State upload/download through page-locked buffers (direct DMA) and through ordinary arrays
    (pooled staging in 8 MB chunks; this state is ~11 MB) give the same bits."""
    import torch
    g = pkg.meshgen.voronoi_bump_channel(350000, seed=4)
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.6), time_step_type="LOCAL")
    a = pkg.Solver(g, case)
    b = pkg.Solver(g, case)
    a.step(2)
    b.step(2)
    pinned = torch.empty(4 * g.num_cells, dtype=torch.float64, pin_memory=True).numpy()
    a.get_state(pinned)
    pageable = b.get_state()
    assert pinned.nbytes > 8 << 20
    assert bits_equal(pinned, pageable)
    a.load_state(pinned)
    b.load_state(pageable)
    a.step(1)
    b.step(1)
    q3 = a.get_state()
    assert bits_equal(q3, b.get_state())
    # two uploads back to back through the reused staging buffer: the second one wins
    b.load_state(q3 * 1.01)
    b.load_state(q3)
    pinned[:] = q3
    a.load_state(pinned)
    a.step(1)
    b.step(1)
    assert bits_equal(a.get_state(), b.get_state())


def test_checkpoint_round_trip_is_exact(pkg, tmp_path):
    """fv2d_write_restart at 17 digits + fv2d_read_restart + fv2d_set_state restores Qbar bit for
    bit; the reference's 6-digit restart file (fv2d_post) differs from it (lossy, as in the reference)."""
    g = pkg.meshgen.voronoi_bump_channel(5000, seed=6)
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.6), time_step_type="LOCAL")
    s = pkg.Solver(g, case)
    s.step(5)
    q = s.get_state()
    path = str(tmp_path / "ckpt.dat")
    s.write_restart(path, 5, digits=17)
    ndx, q2 = pkg.fv2d.read_restart(path, g.num_cells)
    assert ndx == 5 and bits_equal(q2.ravel(), q)
    t = pkg.Solver(g, case)
    t.set_state(q2.ravel())
    assert bits_equal(t.get_state(), q)
    s.write_restart(str(tmp_path / "six.dat"), 5, digits=0)
    _, q6 = pkg.fv2d.read_restart(str(tmp_path / "six.dat"), g.num_cells)
    assert not bits_equal(q6.ravel(), q) and np.allclose(q6.ravel(), q, rtol=1e-5)


def test_step_equals_stages_and_norm(pkg, orc):
    g = pkg.meshgen.channel_bump_quads(64, 32)
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.5))
    a = pkg.Solver(g, case)
    b = pkg.Solver(g, case)
    a.step(5)
    b.stage(15)
    assert bits_equal(a.get_state(), b.get_state())
    port = orc.Oracle("port", grid=g, case=case)
    port.iterate(5)
    r = port.get(orc.RES).reshape(4, -1)
    ref_norm = np.sqrt((r * r).sum(axis=1))
    assert np.allclose(a.residual_norm(), ref_norm, rtol=1e-12, atol=0)


def test_restart_matches_oracle(pkg, orc):
    """set_state is the restart path: fresh face histories, primitives from the given state."""
    g = pkg.meshgen.voronoi_bump_channel(8000, seed=9)
    case = dict(pkg.meshgen.DEFAULT_CASE, u=pkg.meshgen.mach_speed(0.7), time_step_type="LOCAL")
    gpu = pkg.Solver(g, case)
    port = orc.Oracle("port", grid=g, case=case)
    gpu.step(3)
    port.iterate(3)
    q = gpu.get_state()
    assert bits_equal(q, port.get(orc.QBAR))
    gpu.set_state(q)
    port.set_state(q)
    gpu.step(2)
    port.iterate(2)
    assert bits_equal(gpu.get_state(), port.get(orc.QBAR))


def test_conservation_and_freestream(pkg):
    """sum(vol*R) equals minus the net boundary flux; a uniform flow through freestream-only
    boundaries stays uniform to round-off."""
    g = pkg.meshgen.voronoi_cylinder(10000, seed=3, box=(8.0, 4.0), h_wall=0.01, h_far=0.08)
    case = dict(pkg.meshgen.DEFAULT_CASE, eqn="EULER", limiter="SQUEEZE", BC1="FREESTREAM", BC2="FREESTREAM",
                u=pkg.meshgen.mach_speed(0.5))
    s = pkg.Solver(g, case)
    s.set_store_residual(True)
    s.step(3)
    q = s.get_state().reshape(4, -1)
    qinf = np.array([case["rho"], case["rho"] * case["u"], 0.0,
                     case["P"] / 0.4 + 0.5 * case["rho"] * case["u"] ** 2])
    for j in (0, 1, 3):
        assert np.max(np.abs(q[j] / qinf[j] - 1)) < 1e-9
    assert np.max(np.abs(q[2])) < 1e-9 * qinf[1]
    r = s.get(2).reshape(4, -1)
    vol = s.get(40)
    tot = (vol[None, :] * r).sum(axis=1)
    # with a uniform state every interior flux cancels pairwise: the volume-weighted total is round-off
    scale = np.abs(vol[None, :] * r).sum(axis=1) + 1e-300
    assert np.all(np.abs(tot) <= 1e-6 * np.maximum(scale, 1.0))


def test_bad_state_is_reported(pkg):
    g = pkg.meshgen.channel_bump_quads(16, 8)
    s = pkg.Solver(g, dict(pkg.meshgen.DEFAULT_CASE))
    q = s.get_state()
    q[: s.nc][5] = -1.0          # negative density in one cell
    s.set_state(q)
    s.step(1)
    with pytest.raises(pkg.Fv2dError) as e:
        s.synchronize()
    assert e.value.code == 7
