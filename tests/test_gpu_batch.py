"""Batched solves: each solve advances exactly as it would alone (bit for bit: the batch kernels
run the same per-element code), solves can join and leave between iterations, tile shapes do not
change results, and admission refuses what does not fit."""
import numpy as np
import pytest

from conftest import bits_equal, max_rel, wheels_grid

pytestmark = pytest.mark.gpu


def mix(pkg):
    mg = pkg.meshgen
    base = dict(mg.DEFAULT_CASE)
    return [
        (mg.voronoi_bump_channel(6000, seed=1),
         dict(base, eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8, u=mg.mach_speed(0.7))),
        (mg.voronoi_cylinder(9000, seed=2, box=(6.0, 3.0), h_wall=0.01, h_far=0.08),
         dict(base, eqn="NS", mu=0.02, limiter="SQUEEZE", time_step_type="LOCAL", CFL=0.5, BC1="NO_SLIP_WALL",
              BC2="FREESTREAM", u=mg.mach_speed(0.3), v=8.0)),
        (mg.channel_bump_quads(48, 24),
         dict(base, eqn="EULER", solution_poly_order=0, limiter="NONE", time_step_type="LOCAL", CFL=0.9,
              u=mg.mach_speed(0.5))),
        (mg.voronoi_bump_channel(3000, seed=5, thickness=0.06),
         dict(base, eqn="NS", mu=0.01, limiter="NONE", time_step_type="GLOBAL", CFL=0.5, BC1="NO_SLIP_WALL",
              BC2="EXTRAPOLATION", u=mg.mach_speed(0.4))),
        (wheels_grid(pkg),   # 20-faced cells
         dict(base, eqn="EULER", limiter="SQUEEZE", time_step_type="GLOBAL", CFL=0.8, BC1="SLIP_WALL",
              BC2="FREESTREAM", u=mg.mach_speed(0.4), v=5.0)),
    ]


def alone(pkg, grid, case, iters, precision):
    s = pkg.Solver(grid, case, precision=precision)
    s.step(iters)
    q = s.get_state()
    r = s.residual_norm()
    s.close()
    return q, r


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_alone(pkg, precision):
    prec = pkg.FP64 if precision == "fp64" else pkg.FP32
    cases = mix(pkg)
    b = pkg.Batch(200000, 600000, 16, precision=prec)
    ids = [b.add(g, c) for g, c in cases]
    b.step(6)
    norms = b.norms()
    for sid, (g, c) in zip(ids, cases):
        q_alone, r_alone = alone(pkg, g, c, 6, prec)
        q = b.get_state(sid)
        assert bits_equal(q, q_alone), f"solve {sid}: max rel {max_rel(q, q_alone):.2e}"
        nr, it = norms[sid]
        assert it == 6
        # the batch sums each solve's squares per tile and then over its tiles, the single solve
        # over 304 strided partial sums: the same residual, summed in another order, so the norms
        # agree to round-off rather than bit for bit
        assert np.allclose(nr, r_alone, rtol=1e-9 if prec == pkg.FP64 else 1e-5, atol=0)
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_norms_are_reproducible(pkg, precision):
    """The per-solve residual norms are summed in a fixed order (per tile, then over the solve's
    tiles), so the same batch run twice gives the same bits; served retirement at a residual drop is
    therefore reproducible."""
    prec = pkg.FP64 if precision == "fp64" else pkg.FP32
    cases = mix(pkg)
    runs = []
    for _ in range(2):
        b = pkg.Batch(200000, 600000, 16, precision=prec)
        ids = [b.add(g, c) for g, c in cases]
        out = []
        for _ in range(3):
            b.step(2)
            n = b.norms()
            out.append([n[i][0] for i in ids])
        runs.append(out)
        b.close()
    for a, c in zip(runs[0], runs[1]):
        for x, y in zip(a, c):
            assert bits_equal(x, y)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_join_and_leave(pkg, precision):
    prec = pkg.FP64 if precision == "fp64" else pkg.FP32
    cases = mix(pkg)
    b = pkg.Batch(200000, 600000, 8, precision=prec)
    a = b.add(*cases[0])
    c = b.add(*cases[1])
    b.step(2)
    d = b.add(*cases[2])          # joins after 2 iterations
    b.step(1)
    b.remove(c)                    # leaves after 3 iterations
    e = b.add(*cases[3])           # reuses the freed ranges
    early = b.norms()
    assert early[e][1] == 0
    if prec == pkg.FP32:
        # norms are reduced when read, from the last stage's per-tile partials: a solve admitted
        # into slots a removed solve used reads zero until its first iteration
        assert np.all(np.asarray(early[e][0]) == 0.0)
    b.step(3)
    expect = {a: (cases[0], 6), d: (cases[2], 4), e: (cases[3], 3)}
    norms = b.norms()
    assert set(norms) == set(expect)
    for sid, ((g, cs), iters) in expect.items():
        q_alone, r_alone = alone(pkg, g, cs, iters, prec)
        assert bits_equal(b.get_state(sid), q_alone), sid
        assert norms[sid][1] == iters
        assert np.allclose(norms[sid][0], r_alone, rtol=1e-9 if prec == pkg.FP64 else 1e-5, atol=0), sid
    b.close()


def test_batch_tuning_does_not_change_results(pkg):
    cases = mix(pkg)[:2]
    results = []
    for block, mult in ((256, (1, 2, 4)), (128, (1, 1, 1)), (256, (4, 8, 2))):
        b = pkg.Batch(100000, 300000, 4, precision=pkg.FP64)
        b.set_tuning(block, mult, (4000, 8000))
        ids = [b.add(g, c) for g, c in cases]
        b.step(4)
        results.append([b.get_state(i) for i in ids])
        b.close()
    for r in results[1:]:
        for x, y in zip(results[0], r):
            assert bits_equal(x, y)


def test_batch_admission(pkg):
    g, c = mix(pkg)[0]
    need = pkg.Batch.footprint(g, pkg.FP32)
    assert need > 0
    b = pkg.Batch(g.num_cells + 10, g.num_faces + 10, 4, precision=pkg.FP32)
    b.add(g, c)
    with pytest.raises(pkg.Fv2dError) as e:
        b.add(g, c)                # no room left: refused, batch unchanged
    assert e.value.code == 6
    u = b.usage()
    assert u["active"] == 1 and g.num_cells <= u["cells_used"] <= g.num_cells + 4
    b.step(2)
    assert len(b.norms()) == 1
    b.close()


def test_failing_solve_is_isolated(pkg):
    """A solve whose state turns non-physical (CFL far beyond stability) is reported for that solve
    alone (non-finite norms or FV2D_ERR_STATE on its state); its neighbour in the same batch keeps
    advancing exactly as alone."""
    mg = pkg.meshgen
    good_grid, good_case = mix(pkg)[0]
    bad_grid = mg.voronoi_bump_channel(4000, seed=9)
    bad_case = dict(mg.DEFAULT_CASE, eqn="EULER", limiter="NONE", time_step_type="LOCAL", CFL=40.0,
                    u=mg.mach_speed(0.8))
    b = pkg.Batch(100000, 300000, 4, precision=pkg.FP64)
    good = b.add(good_grid, good_case)
    bad = b.add(bad_grid, bad_case)
    b.step(30)
    norms = b.norms()
    failed = not np.all(np.isfinite(norms[bad][0]))
    try:
        b.get_state(bad)
    except pkg.Fv2dError as e:
        failed = failed or e.code == 7
    assert failed, "the unstable solve was not reported"
    assert np.all(np.isfinite(norms[good][0]))
    q_alone, _ = alone(pkg, good_grid, good_case, 30, pkg.FP64)
    assert bits_equal(b.get_state(good), q_alone)
    b.close()
