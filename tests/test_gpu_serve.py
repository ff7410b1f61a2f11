"""Serving on the GPU: requests admitted while others run, capacity-gated, each retired solve's
result identical to the same solve run alone for the same number of iterations."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(pkg):
    from fv2d_gb300 import serve, workloads
    pool = serve.MeshPool(grids=[pkg.meshgen.voronoi_bump_channel(n, seed=k) for k, n in enumerate((2500, 6000, 15000))])
    stream = workloads.c5_stream(rate=8.0, duration=3.0, seed=5, lo=2e3, hi=2e4)
    assert len(stream) >= 10
    cap_cells = 30000                      # forces queueing: a few solves at a time
    b = pkg.Batch(cap_cells, 3 * cap_cells + 1024, 16, precision=pkg.FP32)
    recs = []
    out = serve.serve(b, stream, pool, duration=60.0, target=1e-6, max_iters=150, check_every=25,
                      keep_states=True, records_out=recs)
    b.close()
    done = [r for r in recs if r.finish >= 0]
    assert out["completed"] == len(stream) == len(done)
    assert out["max_queue"] >= 1
    assert out["failed"] == 0
    for r in done:
        arr, spec = stream[r.rid]
        i = pool.index_for(spec["cells"])
        s = pkg.Solver(pool.grids[i], workloads.spec_case(spec), precision=pkg.FP32)
        s.step(r.iterations)
        assert bits_equal(s.get_state(), r.state), r.rid
        s.close()
