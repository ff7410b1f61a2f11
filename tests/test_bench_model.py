"""bench.py's algorithmic byte model (the roofline numerator): each kernel's bytes per launch
follow the per-unit formulas stated with the kernels, including the FP64 single solve's stored
face states (written by the face pass, read by the squeeze instead of the previous stage's Q and G)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

N, F, NB = 999_332, 2_998_000, 2_478
NINC = 2 * F - NB


@pytest.mark.parametrize("s", [4, 8])
def test_gradient_bytes(s):
    base = N * 4 + NINC * 8 + N * 24 + NINC * 4 * s + NB * 2 * s
    assert bench.bytes_per_launch("k_gradient", N, F, NINC, NB, s, True, False) == N * 12 * s + base
    # squeeze recomputing the stale face values: previous Q and limited G per cell
    assert bench.bytes_per_launch("k_gradient", N, F, NINC, NB, s, True, True) == N * 24 * s + base
    # squeeze reading the stored face states: one state per incidence instead
    assert bench.bytes_per_launch("k_gradient", N, F, NINC, NB, s, True, True, fval=True) == \
        N * 12 * s + NINC * 4 * s + base
    assert bench.bytes_per_launch("k_gradient", N, F, NINC, NB, s, True, True, order2=False) == 0.0


def test_face_bytes_and_stored_states():
    s = 8
    plain = bench.bytes_per_launch("k_face", N, F, NINC, NB, s, True, True)
    assert plain == pytest.approx(F * (8 + 10 * s) + N * 12 * s + F * 4 * s + F * s / 3.0)
    stored = bench.bytes_per_launch("k_face", N, F, NINC, NB, s, True, True, fval=True)
    assert stored - plain == pytest.approx((2 * F - NB) * 4 * s)
    euler = bench.bytes_per_launch("k_face", N, F, NINC, NB, s, False, True)
    assert plain - euler == pytest.approx(F * 3 * s)   # lx, ly, dist


def test_single_solve_model_uses_stored_states_for_fp64_only():
    k64 = bench.single_kernel_bytes(N, F, NINC, NB, 8, comp=False)
    k32 = bench.single_kernel_bytes(N, F, NINC, NB, 4, comp=True)
    assert k64["k_gradient"] == bench.bytes_per_launch("k_gradient", N, F, NINC, NB, 8, True, True, fval=True)
    assert k32["k_gradient"] == bench.bytes_per_launch("k_gradient", N, F, NINC, NB, 4, True, True)
    # per cell-stage, the FP32 engine moves well under the FP64 one (half-width state, no stored states)
    assert sum(k32.values()) < 0.6 * sum(k64.values())


def test_spec_bytes_per_cell_stage():
    """The benchmark specification's algorithmic bytes: B = N(40.67 s + 28) + F(9 s + 8) + 4(2F - Nb)
    per stage (Euler geometry), about 617 B (FP64) and 347 B (FP32) per cell-stage on a Voronoi mesh
    with F = 3N; NS adds 5 s per face."""
    import bench
    N, F, Nb = 1_000_000, 3_000_000, 0
    assert abs(bench.bytes_8d(N, F, Nb, 8) / N - 617.3) < 0.1
    assert abs(bench.bytes_8d(N, F, Nb, 4) / N - 346.7) < 0.1
    assert bench.bytes_8d(N, F, Nb, 4, ns=True) - bench.bytes_8d(N, F, Nb, 4) == 5 * 4 * F
    assert bench.bytes_8d(N, F, Nb, 4, ns=True, euler_geometry=True) == bench.bytes_8d(N, F, Nb, 4)
    out = bench.step_8d([(N, F, Nb, 4, False, True)], ms_per_iteration=3 * 0.1, peak=6763.0)
    assert abs(out["bytes_per_cell_stage"] - 346.7) < 0.1
    assert abs(out["achieved"] - 346.7 * N / 0.1e-3 / 1e9) < 1.0
