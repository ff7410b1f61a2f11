"""Autotuner of the batched engine's launch shapes, per solve-size bucket.

FP64 batches: persistent grids over tiles of `block * mult[bucket]` cells or faces of one solve;
the tuner tries the block size with unit tiles, then each bucket's tile multiple in turn.
FP32 batches (one fused kernel per RK stage over 256-cell tiles, one CTA of 256 threads per tile):
the tile is fixed by the mesh layout; the tuner tries each bucket's faces per warp of the flux pass
(flux records a warp takes per grab: 32 x mult) in turn.
Both then try the grid mode (persistent CTAs against one CTA per tile).  The tuner times whole
iterations of the loaded batch (CUDA graph replay, wall clock around synchronised steps) and keeps
the fastest; launch shapes never change results, so tuning runs on the live batch.
"""
from __future__ import annotations

import time

BLOCKS = (128, 256)             # the batch kernels accept blocks up to 256 threads
MULTS = (1, 2, 4, 8)


def time_iterations(batch, iters=5, warmup=2):
    batch.step(warmup)
    batch.synchronize()
    t0 = time.perf_counter()
    batch.step(iters)
    batch.synchronize()
    return (time.perf_counter() - t0) / iters


FP32_MULTS = (1, 2, 4)          # faces per warp of the FP32 flux pass: 32, 64, 128


def tune(batch, iters=5, warmup=2, blocks=BLOCKS, mults=MULTS, edges=None, log=None):
    """Pick the fastest (block, tile_mult per bucket, grid mode) for the solves currently in `batch`."""
    from . import fv2d
    _, mult0, edges0 = batch.get_tuning()
    edges = tuple(edges or edges0)
    if batch.precision == fv2d.FP32:
        blocks, mults = (256,), FP32_MULTS   # the FP32 stage kernel's CTA is fixed at 256 threads
    batch.set_grid_mode(False)
    trials = []
    best = None
    for b in blocks:
        batch.set_tuning(b, (1, 1, 1), edges)
        t = time_iterations(batch, iters, warmup)
        trials.append(((b, (1, 1, 1)), t))
        if best is None or t < best[1]:
            best = ((b, [1, 1, 1]), t)
    block, mult = best[0]
    for bucket in range(3):
        for m in mults[1:]:
            trial = list(mult)
            trial[bucket] = m
            batch.set_tuning(block, tuple(trial), edges)
            t = time_iterations(batch, iters, warmup)
            trials.append(((block, tuple(trial)), t))
            if t < best[1]:
                best = ((block, trial), t)
                mult = trial
    batch.set_tuning(block, tuple(mult), edges)
    # grid mode: persistent (SMs x resident blocks) against one block per tile
    full = False
    batch.set_grid_mode(True)
    t = time_iterations(batch, iters, warmup)
    trials.append(((block, tuple(mult), "full-grid"), t))
    if t < best[1]:
        best = ((block, mult), t)
        full = True
    else:
        batch.set_grid_mode(False)
    if log:
        for (cfg, t) in trials:
            log(f"autotune block={cfg[0]} mult={cfg[1]}: {t * 1e3:.3f} ms/iteration")
    return dict(block=block, tile_mult=list(mult), bucket_edges=list(edges), full_grid=full,
                ms_per_iteration=best[1] * 1e3,
                trials=[dict(block=c[0], tile_mult=list(c[1]), full_grid=len(c) > 2, ms=t * 1e3) for c, t in trials])
