"""Serving: continuous batching of independent solves on one GPU.

Requests (a mesh and flow conditions) arrive as a Poisson process.  The server keeps every
admitted solve resident in one batch (fv2d_batch_*): it admits waiting requests in arrival order
whenever the batch arena has room for them (the arena is sized from an HBM budget), advances all
active solves together `check_every` iterations at a time (admissions are made while those
iterations run on the GPU and join the next round), and retires a solve when every
component of its residual L2 norm has dropped by `target` relative to its first check, when it
reaches `max_iters`, when its state turns non-physical, or (optionally, `stall_iters`) when its
residual has stopped dropping - the squeeze-limited scheme stalls near a few percent drop and can
never reach a 1e-6 target, so running it to `max_iters` only delays the queue.  Reported: p50/p99 time-to-converge
(completion - arrival) of retired requests, the fraction that met the target, and aggregate
cell-stage updates/s.  The baseline serves the same stream one request at a time through the plain
FP64 path (fv2d_create / fv2d_step).

Meshes come from a pool generated before the stream starts (log-spaced sizes over the request
size range); each request runs on the pool mesh nearest its drawn cell count, with its own flow
conditions, so mesh generation is not part of the serving path.  Host meshes (geometry) are cached
per pool mesh and boundary-code pair and admitted with fv2d_batch_add_mesh.
"""
from __future__ import annotations

import dataclasses
import math
import time
from collections import deque

import numpy as np

from . import fv2d, workloads


@dataclasses.dataclass
class Record:
    rid: int
    arrival: float
    cells: int
    admit: float = -1.0
    finish: float = -1.0
    iterations: int = 0
    converged: bool = False
    stalled: bool = False
    failed: bool = False
    state: object = None
    stage_bytes: float = 0.0


class Progress:
    """Residual history of one solve.  r0 = the norms at its first check; 'converged' once every
    component is at most target * r0; 'stalled' (with stall_iters > 0) once the best ratio so far
    (largest component of r / r0) has not improved by the relative amount stall_gain within the
    last stall_iters iterations; 'failed' on a non-finite norm."""

    def __init__(self, target, stall_iters=0, stall_gain=0.01):
        self.target, self.stall_iters, self.stall_gain = target, stall_iters, stall_gain
        self.r0 = None
        self.best = math.inf
        self.best_it = 0

    def update(self, norms, iteration):
        if not np.all(np.isfinite(norms)):
            return "failed"
        if self.r0 is None:
            self.r0 = np.maximum(norms, 1e-300)
            self.best_it = iteration
            return None
        ratio = norms / self.r0
        if np.all(ratio <= self.target):
            return "converged"
        worst = float(np.max(ratio))
        if worst < self.best * (1.0 - self.stall_gain):
            self.best, self.best_it = worst, iteration
        elif self.stall_iters > 0 and iteration - self.best_it >= self.stall_iters:
            return "stalled"
        return None


class MeshPool:
    """Pre-generated bump-channel Voronoi meshes with log-spaced sizes."""

    def __init__(self, lo=5e3, hi=2e6, n=16, seed=0, grids=None):
        if grids is None:
            sizes = np.exp(np.linspace(math.log(lo), math.log(hi), n))
            rng = np.random.default_rng(seed)
            specs = [dict(cells=int(round(c)), seed=int(rng.integers(1 << 30)), thickness=float(rng.uniform(0.04, 0.12)))
                     for c in sizes]
            grids = workloads.grids_parallel(specs)
        self.grids = grids
        self.cells = np.array([g.num_cells for g in grids], dtype=np.float64)
        self._cache = {}

    def prebuild(self):
        """Build every host mesh the workload's two boundary-code pairs need (before serving)."""
        for ns in (False, True):
            case = workloads.spec_case(dict(mach=0.5, angle=0.0, ns=ns, re=5e3))
            for i in range(len(self.grids)):
                self.host_mesh(i, case)

    def index_for(self, cells):
        return int(np.argmin(np.abs(np.log(self.cells) - math.log(cells))))

    def host_mesh(self, i, case):
        key = (i, case["BC1"], case["BC2"])
        if key not in self._cache:
            self._cache[key] = fv2d.HostMesh(self.grids[i], fv2d.case_from_dict(case))
        return self._cache[key]


def _percentiles(vals):
    if not vals:
        return None, None
    a = np.asarray(vals)
    return float(np.percentile(a, 50)), float(np.percentile(a, 99))


def serve(batch, stream, pool, duration, target=1e-6, max_iters=2000, check_every=25, clock=time.monotonic,
          sleep=time.sleep, keep_states=False, records_out=None, stall_iters=0, stall_gain=0.01,
          stage_bytes=None):
    """Continuous batching over `stream` [(arrival s, spec)] for `duration` seconds.  With
    keep_states the final state of every retired solve is kept on its record (records_out).
    stall_iters > 0 also retires solves whose residual stopped dropping (Progress).
    stage_bytes(grid, spec): algorithmic bytes of one RK stage of a request, summed over the
    stages run into `bytes_per_s`.
    Time in service (admission to retirement) is reported apart from the queue wait (arrival to
    admission); time-to-converge is their sum."""
    t0 = clock()
    pending = deque()
    active = {}                # sid -> (record, r0 or None)
    records = []
    idx = 0
    cell_stages = 0.0
    nbytes = 0.0
    max_queue = 0
    steps = 0
    active_sum = 0
    while True:
        now = clock() - t0
        if now >= duration:
            break
        while idx < len(stream) and stream[idx][0] <= now:
            arr, spec = stream[idx]
            rec = Record(rid=idx, arrival=arr, cells=int(pool.cells[pool.index_for(spec["cells"])]))
            records.append(rec)
            pending.append((rec, spec))
            idx += 1
        # the active solves' next iterations go to the GPU first (asynchronous); admissions then
        # overlap them - their uploads queue behind the step, and they join the next one
        stepped = bool(active)
        if stepped:
            batch.step(check_every)
            steps += 1
            active_sum += len(active)
            cell_stages += 3.0 * check_every * sum(a[0].cells for a in active.values())
            nbytes += 3.0 * check_every * sum(a[0].stage_bytes for a in active.values())
        admitted = 0
        while pending:                                   # FIFO admission while the arena has room
            rec, spec = pending[0]
            case = workloads.spec_case(spec)
            hm = pool.host_mesh(pool.index_for(spec["cells"]), case)
            try:
                sid = batch.add_mesh(hm, case)
            except fv2d.Fv2dError as e:
                if e.code == 6:
                    break
                raise
            rec.admit = clock() - t0
            if stage_bytes is not None:
                rec.stage_bytes = float(stage_bytes(pool.grids[pool.index_for(spec["cells"])], spec))
            active[sid] = [rec, Progress(target, stall_iters, stall_gain)]
            pending.popleft()
            admitted += 1
        max_queue = max(max_queue, len(pending))
        if not stepped:
            if admitted:
                continue
            if idx >= len(stream):
                break
            sleep(max(0.0, min(stream[idx][0] - (clock() - t0), duration - (clock() - t0))))
            continue
        norms = batch.norms()
        now = clock() - t0
        for sid, (nr, it) in norms.items():
            if sid not in active or it == 0:
                continue
            rec, prog = active[sid]
            rec.iterations = it
            status = prog.update(nr, it)
            rec.failed = status == "failed"
            rec.converged = status == "converged"
            rec.stalled = status == "stalled"
            done = status is not None or it >= max_iters
            if done:
                rec.finish = now
                if keep_states:
                    try:
                        rec.state = batch.get_state(sid)
                    except fv2d.Fv2dError:
                        rec.state = None
                batch.remove(sid)
                del active[sid]
    elapsed = clock() - t0
    if records_out is not None:
        records_out.extend(records)
    finished = [r for r in records if r.finish >= 0]
    ttc = [r.finish - r.arrival for r in finished]
    p50, p99 = _percentiles(ttc)
    w50, w99 = _percentiles([r.admit - r.arrival for r in records if r.admit >= 0])
    s50, s99 = _percentiles([r.finish - r.admit for r in finished])
    return dict(mode="continuous batching", duration_s=round(elapsed, 2), arrived=len(records), admitted=sum(r.admit >= 0 for r in records),
                completed=len(finished), converged=sum(r.converged for r in finished), stalled=sum(r.stalled for r in finished),
                failed=sum(r.failed for r in finished), failed_requests=[r.rid for r in finished if r.failed][:32],
                in_flight=len(active), queued=len(pending), max_queue=max_queue,
                mean_active=round(active_sum / steps, 1) if steps else 0,
                ttc_p50_s=p50, ttc_p99_s=p99, wait_p50_s=w50, wait_p99_s=w99, service_p50_s=s50, service_p99_s=s99,
                retired_by={"converged": sum(r.converged for r in finished), "stalled": sum(r.stalled for r in finished),
                            "max_iters": sum(not (r.converged or r.stalled or r.failed) for r in finished),
                            "failed": sum(r.failed for r in finished)},
                cell_stage_per_s=cell_stages / elapsed if elapsed > 0 else 0.0,
                bytes_per_s=nbytes / elapsed if elapsed > 0 and stage_bytes is not None else None,
                target=target, max_iters=max_iters, check_every=check_every, stall_iters=stall_iters)


def serve_one_at_a_time(stream, pool, duration, precision=fv2d.FP64, target=1e-6, max_iters=2000, check_every=25,
                        clock=time.monotonic, sleep=time.sleep, stall_iters=0, stall_gain=0.01):
    """The baseline: the same stream, one request at a time, each through fv2d_create/fv2d_step."""
    t0 = clock()
    records = []
    cell_stages = 0.0
    idx = 0
    while idx < len(stream):
        now = clock() - t0
        if now >= duration:
            break
        arr, spec = stream[idx]
        if arr > now:
            sleep(min(arr - now, duration - now))
            continue
        i = pool.index_for(spec["cells"])
        rec = Record(rid=idx, arrival=arr, cells=int(pool.cells[i]), admit=now)
        records.append(rec)
        s = fv2d.Solver(pool.grids[i], workloads.spec_case(spec), precision=precision)
        prog = Progress(target, stall_iters, stall_gain)
        while clock() - t0 < duration:
            s.step(check_every)
            cell_stages += 3.0 * check_every * rec.cells
            rec.iterations += check_every
            try:
                nr = s.residual_norm()
            except fv2d.Fv2dError:
                rec.failed = True
                break
            status = prog.update(nr, rec.iterations)
            rec.failed = status == "failed"
            rec.converged = status == "converged"
            rec.stalled = status == "stalled"
            if status is not None or rec.iterations >= max_iters:
                break
        s.close()
        if clock() - t0 < duration or rec.converged or rec.stalled or rec.failed or rec.iterations >= max_iters:
            rec.finish = clock() - t0
        idx += 1
    elapsed = clock() - t0
    arrived = sum(1 for a, _ in stream if a <= elapsed)
    finished = [r for r in records if r.finish >= 0]
    p50, p99 = _percentiles([r.finish - r.arrival for r in finished])
    return dict(mode="one at a time", precision="fp64" if precision == fv2d.FP64 else "fp32",
                duration_s=round(elapsed, 2), arrived=arrived, completed=len(finished),
                converged=sum(r.converged for r in finished), stalled=sum(r.stalled for r in finished),
                failed=sum(r.failed for r in finished), failed_requests=[r.rid for r in finished if r.failed][:32],
                ttc_p50_s=p50, ttc_p99_s=p99, cell_stage_per_s=cell_stages / elapsed if elapsed > 0 else 0.0,
                target=target, max_iters=max_iters, check_every=check_every, stall_iters=stall_iters)


# Arena limits: the FP64 batch stores arena face ids as 32-bit (face << 1 | side); the FP32 batch's
# tile layout keeps solve-local ids and 64-bit block offsets, with 32-bit cell ids (<= 2^30 cells).
MAX_ARENA_FACES = {fv2d.FP64: (1 << 29) - (1 << 20), fv2d.FP32: (1 << 31) - (1 << 24)}
MAX_ARENA_CELLS = {fv2d.FP64: 1 << 30, fv2d.FP32: (1 << 30) - (1 << 20)}


def capacity_from_budget(pool, budget_bytes, precision=fv2d.FP32):
    """Batch capacity (cells, faces, solves) whose arena fits in `budget_bytes`, in the proportion
    of faces to cells of the pool's meshes, within the arena's id limits; also which bound set it
    ("budget" or "ids")."""
    per_cell = np.mean([fv2d.Batch.footprint(g, precision) / g.num_cells for g in pool.grids])
    faces_per_cell = float(np.mean([g.num_faces / g.num_cells for g in pool.grids]))
    by_budget = budget_bytes / per_cell
    by_ids = min(MAX_ARENA_CELLS[precision], MAX_ARENA_FACES[precision] / faces_per_cell)
    cells = int(min(by_budget, by_ids))
    return (cells, int(cells * faces_per_cell) + 1024, max(16, min(8192, int(cells / 4000))),
            "budget" if by_budget <= by_ids else "ids")
