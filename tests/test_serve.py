"""Host logic of the serving loop (no GPU): FIFO admission gated by capacity, retirement at the
residual-drop target or the iteration cap, percentiles and throughput accounting."""
import numpy as np
import pytest


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-3)


class FakeMesh:
    def __init__(self, nc):
        self.nc = nc


class FakePool:
    def __init__(self, sizes):
        self.cells = np.array(sizes, dtype=np.float64)

    def index_for(self, cells):
        return int(np.argmin(np.abs(np.log(self.cells) - np.log(cells))))

    def host_mesh(self, i, case):
        return FakeMesh(int(self.cells[i]))


class FakeBatch:
    """Capacity in cells; each iteration costs 1e-8 s per active cell; solve k's residual decays
    by a factor 10 every (10 + k % 5) iterations."""

    def __init__(self, capacity, clock, err):
        self.cap, self.clock, self.err = capacity, clock, err
        self.used = 0
        self.solves = {}
        self.next = 0

    def add_mesh(self, hm, case):
        if self.used + hm.nc > self.cap:
            raise self.err(6, "no room")
        sid = self.next
        self.next += 1
        self.solves[sid] = [hm.nc, 0, 10 + sid % 5]
        self.used += hm.nc
        return sid

    def remove(self, sid):
        self.used -= self.solves.pop(sid)[0]

    def step(self, n):
        for s in self.solves.values():
            s[1] += n
        self.clock.t += 1e-8 * n * sum(s[0] for s in self.solves.values())

    def norms(self):
        return {sid: (np.full(4, 10.0 ** (-s[1] / s[2])), s[1]) for sid, s in self.solves.items()}

    def get_state(self, sid):
        return np.zeros(4)


def test_serve_admits_fifo_and_retires(pkg):
    from fv2d_gb300 import serve, workloads
    clock = FakeClock()
    pool = FakePool([5e3, 5e4, 5e5])
    stream = workloads.c5_stream(rate=20.0, duration=5.0, seed=3, lo=5e3, hi=5e5)
    batch = FakeBatch(capacity=1_200_000, clock=clock, err=pkg.Fv2dError)
    recs = []
    out = serve.serve(batch, stream, pool, duration=30.0, target=1e-6, max_iters=200, check_every=5,
                      clock=clock, sleep=clock.sleep, keep_states=True, records_out=recs)
    assert out["arrived"] == len(stream)
    assert out["completed"] + out["in_flight"] + out["queued"] + (out["arrived"] - out["admitted"] - out["queued"]) >= 0
    done = [r for r in recs if r.finish >= 0]
    assert done and all(r.converged for r in done)          # every fake solve reaches the target
    assert all(r.iterations <= 200 for r in done)
    # FIFO: admission times are non-decreasing in arrival order
    adm = [r.admit for r in recs if r.admit >= 0]
    assert adm == sorted(adm)
    assert out["ttc_p50_s"] <= out["ttc_p99_s"]
    assert out["cell_stage_per_s"] > 0
    assert batch.used == sum(s[0] for s in batch.solves.values())


def test_serve_capacity_gates_admission(pkg):
    from fv2d_gb300 import serve, workloads
    clock = FakeClock()
    pool = FakePool([4e5])
    stream = [(0.0, dict(cells=4e5, seed=0, thickness=0.1, mach=0.5, angle=0.0, ns=False, re=1e3)) for _ in range(5)]
    batch = FakeBatch(capacity=900_000, clock=clock, err=pkg.Fv2dError)   # room for two at a time
    out = serve.serve(batch, stream, pool, duration=100.0, target=1e-30, max_iters=50, check_every=10,
                      clock=clock, sleep=clock.sleep)
    assert out["max_queue"] == 3
    assert out["completed"] == 5 and out["converged"] == 0       # retired at the iteration cap


def test_progress_converged_stalled_failed(pkg):
    from fv2d_gb300 import serve
    p = serve.Progress(1e-6, stall_iters=100, stall_gain=0.01)
    assert p.update(np.full(4, 10.0), 25) is None               # r0
    assert p.update(np.full(4, 5.0), 50) is None                # improving
    assert p.update(np.full(4, 4.99), 100) is None              # < 1 % better: best stays at it 50
    assert p.update(np.full(4, 5.0), 150) == "stalled"          # 100 iterations without a 1 % gain
    q = serve.Progress(1e-6)
    q.update(np.full(4, 1.0), 25)
    assert q.update(np.full(4, 1e-7), 50) == "converged"
    assert q.update(np.array([1.0, np.nan, 1.0, 1.0]), 75) == "failed"
    never = serve.Progress(1e-6, stall_iters=0)                   # stall detection off
    never.update(np.full(4, 1.0), 25)
    assert all(never.update(np.full(4, 1.0), it) is None for it in range(50, 5000, 25))


class StallingBatch(FakeBatch):
    """Residuals drop to 5 % and stay there (the squeeze limiter's stall)."""

    def norms(self):
        return {sid: (np.full(4, max(0.05, 10.0 ** (-s[1] / 20))), s[1]) for sid, s in self.solves.items()}


def test_serve_retires_stalled_solves(pkg):
    from fv2d_gb300 import serve, workloads
    clock = FakeClock()
    pool = FakePool([5e3, 5e4])
    stream = workloads.c5_stream(rate=10.0, duration=3.0, seed=5, lo=5e3, hi=5e4)
    batch = StallingBatch(capacity=10 ** 6, clock=clock, err=pkg.Fv2dError)
    recs = []
    out = serve.serve(batch, stream, pool, duration=60.0, target=1e-6, max_iters=5000, check_every=25,
                      clock=clock, sleep=clock.sleep, records_out=recs, stall_iters=200)
    done = [r for r in recs if r.finish >= 0]
    assert done and all(r.stalled and not r.converged for r in done)
    assert all(r.iterations < 1000 for r in done)                # well before max_iters
    assert out["stalled"] == len(done) and out["converged"] == 0
