"""bench.py's multi-process logic on CPU: world_size-2 gloo ranks (no GPU).

The GPU arm runs one replica per rank and reports the whole-job rate from the slowest rank's time
(max_over_ranks); the reference arm runs on rank 0 only.  Rendezvous on 127.0.0.1.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_env() == (ws, rank, rank)
    got = bench.max_over_ranks(10.0 + 5.0 * rank, ws)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 15.0, 1: 15.0}      # every rank sees the slowest rank's time


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_sample_is_bounded():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reference_iterations(100, 1_000_000) < 100
    assert bench.reference_iterations(5, 2000) == 5
    assert bench.reference_iterations(100, 10 ** 9) == 1


def _bench(args, env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          timeout=600, env=env, cwd=ROOT)


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench(["--impl", "reference", "--gpus", "2", "--cells", "3000", "--steps", "1"],
               {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1", "MASTER_ADDR": "127.0.0.1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_rank0_prints_one_line():
    r = _bench(["--impl", "reference", "--gpus", "2", "--cells", "3000", "--steps", "2", "--cpu-cores", "2"],
               {"RANK": "0", "WORLD_SIZE": "2", "LOCAL_RANK": "0", "MASTER_ADDR": "127.0.0.1"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["config"]["cells"] > 2000
