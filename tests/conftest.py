import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden_names(long=False):
    """Golden fixture names: per-stage cases, or (long=True) the whole-run cases long_*.npz."""
    import glob
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return [n for n in names if n.startswith("long_") == long]


REFERENCE_TREE = entry.REFERENCE_TREE


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    p = entry.load_package()
    p.build.build()
    return p


@pytest.fixture(scope="session")
def orc():
    o = entry.load_oracle()
    o.build(ref_dir=REFERENCE_TREE if os.path.isdir(REFERENCE_TREE) else "/nonexistent")
    return o


@pytest.fixture(scope="session")
def has_ref(orc):
    return orc.available("ref")


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def max_rel(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / d) if d > 0 else float(np.linalg.norm(a - b))


def wheels_grid(pkg, k=24, m=20, r1=0.5, r2=1.0):
    """k disjoint wheels, each an m-gon hub cell ringed by m quadrilaterals.  The hubs' m faces exceed
    the limiter's 16-incidence chunks, and after the face-count ordering they share a warp with
    4-faced ring cells.  Outer faces (numbered first) alternate BC1 and BC2, so the flow is not uniform."""
    xs, ys, faces = [], [], ([], [], [], [])
    th = 2.0 * np.pi * np.arange(m) / m
    nxt, prv = (np.arange(m) + 1) % m, (np.arange(m) - 1) % m
    outer, inner = [], []
    for w in range(k):
        cx, cy = 3.0 * (w % 6), 3.0 * (w // 6)
        p = 2 * m * w                                                               # points so far
        pid = 1 + p + np.arange(m)
        qid = 1 + p + m + np.arange(m)
        xs += [cx + r1 * np.cos(th), cx + r2 * np.cos(th)]
        ys += [cy + r1 * np.sin(th), cy + r2 * np.sin(th)]
        hub = 1 + w * (m + 1)
        ring = hub + 1 + np.arange(m)
        outer.append((qid, qid[nxt], ring, -(np.arange(m) % 2)))                  # ring cell on the left
        inner.append((pid, pid[nxt], np.full(m, hub), ring))                       # hub on the left
        inner.append((pid, qid, ring, ring[prv]))                                  # radial: cell i on the left
    for grp in (outer, inner):
        for f in grp:
            for dst, a in zip(faces, f):
                dst.append(np.asarray(a))
    cat = lambda L: np.concatenate(L).astype(np.int32)  # noqa: E731
    return pkg.meshgen.Grid(np.concatenate(xs), np.concatenate(ys), cat(faces[0]), cat(faces[1]), cat(faces[2]),
                            cat(faces[3]), k * (m + 1), f"wheels_{k}x{m}")
