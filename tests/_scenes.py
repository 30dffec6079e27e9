"""Seeded scenes shared by the tests (same builders as tests/golden/make_golden.py)."""
import json
import os

import numpy as np

import svdag_gb300 as sv

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def box_scene(n, levels, seed):
    rng = np.random.default_rng(seed)
    res = 2 ** levels
    lo = rng.integers(0, res - 8, size=(n, 3))
    side = rng.integers(1, 16, size=(n, 3))
    hi = np.minimum(lo + side, res)
    return sv.boxes((lo + 0.25) / res, (hi - 0.25) / res)


def cavity_scene():
    """A closed box shell with a sealed box cavity inside it."""
    outer = sv.boxes(np.array([[0.2, 0.2, 0.2]]), np.array([[0.8, 0.8, 0.8]]))
    inner = sv.boxes(np.array([[0.4, 0.4, 0.4]]), np.array([[0.6, 0.6, 0.6]]))
    return np.concatenate([outer, inner])


def levels_digest(levels):
    """SHA-256 over per-level byte arrays (u64 count, then the bytes), the
    form of the golden outside-mask digests."""
    import hashlib

    h = hashlib.sha256()
    for lev in levels:
        h.update(np.uint64(len(lev)).tobytes())
        h.update(np.ascontiguousarray(lev).tobytes())
    return h.hexdigest()


SCENES = {
    "ico5_L9": lambda: sv.icosphere(5, 0.4, 0.08, 1234),
    "ico5_L7": lambda: sv.icosphere(5, 0.4, 0.08, 1234),
    "ico3_L6": lambda: sv.icosphere(3, 0.4, 0.08, 99),
    "ico4_L8_seed5": lambda: sv.icosphere(4, 0.35, 0.08, 5),
    "terrain65_L8": lambda: sv.terrain(65, 8, 0.3, 7),
    "terrain129_L9": lambda: sv.terrain(129, 8, 0.3, 11),
    "terrain129_L9_step1": lambda: sv.terrain(129, 8, 0.3, 11),
    "terrain257_L10": lambda: sv.terrain(257, 8, 0.3, 3),
    "boxes_L8": lambda: box_scene(300, 8, 21),
    "cavity_L7": lambda: cavity_scene(),
    # the benchmark's headline workload (8,396,796 triangles, depth 12)
    "terrain2048_L12": lambda: sv.terrain(2048, 8, 0.3, 7),
}

# golden cases too large for the CPU suite's single-threaded oracle runs
HEAVY = {"terrain2048_L12"}


def traverse_points(levels, seed=2024, n_random=300000):
    """Query points of the traversal fixtures: every voxel centre (levels
    <= 7), then seeded uniform points in [-0.05, 1.05)^3 (some outside the
    box)."""
    pts = []
    if levels <= 7:
        r = 1 << levels
        pts.append((np.indices((r, r, r)).reshape(3, -1).T.astype(np.float64) + 0.5) / r)
    pts.append(np.random.default_rng(seed).uniform(-0.05, 1.05, (n_random, 3)))
    return np.concatenate(pts).astype(np.float32)


def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)
