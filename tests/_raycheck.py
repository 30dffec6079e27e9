"""Helpers for the ray-casting tests: encoded SSVDAG files of oracle-built
scenes, and an independent float64 voxel walk (Amanatides-Woo) over the
dense occupancy grid that finds the first set voxel along each camera ray."""
import numpy as np

import oracle_py
import svdag_gb300 as sv
from _occupancy import occupancy
from _scenes import SCENES


def encoded_scene(name, levels, tmp_path, builder="oracle"):
    if builder == "oracle":
        o = oracle_py.OracleOctree()
        o.buildSVO(SCENES[name](), levels)
    else:
        o = sv.Octree()
        o.upload_triangles(SCENES[name]())
        o.buildSVO(levels)
    grid = occupancy(o.pool())
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / (name + ".ssvdag"))
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    return grid, oracle_py.read_ssvdag(p)


def camera_rays(cam):
    W, H = cam["width"], cam["height"]
    vi = np.asarray(cam["view_inv"], np.float64).reshape(4, 4).T
    pi = np.asarray(cam["proj_inv"], np.float64).reshape(4, 4).T
    for py in range(H):
        for px in range(W):
            sx, sy = (px + 0.5) / W * 2 - 1, (py + 0.5) / H * 2 - 1
            a, b = pi @ [sx, sy, 0, 1], pi @ [sx, sy, 1, 1]
            d = b[:3] / b[3] - a[:3] / a[3]
            d /= np.linalg.norm(d)
            o = (vi @ [0, 0, 0, 1])[:3]
            d = (vi @ [*d, 1])[:3] - o
            yield o, d / np.linalg.norm(d)


def first_voxel(grid, o, d):
    n = grid.shape[0]
    d = np.where(np.abs(d) < 1e-12, 1e-12, d)
    t1, t2 = (0 - o) / d, (1 - o) / d
    tin, tout = max(np.minimum(t1, t2).max(), 0.0), np.maximum(t1, t2).min()
    if tin >= tout:
        return None
    idx = np.clip(((o + (tin + 1e-9) * d) * n).astype(int), 0, n - 1)
    step = np.sign(d).astype(int)
    tnext = ((idx + (step > 0)) / n - o) / d
    tdelta = np.abs(1 / (n * d))
    while True:
        if grid[idx[0], idx[1], idx[2]]:
            return tuple(int(v) for v in idx)
        k = int(np.argmin(tnext))
        idx[k] += step[k]
        if idx[k] < 0 or idx[k] >= n:
            return None
        tnext[k] += tdelta[k]


def coarse(grid, shift):
    """Occupancy of the cells 2^shift voxels wide."""
    n = grid.shape[0] >> shift
    s = 1 << shift
    return grid.reshape(n, s, n, s, n, s).any(axis=(1, 3, 5))
