"""Dense voxel occupancy of a node pool (SVO or DAG, levels of 48-byte
records as returned by pool()), and the voxel-centre query points of a unit
cube grid -- helpers for the traversal tests."""
import numpy as np


def occupancy(pool):
    L = len(pool)
    coords = np.zeros((1, 3), np.int64)
    nodes = np.zeros(1, np.int64)
    for l in range(L):
        lev = pool[l]
        hdr = lev["hdr"][nodes] & 0xFF
        ch = lev["ch"][nodes]
        nxt_c, nxt_n = [], []
        for c in range(8):
            has = (hdr >> c) & 1 == 1
            off = np.array([(c >> 2) & 1, (c >> 1) & 1, c & 1], np.int64)
            nxt_c.append(coords[has] * 2 + off)
            nxt_n.append(ch[has, c].astype(np.int64) if l + 1 < L else np.zeros(int(has.sum()), np.int64))
        coords = np.concatenate(nxt_c)
        nodes = np.concatenate(nxt_n)
    side = 1 << L
    grid = np.zeros((side, side, side), bool)
    grid[coords[:, 0], coords[:, 1], coords[:, 2]] = True
    return grid


def voxel_centres(levels):
    side = 1 << levels
    i = (np.arange(side, dtype=np.float64) + 0.5) / side
    x, y, z = np.meshgrid(i, i, i, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)
