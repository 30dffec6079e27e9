"""The restated hidden-geometry flood fill (oracle, geom_octree_extension.cpp:
1651-1891) against the reference's own hiddenGeometryFloodfill (golden
outside masks, compiled reference, masks zeroed first because the reference
never initialises them) and against a dense 6-connected labelling of the
voxel grid: the empty cells it marks cover exactly the empty voxels
connected to the corner, and the set voxels it marks are exactly those
touching them.  No GPU."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _floodcheck import dense_outside, marked_voxels
from _occupancy import occupancy
from _scenes import SCENES, golden, levels_digest

G = golden()
FLOOD = sorted(k for k in G if "outside" in G[k])


@pytest.mark.parametrize("name", FLOOD)
def test_oracle_flood_fill_matches_reference_masks(name):
    g = G[name]
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES[name](), g["levels"])
    masks, n_empty, n_surface = o.hiddenGeometryFloodfill()
    assert [len(m) for m in masks] == g["outside"]["counts"]
    assert levels_digest(masks) == g["outside"]["digest"]


def _shell_with_cavity():
    """A closed box with a closed inner box: the cavity between them is
    unreachable from the corner."""
    outer = sv.boxes(np.array([[0.2, 0.2, 0.2]]), np.array([[0.8, 0.8, 0.8]]))
    inner = sv.boxes(np.array([[0.4, 0.4, 0.4]]), np.array([[0.6, 0.6, 0.6]]))
    return np.concatenate([outer, inner])


@pytest.mark.parametrize("name,L", [("ico3_L6", 6), ("terrain65_L8", 8), ("cavity_L6", 6)])
def test_oracle_flood_fill_matches_dense_labelling(name, L):
    tris = _shell_with_cavity() if name == "cavity_L6" else SCENES[name]()
    o = oracle_py.OracleOctree()
    o.buildSVO(tris, L)
    pool = o.pool()
    masks, n_empty, n_surface = o.hiddenGeometryFloodfill()
    occ = occupancy(pool)
    empty_out, set_out = marked_voxels(pool, masks)
    want_empty, want_set = dense_outside(occ)
    assert np.array_equal(empty_out, want_empty)
    assert np.array_equal(set_out, want_set)
    assert n_surface == int(set_out.sum())
    assert (~occ & ~want_empty).any() or name != "cavity_L6"  # the cavity stays inside


def test_oracle_flood_fill_start_cell_set():
    tris = sv.boxes(np.array([[0.9, 0.9, 0.9]]), np.array([[1.0, 1.0, 1.0]]))
    o = oracle_py.OracleOctree()
    o.buildSVO(tris, 5)
    assert o.hiddenGeometryFloodfill() is None
