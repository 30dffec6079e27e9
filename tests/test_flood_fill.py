"""GPU hidden-geometry flood fill (svdag_flood_fill): the outside masks of
every level and the counts equal the restated hiddenGeometryFloodfill
(oracle) on GPU-built SVOs -- a sphere, a terrain, a shell with a sealed
cavity, a box scene -- and the dense 6-connected labelling on one at full
resolution; a set start cell and a non-SVO octree are errors."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _floodcheck import dense_outside, marked_voxels
from _occupancy import occupancy
from _scenes import SCENES, golden, levels_digest

pytestmark = pytest.mark.gpu


def _cavity():
    outer = sv.boxes(np.array([[0.2, 0.2, 0.2]]), np.array([[0.8, 0.8, 0.8]]))
    inner = sv.boxes(np.array([[0.4, 0.4, 0.4]]), np.array([[0.6, 0.6, 0.6]]))
    return np.concatenate([outer, inner])


def _scene(name):
    if name == "cavity":
        return _cavity()
    return SCENES[name]()


@pytest.mark.parametrize("name,L", [("ico3_L6", 6), ("ico5_L7", 7), ("terrain65_L8", 8), ("cavity", 7),
                                     ("terrain129_L9", 9)])
def test_flood_fill_matches_oracle(name, L):
    tris = _scene(name)
    g = sv.Octree()
    g.upload_triangles(tris)
    g.buildSVO(L)
    masks, ne, ns = g.hiddenGeometryFloodfill()
    o = oracle_py.OracleOctree()
    o.buildSVO(tris, L)
    wmasks, we, ws = o.hiddenGeometryFloodfill()
    assert (ne, ns) == (we, ws)
    for a, b in zip(masks, wmasks):
        assert np.array_equal(a, b)
    if L <= 7:
        pool = g.pool()
        e, s = marked_voxels(pool, masks)
        de, ds = dense_outside(occupancy(pool))
        assert np.array_equal(e, de) and np.array_equal(s, ds)
    # the masks belong to the SVO: gone after toDAG
    g.toDAG()
    with pytest.raises(sv.SvdagError):
        g.hiddenGeometryFloodfill()


G = golden()


@pytest.mark.parametrize("name", sorted(k for k in G if "outside" in G[k]))
def test_flood_fill_matches_reference_masks(name):
    """The outside masks of every level equal those of the reference's own
    hiddenGeometryFloodfill (compiled from its sources, masks zeroed first;
    golden digests) on the reference's node numbering."""
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    assert oracle_py.pool_digest(o.pool()) == g["svo"]["digest"]
    masks, _, _ = o.hiddenGeometryFloodfill()
    assert [len(m) for m in masks] == g["outside"]["counts"]
    assert levels_digest(masks) == g["outside"]["digest"]


def test_flood_fill_start_cell_set():
    g = sv.Octree()
    g.upload_triangles(sv.boxes(np.array([[0.9, 0.9, 0.9]]), np.array([[1.0, 1.0, 1.0]])))
    g.buildSVO(5)
    with pytest.raises(sv.SvdagError):
        g.hiddenGeometryFloodfill()
