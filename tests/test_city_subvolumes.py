"""The depth-15 city workload (4096^2 fBm terrain + 200,000 boxes, built in
chunks by the benchmark) checked on sampled subvolumes: the GPU build of a
subvolume at the full scene's voxel resolution equals the oracle's restated
reference build of the same box (buildSVO -> toDAG -> toSDAG), as buildDAG
builds its chunks (geom_octree.cpp:339-344).  Only the triangles whose box
meets the subvolume are passed; the others add nothing to it and the order
of the rest is kept."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from test_gpu_parity import first_mismatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def city():
    return sv.city()  # 35,970,812 triangles


def _subvolume(tris, lo, side):
    b = tris.reshape(-1, 3, 3)
    mn, mx = b.min(axis=1), b.max(axis=1)
    keep = np.all(mx >= lo - 1e-6, axis=1) & np.all(mn <= lo + side + 1e-6, axis=1)
    return np.ascontiguousarray(tris[keep])


@pytest.mark.parametrize("box_index", [17, 90001, 199998])
def test_city_subvolume_matches_oracle(city, box_index):
    levels_full, cell_level = 15, 6  # subvolume = one level-6 cell, built to depth 15
    n_terrain = 2 * 4095 * 4095 + 8 * 4095 + 2
    box = city[n_terrain + 12 * box_index: n_terrain + 12 * box_index + 12].reshape(-1, 3)
    centre = (box.min(axis=0) + box.max(axis=0)) / 2
    side = 1.0 / (1 << cell_level)
    lo = np.floor(centre / side) * side
    tris = _subvolume(city, lo, side)
    bbox = tuple(lo) + tuple(lo + side)
    levels = levels_full - cell_level
    ref = oracle_py.OracleOctree()
    ref.buildSVO(tris, levels, bbox)
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(levels, bbox)
    assert o.stats()["n_total_voxels"] == ref.stats()["n_total_voxels"] > 0
    assert first_mismatch(o.pool(), ref.pool()) is None
    ref.toDAG()
    o.toDAG()
    assert first_mismatch(o.pool(), ref.pool()) is None
    ref.toSDAG()
    o.toSDAG()
    assert first_mismatch(o.pool(), ref.pool()) is None
