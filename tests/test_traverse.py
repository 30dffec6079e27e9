"""GPU point queries of encoded SSVDAGs (svdag_ssvdag_traverse): the depth
every voxel centre reaches equals the restated EncodedSSVDAG::traverse, and
the voxels it reports set are exactly the voxels the GPU build produced --
for the SSVDAG file the pipeline writes (GPU SDAG, host encoder)."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _occupancy import occupancy, voxel_centres
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L7", "terrain65_L8"])
def test_ssvdag_point_queries(name, tmp_path):
    g = G[name]
    L = g["levels"]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(L)
    grid = occupancy(o.pool())
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    f = oracle_py.read_ssvdag(p)
    pts = voxel_centres(L)
    got = sv.ssvdag_traverse(f, pts)
    assert np.array_equal(got, oracle_py.ssvdag_traverse(f, pts))
    assert np.array_equal(got == L, grid.ravel())
    outside = np.array([[1.5, 0.5, 0.5], [-0.1, 0.2, 0.3]], np.float32)
    assert (sv.ssvdag_traverse(f, outside) == -1).all()


def test_ssvdag_truncated_file_is_an_error(tmp_path):
    """Pointers past the end of a truncated leaf array are caught by the
    kernel's bounds checks: the call returns an error status."""
    o = sv.Octree()
    o.upload_triangles(SCENES["ico3_L6"]())
    o.buildSVO(6)
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    f = dict(oracle_py.read_ssvdag(p))
    f["leaves"] = f["leaves"][: f["leaves"].size // 2].copy()
    with pytest.raises(sv.SvdagError):
        sv.ssvdag_traverse(f, voxel_centres(6))
