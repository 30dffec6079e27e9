"""GPU point queries of encoded SSVDAGs (svdag_ssvdag_traverse): the depth
every voxel centre reaches equals the restated EncodedSSVDAG::traverse, and
the voxels it reports set are exactly the voxels the GPU build produced --
for the SSVDAG file the pipeline writes (GPU SDAG, host encoder) -- and the
reference's own EncodedSSVDAG::traverse (compiled from its sources; golden
results) gives the same depth wherever its walk ends above the leaf bricks.

What the reference comparison covers: with one-word child pointers (the
files used), the reference reads its inner nodes, pointers and mirror flags
as its encoder writes them, so every query that stops above the brick level
(depth <= levels - 3, or -1 outside the box) must match exactly.  At the
bricks the reference's traverse reads byte `child` of the 8-byte brick as a
2x2x2 sub-brick (encoded_ssvdag.cpp:556-569) while its encoder writes the
4x4x4 brick in voxel-matrix order (:317-345, enabled at :32); there the
kernel follows the encoder, and the test checks only that both walks reached
the brick level."""
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


@pytest.mark.parametrize("name", sorted(k for k in G if "traverse" in G[k]))
def test_ssvdag_point_queries_match_the_reference_traverse(name, tmp_path):
    import hashlib
    import os

    from _scenes import GOLDEN, traverse_points

    g = G[name]
    L = g["levels"]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(L)
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    with open(p, "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == g["files"]["ssvdag"]  # the reference's own file
    f = oracle_py.read_ssvdag(p)
    pts = traverse_points(L)
    ref = np.load(os.path.join(GOLDEN, g["traverse"]["file"]))["depth"].astype(np.int32)
    assert ref.size == pts.shape[0] == g["traverse"]["points"]
    got = sv.ssvdag_traverse(f, pts)
    above = ref <= L - 3
    assert above.sum() > 0 and (~above).sum() > 0
    assert np.array_equal(got[above], ref[above])
    assert (got[~above] >= L - 2).all()


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
