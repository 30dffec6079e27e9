"""buildSVO's leavesCenters output (GeomOctree::buildSVO(levels, bbox,
internalCall, &leavesCenters), src/symvox/geom_octree.cpp:245-246) on the
GPU: the fp64 centre of every leaf-level node in creation order, equal to
the list the compiled reference fills (golden SHA-256 of the doubles)."""
import hashlib

import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L7", "terrain65_L8", "terrain129_L9", "boxes_L8", "cavity_L7"])
def test_leaf_centers_match_reference(name):
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    c = o.buildSVO(g["levels"], leaves_centers=True)
    assert c.shape == (g["leaf_centers"]["count"], 3) == (g["svo"]["counts"][-1], 3)
    assert hashlib.sha256(np.ascontiguousarray(c, "<f8").tobytes()).hexdigest() == g["leaf_centers"]["sha256"]
    # the SVO is the one the plain build makes
    assert oracle_py.pool_digest(o.pool()) == g["svo"]["digest"]


def test_leaf_centers_kept_only_on_request():
    o = sv.Octree()
    o.upload_triangles(SCENES["ico3_L6"]())
    assert o.buildSVO(6, leaves_centers=True).shape[0] > 0
    o.buildSVO(6)  # a plain build drops them
    n = sv.ctypes.c_uint64(7)
    o._check(o._lib.svdag_download_leaf_centers(o._h, None, 0, sv.ctypes.byref(n)))
    assert n.value == 0
    assert o.buildSVO(1, leaves_centers=True).shape == (0, 3)  # the root is the leaf
