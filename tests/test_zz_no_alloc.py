"""svdag_reduce_dag_noalloc -- toDAG on the library's static device scratch,
for callers that cannot allocate device memory mid-work -- against
svdag_reduce_dag: the same pools and counts, call after call (big and small
trees in a row, so what one call leaves in the scratch cannot leak into the
next), no device allocation during the call (the library's allocation
counter stands still across it and moves across svdag_reduce_dag), the same
octree state afterwards (the SVO's outside masks gone, clones the same size),
the in-place levels read by the later phases like freshly allocated ones,
and a tree too big for the scratch rejected with the octree unchanged."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()
OVERFLOW = 5  # SVDAG_ERR_OVERFLOW


def _svo(tris, levels):
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(levels)
    return o


def _same_pool(a, b):
    assert len(a) == len(b)
    for l, (x, y) in enumerate(zip(a, b)):
        assert len(x) == len(y), "level %d: %d vs %d nodes" % (l, len(x), len(y))
        assert np.array_equal(x, y), "level %d differs" % l


def test_two_calls_in_a_row_match_reduce_dag():
    for name in ["terrain257_L10", "ico3_L6", "terrain257_L10", "ico5_L9"]:
        g = G[name]
        svo = _svo(SCENES[name](), g["levels"])
        want = svo.clone()
        want.toDAG()
        for _ in range(2):
            o = svo.clone()
            before = o.stats()["gpu_launches"]
            o.toDAG_noalloc()
            st = o.stats()
            assert st["gpu_launches"] > before
            assert st["state_name"] == "S_DAG"
            assert st["n_nodes_dag"] == st["n_nodes"] == want.stats()["n_nodes_dag"] == g["nNodesDAG"]
            _same_pool(o.pool(), want.pool())
            o.initChildLevels()  # the reference digests carry child levels
            assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]


def test_no_device_allocation_and_same_state():
    name = "terrain257_L10"
    g = G[name]
    svo = _svo(SCENES[name](), g["levels"])
    svo.hiddenGeometryFloodfill()  # outside masks on the SVO's levels
    want, o = svo.clone(), svo.clone()
    o.toDAG_noalloc()  # the first call on the device looks the array up
    o = svo.clone()
    n0 = sv.device_alloc_count()
    o.toDAG_noalloc()
    assert sv.device_alloc_count() == n0, "svdag_reduce_dag_noalloc allocated device memory"
    n1 = sv.device_alloc_count()
    want.toDAG()
    assert sv.device_alloc_count() > n1  # the counter does see the allocating path
    _same_pool(o.pool(), want.pool())
    for oc in (o, want):
        with pytest.raises(sv.SvdagError) as e:  # outside masks belong to the SVO only
            _masks(oc, 1)
        assert e.value.status == 2  # SVDAG_ERR_INVALID_STATE
    # a clone copies only the reduced levels' live nodes, whichever path reduced them
    a, b = o.clone(), want.clone()
    _same_pool(a.pool(), b.pool())
    assert a.stats()["n_nodes_dag"] == b.stats()["n_nodes_dag"] == g["nNodesDAG"]


def _masks(o, level):
    out = np.zeros(max(o.level_count(level), 1), np.uint8)
    o._check(o._lib.svdag_download_outside_masks(o._h, level, out.ctypes.data))
    return out


def test_later_phases_read_the_reduced_levels():
    name = "ico5_L9"
    g = G[name]
    o = _svo(SCENES[name](), g["levels"])
    o.toDAG_noalloc()
    o.toDAG_noalloc()  # a DAG reduces to itself
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s = o.clone()
    s.toSDAG()
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    c = o.clone()
    c.mergeAcrossAllLevels()
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


@pytest.mark.parametrize("levels", [1, 2, 3])
def test_empty_and_shallow_trees(levels):
    for tris in (np.zeros((0, 9), np.float32), sv.icosphere(2, 0.4, 0.08, 3)):
        svo = _svo(tris, levels)
        want = svo.clone()
        want.toDAG()
        o = svo.clone()
        o.toDAG_noalloc()
        _same_pool(o.pool(), want.pool())
        assert o.stats()["n_nodes_dag"] == want.stats()["n_nodes_dag"]


def test_tree_above_the_scratch_is_rejected_untouched():
    o = _svo(sv.icosphere(5, 0.4, 0.08, 11), 12)
    counts = [o.level_count(l) for l in range(12)]
    assert max(counts[1:-1]) > 1398101  # an inner level larger than 64 MiB of scratch holds
    with pytest.raises(sv.SvdagError) as e:
        o.toDAG_noalloc()
    assert e.value.status == OVERFLOW
    assert "level" in str(e.value) and "scratch" in str(e.value)
    assert o.stats()["state_name"] == "S_SVO"
    assert [o.level_count(l) for l in range(12)] == counts
    # the unlimited entry point still reduces the same octree, and the
    # static scratch still serves a tree that fits
    o.toDAG()
    assert o.stats()["state_name"] == "S_DAG"
    g = G["ico3_L6"]
    small = _svo(SCENES["ico3_L6"](), g["levels"])
    small.toDAG_noalloc()
    small.initChildLevels()
    assert oracle_py.pool_digest(small.pool()) == g["dag"]["digest"]
