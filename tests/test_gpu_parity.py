"""Parity of the sm_103a build path (through the C ABI) with the reference:
golden digests made by the compiled reference, and full pools from the
restated oracle on further seeded scenes.  Integer/index work: bit-exact."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()
PLAIN = sorted(k for k in G if not G[k]["step_levels"])


def first_mismatch(a, b):
    for l, (x, y) in enumerate(zip(a, b)):
        if len(x) != len(y):
            return "level %d: %d vs %d nodes" % (l, len(x), len(y))
        if not np.array_equal(x, y):
            i = int(np.nonzero(x != y)[0][0])
            return "level %d node %d: %s vs %s" % (l, i, x[i], y[i])
    if len(a) != len(b):
        return "levels %d vs %d" % (len(a), len(b))
    return None


def gpu_build(tris, levels):
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(levels)
    return o


@pytest.mark.parametrize("name", PLAIN)
def test_svo_dag_sdag_match_reference_digests(name):
    g = G[name]
    o = gpu_build(SCENES[name](), g["levels"])
    st = o.stats()
    assert st["n_total_voxels"] == g["nTotalVoxels"]
    assert st["n_nodes_svo"] == g["nNodesSVO"]
    assert [len(l) for l in o.pool()] == g["svo"]["counts"]
    assert oracle_py.pool_digest(o.pool()) == g["svo"]["digest"]
    o.toDAG()
    o.initChildLevels()
    assert o.stats()["n_nodes_dag"] == g["nNodesDAG"]
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s = o.clone()
    s.toSDAG()
    assert s.stats()["n_nodes_sdag"] == g["nNodesSDAG"]
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    c = o.clone()
    assert c.mergeAcrossAllLevels() == g["nCrossLevelMerged"]
    assert c.stats()["n_nodes"] == g["nNodesCSVDAG"]
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


def test_imported_chunked_dag_reduces_like_reference():
    """A DAG from the reference's chunked OpenMP build (buildDAG, restated by
    the oracle and pinned by its golden digest) imported through the C ABI
    (the GeomOctree(NodeData) route) gives the reference's SDAG and CSVDAG."""
    g = G["terrain129_L9_step1"]
    ref = oracle_py.OracleOctree()
    ref.buildDAG(SCENES["terrain129_L9_step1"](), g["levels"], g["step_levels"])
    ref.initChildLevels()
    assert oracle_py.pool_digest(ref.pool()) == g["dag"]["digest"]
    o = sv.Octree()
    o.importDAG(ref.pool(), n_total_voxels=g["nTotalVoxels"])
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s = o.clone()
    s.toSDAG()
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    c = o.clone()
    c.mergeAcrossAllLevels()
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("kind", ["ico", "terrain", "boxes"])
def test_random_scenes_match_oracle(kind, seed):
    if kind == "ico":
        tris, levels = sv.icosphere(4, 0.3 + 0.02 * seed, 0.08, 1000 + seed), 7 + seed % 2
    elif kind == "terrain":
        tris, levels = sv.terrain(33 + 16 * seed, 8, 0.3, 50 + seed), 8
    else:
        from _scenes import box_scene

        tris, levels = box_scene(50 * seed, 7, seed), 7
    ref = oracle_py.OracleOctree()
    ref.buildSVO(tris, levels)
    o = gpu_build(tris, levels)
    assert first_mismatch(o.pool(), ref.pool()) is None
    ref.toDAG()
    ref.initChildLevels()
    o.toDAG()
    o.initChildLevels()
    assert first_mismatch(o.pool(), ref.pool()) is None
    rs, s = ref.clone(), o.clone()
    rs.toSDAG()
    s.toSDAG()
    assert first_mismatch(s.pool(), rs.pool()) is None
    assert s.stats()["n_nodes_sdag"] == rs.stats()["n_nodes_sdag"]
    rc, c = ref.clone(), o.clone()
    rc.mergeAcrossAllLevels()
    c.mergeAcrossAllLevels()
    assert first_mismatch(c.pool(), rc.pool()) is None
    assert c.stats()["n_cross_level_merged"] == rc.stats()["n_cross_level_merged"]
    assert c.stats()["n_missing_correspondences"] == rc.stats()["n_missing_correspondences"]


def _edge(tris, levels):
    ref = oracle_py.OracleOctree()
    ref.buildSVO(tris, levels)
    o = gpu_build(tris, levels)
    assert first_mismatch(o.pool(), ref.pool()) is None
    assert o.stats()["n_total_voxels"] == ref.stats()["n_total_voxels"]
    ref.toDAG()
    o.toDAG()
    assert first_mismatch(o.pool(), ref.pool()) is None
    ref.initChildLevels()
    o.initChildLevels()
    if levels >= 2:  # the reference's merge indexes level 1, which a 1-level tree lacks
        rc, c = ref.clone(), o.clone()
        rc.mergeAcrossAllLevels()
        c.mergeAcrossAllLevels()
        assert first_mismatch(c.pool(), rc.pool()) is None
    ref.toSDAG()
    o.toSDAG()
    assert first_mismatch(o.pool(), ref.pool()) is None


def test_empty_scene():
    _edge(np.zeros((0, 9), np.float32), 5)


@pytest.mark.parametrize("levels", [1, 2, 3])
def test_shallow_trees(levels):
    _edge(sv.icosphere(2, 0.4, 0.08, 3), levels)


def test_single_and_degenerate_triangles():
    t = np.array([[0.1, 0.1, 0.1, 0.9, 0.2, 0.3, 0.4, 0.8, 0.7],      # regular
                  [0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5],      # point
                  [0.2, 0.2, 0.2, 0.4, 0.4, 0.4, 0.8, 0.8, 0.8],      # collinear
                  [0.25, 0.25, 0.25, 0.75, 0.25, 0.25, 0.25, 0.75, 0.25],  # on voxel boundaries
                  [1.5, 1.5, 1.5, 2.0, 1.5, 1.5, 1.5, 2.0, 1.5]],     # outside the box
                 np.float32)
    _edge(t, 6)
    _edge(t[:1], 6)


def test_duplicate_triangles():
    t = sv.icosphere(2, 0.4, 0.08, 8)
    _edge(np.concatenate([t, t[::-1]]), 6)


def test_build_dag_matches_reference_digests():
    """GeomOctree::buildDAG (chunked, step level 1) through the C ABI: the
    reference's node order, counts and pools."""
    name = "terrain129_L9_step1"
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildDAG(g["levels"], g["step_levels"])
    st = o.stats()
    assert st["state_name"] == "S_DAG"
    assert st["n_total_voxels"] == g["nTotalVoxels"]
    assert st["n_nodes_svo"] == g["nNodesSVO"]
    assert st["n_nodes_dag"] == g["nNodesDAG"]
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s = o.clone()
    s.toSDAG()
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    c = o.clone()
    c.mergeAcrossAllLevels()
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


@pytest.mark.parametrize("step", [1, 2])
@pytest.mark.parametrize("kind", ["ico", "terrain", "boxes"])
def test_build_dag_random_scenes_match_oracle(kind, step):
    if kind == "ico":
        tris, levels = sv.icosphere(4, 0.33, 0.08, 70 + step), 8
    elif kind == "terrain":
        tris, levels = sv.terrain(65, 8, 0.3, 90 + step), 8
    else:
        from _scenes import box_scene

        tris, levels = box_scene(120, 7, 30 + step), 7
    ref = oracle_py.OracleOctree()
    ref.buildDAG(tris, levels, step)
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildDAG(levels, step)
    assert first_mismatch(o.pool(), ref.pool()) is None
    rs, st = ref.stats(), o.stats()
    for k in ("n_total_voxels", "n_nodes_svo", "n_nodes_last_lev_svo", "n_nodes_dag"):
        assert st[k] == rs[k], k


def test_build_dag_rejects_bad_step_levels():
    o = sv.Octree()
    o.upload_triangles(sv.icosphere(2, 0.4, 0.08, 3))
    for step in (0, 5, 6):
        with pytest.raises(sv.SvdagError) as e:
            o.buildDAG(6, step)
        assert e.value.status == 1


def test_concurrent_reductions_on_two_streams():
    """The SSVDAG and CSVDAG reductions of one DAG on two clones placed on
    their own streams (svdag_clone_on), driven from two host threads at once,
    give the golden digests."""
    import concurrent.futures

    import torch

    name = "terrain65_L8"
    g = G[name]
    o = gpu_build(SCENES[name](), g["levels"])
    o.toDAG()
    o.initChildLevels()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s = o.clone(stream=s1.cuda_stream)
    c = o.clone(stream=s2.cuda_stream)
    with concurrent.futures.ThreadPoolExecutor(2) as pool:
        fs = pool.submit(s.toSDAG)
        fc = pool.submit(c.mergeAcrossAllLevels)
        fs.result()
        assert fc.result() == g["nCrossLevelMerged"]
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]
