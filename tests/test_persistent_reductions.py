"""The reduction phases (toDAG, toSDAG, mergeAcrossAllLevels) as persistent
cooperative kernels: one launch per phase, results equal to the reference's
golden digests when the phases of several octrees run side by side on their
own streams (toSDAG and the merge of one DAG, as the benchmark pipeline
does), and when a deep, narrow octree gives many tiny levels."""
import concurrent.futures

import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()
NAMES = ["ico3_L6", "ico5_L7", "terrain65_L8", "terrain129_L9", "cavity_L7"]


def launches(o):
    return o.stats()["gpu_launches"]


@pytest.mark.parametrize("name", NAMES)
def test_one_launch_per_phase(name):
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    n0 = launches(o)
    o.toDAG()
    assert launches(o) - n0 == 1
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s, c = o.clone(), o.clone()
    n0 = launches(s)
    s.toSDAG()
    assert launches(s) - n0 == 1
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    n0 = launches(c)
    assert c.mergeAcrossAllLevels() == g["nCrossLevelMerged"]
    assert launches(c) - n0 == 1
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


def test_phases_side_by_side_on_streams():
    """toSDAG and the merge of four DAGs at once, each octree on its own
    stream, driven from eight host threads."""
    torch = pytest.importorskip("torch")
    builds = []
    for name in NAMES[:4]:
        g = G[name]
        o = sv.Octree()
        o.upload_triangles(SCENES[name]())
        o.buildSVO(g["levels"])
        o.toDAG()
        o.initChildLevels()
        builds.append((name, o))
    streams = [torch.cuda.Stream() for _ in range(2 * len(builds))]
    jobs = []
    for k, (name, o) in enumerate(builds):
        jobs.append((name, "sdag", o.clone(stream=streams[2 * k].cuda_stream)))
        jobs.append((name, "csv", o.clone(stream=streams[2 * k + 1].cuda_stream)))

    def run(job):
        name, kind, oc = job
        if kind == "sdag":
            oc.toSDAG()
        else:
            oc.mergeAcrossAllLevels()
        return name, kind, oracle_py.pool_digest(oc.pool())

    with concurrent.futures.ThreadPoolExecutor(len(jobs)) as ex:
        for name, kind, digest in ex.map(run, jobs):
            assert digest == G[name][kind]["digest"], (name, kind)


def test_deep_narrow_octree():
    """Two small triangles in a deep octree: 17 levels of a few nodes each
    (many barriers over almost no work) against the oracle's reductions."""
    tris = np.array([[0.1, 0.1, 0.1, 0.1003, 0.1001, 0.1, 0.1001, 0.1003, 0.1002],
                     [0.6, 0.55, 0.7, 0.6002, 0.5501, 0.7, 0.6, 0.5502, 0.7003]], np.float32)
    levels = 17
    ref = oracle_py.OracleOctree()
    ref.buildSVO(tris, levels)
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(levels)
    assert oracle_py.pool_digest(o.pool()) == oracle_py.pool_digest(ref.pool())
    ref.toDAG()
    ref.initChildLevels()
    o.toDAG()
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == oracle_py.pool_digest(ref.pool())
    rs, s = ref.clone(), o.clone()
    rs.toSDAG()
    s.toSDAG()
    assert oracle_py.pool_digest(s.pool()) == oracle_py.pool_digest(rs.pool())
    rc, c = ref.clone(), o.clone()
    rc.mergeAcrossAllLevels()
    c.mergeAcrossAllLevels()
    assert oracle_py.pool_digest(c.pool()) == oracle_py.pool_digest(rc.pool())
    assert c.stats()["n_cross_level_merged"] == rc.stats()["n_cross_level_merged"]


@pytest.mark.parametrize("blocks", [1, 3])
def test_capped_grids_give_the_same_result(blocks):
    """svdag_set_persistent_blocks caps the reduction grids; one block (the
    barrier's trivial case, every wait of the SSVDAG resolution inside one
    block) and three blocks give the reference's digests."""
    name = "terrain129_L9"
    g = G[name]
    o = sv.Octree()
    o.set_persistent_blocks(blocks)
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    s, c = o.clone(), o.clone()
    s.toSDAG()
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]
    assert c.mergeAcrossAllLevels() == g["nCrossLevelMerged"]
    assert oracle_py.pool_digest(c.pool()) == g["csv"]["digest"]


def test_phase_trace_reports_steps(monkeypatch, capfd):
    """SVDAG_PHASE_TRACE prints each phase's step times (stderr) and changes
    no result."""
    name = "ico3_L6"
    g = G[name]
    monkeypatch.setenv("SVDAG_PHASE_TRACE", "1")
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    s = o.clone()
    s.toSDAG()
    err = capfd.readouterr().err
    assert "[svdag trace] toDAG" in err and "[svdag trace] toSDAG" in err
    assert "candidates" in err and "insert" in err
    assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]


@pytest.mark.parametrize("bulk", ["0", "2000"])
def test_bulk_levels_then_persistent(monkeypatch, bulk):
    """toDAG reduces its largest bottom levels with ordinary launches and the
    rest with the persistent kernel (the threshold is lowered so that small
    scenes take both paths; 0 = every level by launches): the reference's
    digests either way."""
    monkeypatch.setenv("SVDAG_BULK_LEVEL_NODES", bulk)
    for name in ["terrain129_L9", "ico5_L7"]:
        g = G[name]
        o = sv.Octree()
        o.upload_triangles(SCENES[name]())
        o.buildSVO(g["levels"])
        o.toDAG()
        o.initChildLevels()
        assert o.stats()["n_nodes_dag"] == g["nNodesDAG"]
        assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
        s = o.clone()
        s.toSDAG()
        assert oracle_py.pool_digest(s.pool()) == g["sdag"]["digest"]


def test_concurrent_merges_with_large_bitmaps():
    """Four merges of the 2048² depth-12 terrain's DAG at once, from four host
    threads on four streams: their check-set bitmaps exceed 48 KB of shared
    memory, so the kernel's shared-memory limit is raised -- once, never
    lowered under another thread's launch.  Each result is the reference's."""
    torch = pytest.importorskip("torch")
    name = "terrain2048_L12"
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    streams = [torch.cuda.Stream() for _ in range(4)]
    clones = [o.clone(stream=s.cuda_stream) for s in streams]

    def run(c):
        merged = c.mergeAcrossAllLevels()
        return merged, oracle_py.pool_digest(c.pool())

    with concurrent.futures.ThreadPoolExecutor(4) as ex:
        for merged, digest in ex.map(run, clones):
            assert merged == g["nCrossLevelMerged"]
            assert digest == g["csv"]["digest"]
