"""toSDAG with skipSymmetry -- GeomOctree::toSDAG(false, true), pointer
compression only (src/symvox/geom_octree.cpp:596-601) -- on the GPU: the
reference's own pools (golden digests written by the compiled reference),
and imported pools holding empty nodes, which it drops (a pointer to one
takes the default correspondence, id 0).  And toSDAG straight on an SVO
(the reference's direct "SVO -> SDAG", :554-556), plain and skipSymmetry."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()
NULL = 0xFFFFFFFE


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L7", "terrain65_L8", "terrain129_L9", "boxes_L8", "cavity_L7"])
def test_skip_symmetry_matches_reference(name):
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    s = o.clone()
    s.toSDAG(skip_symmetry=True)
    assert oracle_py.pool_digest(s.pool()) == g["sdagskip"]["digest"]
    assert s.stats()["n_nodes_sdag"] == g["nNodesSDAGSkipSymmetry"]
    # still a valid SDAG: the cross-level merge's precondition is a DAG, so
    # check instead that a second toSDAG is refused
    with pytest.raises(sv.SvdagError):
        s.toSDAG()


def test_skip_symmetry_drops_empty_nodes():
    """An imported DAG with empty nodes planted in two levels (and one parent
    pointer aimed at one of them): the kept nodes in order, invariance bytes
    zero, pointers following them, the stray pointer 0."""
    g = G["ico3_L6"]
    o = sv.Octree()
    o.upload_triangles(SCENES["ico3_L6"]())
    o.buildSVO(g["levels"])
    o.toDAG()
    base = [lev.copy() for lev in o.pool()]
    L = len(base)
    planted = {L - 1: [0, 5], 3: [2]}  # level -> positions (in the new level) of empty nodes
    pool = [lev.copy() for lev in base]
    for lev, pos in sorted(planted.items(), reverse=True):
        n_old = len(pool[lev])
        keep = np.ones(n_old + len(pos), bool)
        keep[pos] = False
        new_of_old = np.flatnonzero(keep)  # old index -> new index
        rec = np.zeros(n_old + len(pos), sv.REC)
        rec["ch"] = NULL
        rec[keep] = pool[lev]
        pool[lev] = rec
        par = pool[lev - 1]
        ch = par["ch"]
        m = ch != NULL
        ch[m] = new_of_old[ch[m]]
        par["ch"] = ch
    # one parent pointer aimed at an empty node of level 3
    par = pool[2]
    p = int(np.flatnonzero((par["ch"] != NULL).any(axis=1))[0])
    j = int(np.flatnonzero(par["ch"][p] != NULL)[0])
    par["ch"][p, j] = planted[3][0]
    want = [lev.copy() for lev in base]
    want[2]["ch"][p, j] = 0
    d = sv.Octree()
    d.importDAG([(lev["hdr"], lev["ch"]) for lev in pool])
    d.toSDAG(skip_symmetry=True)
    got = d.pool()
    assert [len(l) for l in got] == [len(l) for l in want]
    for l in range(L):
        np.testing.assert_array_equal(got[l]["hdr"], want[l]["hdr"], err_msg=str(l))
        if l + 1 < L:
            np.testing.assert_array_equal(got[l]["ch"], want[l]["ch"], err_msg=str(l))
        if l >= 1:
            assert not got[l]["inv"].any()
    assert d.stats()["n_nodes_sdag"] == sum(len(l) for l in want[1:])


@pytest.mark.parametrize("name", ["ico3_L6", "terrain65_L8", "cavity_L7"])
def test_sdag_straight_from_svo(name):
    """The compiled reference's direct pass gives the golden SDAG pools (its
    toSDAG on a copy of the SVO, oracle/ref_dump --sdag-from-svo); so does
    the GPU's, and nNodesDAG stays as it was."""
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.initChildLevels()
    dag_before = o.stats()["n_nodes_dag"]
    o.toSDAG()
    assert oracle_py.pool_digest(o.pool()) == g["sdagsvo"]["digest"]
    assert o.stats()["n_nodes_sdag"] == g["nNodesSDAG"]
    assert o.stats()["n_nodes_dag"] == dag_before


@pytest.mark.parametrize("name", ["ico3_L6", "terrain65_L8"])
def test_skip_symmetry_on_svo_matches_oracle(name):
    """skipSymmetry on an SVO drops only its empty nodes (duplicates stay)."""
    g = G[name]
    tris = SCENES[name]()
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(g["levels"])
    o.initChildLevels()
    o.toSDAG(skip_symmetry=True)
    r = oracle_py.OracleOctree()
    r.buildSVO(tris, g["levels"])
    r.initChildLevels()
    r.toSDAG(skip_symmetry=True)
    assert oracle_py.pool_digest(o.pool()) == oracle_py.pool_digest(r.pool())
    assert o.stats()["n_nodes_sdag"] == r.stats()["n_nodes_sdag"] > g["nNodesDAG"]
