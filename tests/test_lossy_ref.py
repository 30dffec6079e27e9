"""The reference's lossy candidate stage on the GPU (through the C ABI):
svdag_sort_by_effective_refcount gives the restated sortByEffectiveRefCount's
pools bit for bit, and svdag_lossy_candidates gives the edges the reference's
own toLossyDag wrote before its MCL clustering -- levels - 2 (one-bit hash
probe) and levels - 3 (equal hash, diffSubtrees with its abort rules,
acceptance bound and weights, the level below clustered into singletons)."""
import numpy as np
import pytest

import lossy_ref
import oracle_py
import svdag_gb300 as sv
from _lossyref import assert_same_edges, reference_edges, reps_from_edges
from _scenes import SCENES, golden
from test_gpu_parity import first_mismatch

pytestmark = pytest.mark.gpu
G = golden()
CASES = sorted(k for k in G if "lossy" in G[k])


@pytest.mark.parametrize("name", CASES)
def test_gpu_candidate_edges_match_reference(name):
    g = G[name]
    L = g["levels"]
    infl, diff, refs = g["lossy"]["params"]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(L)
    o.toDAG()
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    want_pool, _ = lossy_ref.sort_by_effective_refcount(o.pool())
    o.sortByEffectiveRefCount()
    assert first_mismatch(o.pool(), want_pool) is None
    ref = reference_edges(g)
    s2, t2, w2 = o.lossyCandidates(L - 2, diff, refs)
    assert_same_edges(s2, t2, w2, ref[L - 2], "level %d" % (L - 2))
    reps = reps_from_edges(s2, t2, o.level_count(L - 2))
    s3, t3, w3 = o.lossyCandidates(L - 3, diff, refs, reps)
    assert_same_edges(s3, t3, w3, ref[L - 3], "level %d" % (L - 3))


def test_candidates_on_higher_levels_match_the_restatement():
    """Levels whose node hash has depth 2 and more (no reference edges there:
    they depend on the MCL clustering below them) against the restated stage,
    with a seeded set of representatives below."""
    name = "terrain129_L9"
    L = G[name]["levels"]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(L)
    o.toDAG()
    o.initChildLevels()
    o.sortByEffectiveRefCount()
    pool = o.pool()
    rc = lossy_ref.effective_refcounts(pool)
    rng = np.random.default_rng(3)
    for lev in (L - 4, L - 5):
        reps = (rng.random(len(pool[lev + 1])) < 0.05).astype(np.uint8)
        want = lossy_ref.candidate_edges(pool, rc, lev, 2.0, 4, reps)
        s, t, w = o.lossyCandidates(lev, 2.0, 4, reps)
        assert [(int(a), int(b)) for a, b in zip(s, t)] == [(a, b) for a, b, _ in want], lev
        assert np.array_equal(np.asarray(w, np.float32), np.array([x for _, _, x in want], np.float32)), lev


def test_candidates_reject_bad_arguments():
    o = sv.Octree()
    o.upload_triangles(SCENES["ico3_L6"]())
    o.buildSVO(6)
    with pytest.raises(sv.SvdagError):  # not a DAG yet
        o.lossyCandidates(3)
    o.toDAG()
    for lev in (0, 5, 6):
        with pytest.raises(sv.SvdagError):
            o.lossyCandidates(lev)
