"""The restated candidate-edge stage of the reference's lossy LSVDAG
(oracle/lossy_ref.py: sortByEffectiveRefCount, computeNodeHash, the one-bit
and equal-hash candidates, diffSubtrees with its abort rules, the acceptance
bound and the weights) against the edges the reference's own toLossyDag
wrote before its MCL clustering, on the two lowest levels it processes
(the level below clustered into singletons).  No GPU."""
import numpy as np
import pytest

import lossy_ref
import oracle_py
from _lossyref import assert_same_edges, reference_edges, reps_from_edges
from _scenes import SCENES, golden

G = golden()
CASES = sorted(k for k in G if "lossy" in G[k])


@pytest.mark.parametrize("name", CASES)
def test_oracle_candidate_edges_match_reference(name):
    g = G[name]
    L = g["levels"]
    infl, diff, refs = g["lossy"]["params"]
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES[name](), L)
    o.toDAG()
    o.initChildLevels()
    assert oracle_py.pool_digest(o.pool()) == g["dag"]["digest"]
    pool, rc = lossy_ref.sort_by_effective_refcount(o.pool())
    ref = reference_edges(g)
    e2 = lossy_ref.candidate_edges(pool, rc, L - 2, diff, refs)
    assert_same_edges([e[0] for e in e2], [e[1] for e in e2], [e[2] for e in e2], ref[L - 2], "level %d" % (L - 2))
    reps = reps_from_edges([e[0] for e in e2], [e[1] for e in e2], len(pool[L - 2]))
    e3 = lossy_ref.candidate_edges(pool, rc, L - 3, diff, refs, reps)
    assert_same_edges([e[0] for e in e3], [e[1] for e in e3], [e[2] for e in e3], ref[L - 3], "level %d" % (L - 3))
