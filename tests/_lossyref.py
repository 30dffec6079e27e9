"""Shared checks of the lossy candidate-edge stage against the edges the
reference's own toLossyDag wrote (tests/golden/<case>_lossy.npz)."""
import os

import numpy as np

from _scenes import GOLDEN


def reference_edges(g):
    z = np.load(os.path.join(GOLDEN, g["lossy"]["file"]))
    out = {}
    for lev in map(int, g["lossy"]["edges"]):
        out[lev] = (z["l%d_src" % lev], z["l%d_tgt" % lev], z["l%d_w" % lev])
    return out


def weight_text(w):
    """A float weight as the reference's ofstream << float prints it (6
    significant digits, %g)."""
    return "%g" % float(np.float32(w))


def assert_same_edges(src, tgt, w, ref, what):
    rs, rt, rw = ref
    assert len(src) == len(rs), "%s: %d edges, the reference %d" % (what, len(src), len(rs))
    assert np.array_equal(np.asarray(src, np.uint32), rs), what
    assert np.array_equal(np.asarray(tgt, np.uint32), rt), what
    got = [weight_text(x) for x in w]
    bad = [i for i in range(len(got)) if got[i] != rw[i]]
    assert not bad, "%s: weight %s vs %s at edge %d" % (what, got[bad[0]], rw[bad[0]], bad[0])


def reps_from_edges(src, tgt, n):
    """Cluster representatives of a level whose clustering is singletons:
    every node with an edge."""
    reps = np.zeros(n, np.uint8)
    reps[np.asarray(src, np.int64)] = 1
    reps[np.asarray(tgt, np.int64)] = 1
    return reps
