"""Restatement of the candidate-edge stage of the reference's lossy LSVDAG
(TEST INFRASTRUCTURE: the tests check it against edges the reference's own
toLossyDag wrote, and the GPU stage against both; the product never uses
it).  Pure Python over node pools as oracle_py returns them (REC records);
meant for the small test scenes.

  sort_by_effective_refcount  GeomOctree::sortByEffectiveRefCount
                              (src/symvox/geom_octree_extension.cpp:521-620)
  candidate_edges             toLossyDag's edges of one level (:904-1049),
                              computeNodeHash (:34-74), diffSubtrees (:294-368)
"""
import math

import numpy as np

import oracle_py

NULL = 0xFFFFFFFE
M64 = (1 << 64) - 1


def _mask(rec):
    return int(rec["hdr"]) & 0xFF


def effective_refcounts(pool):
    """Root paths to every node, summed in 32-bit unsigned arithmetic."""
    rc = [np.ones(1, np.uint64)]
    for lev in range(1, len(pool)):
        cur = np.zeros(len(pool[lev]), np.uint64)
        par = pool[lev - 1]
        for p in range(len(par)):
            for c in par["ch"][p]:
                if c != NULL:
                    cur[c] = (cur[c] + rc[lev - 1][p]) & 0xFFFFFFFF
        rc.append(cur)
    return [r.astype(np.uint32) for r in rc]


def sort_by_effective_refcount(pool):
    """The levels reordered as the reference's std::sort by effective count
    (descending; libstdc++'s unstable order through oracle_py.refcount_order),
    children renamed; returns (pool, refcounts in the new order)."""
    rc = effective_refcounts(pool)
    out = [None] * len(pool)
    out_rc = [None] * len(pool)
    ind = None
    for lev in range(len(pool) - 1, -1, -1):
        lv = pool[lev].copy()
        n = len(lv)
        order = oracle_py.refcount_order(rc[lev]) if lev > 0 and n else np.arange(n, dtype=np.uint32)
        if lev + 1 < len(pool):
            for i in range(n):
                m = _mask(lv[i])
                for c in range(8):
                    if (m >> c) & 1:
                        lv["ch"][i][c] = ind[lv["ch"][i][c]]
        out[lev] = lv[order]
        out_rc[lev] = rc[lev][order]
        ind = np.empty(n, np.uint32)
        ind[order] = np.arange(n, dtype=np.uint32)
    return out, out_rc


def node_hash(pool, lev, i, depth):
    """computeNodeHash(node, depth) with libstdc++'s identity std::hash."""
    rec = pool[lev][i]
    if depth == 0:
        return _mask(rec)
    key = 0
    if depth == 1:
        for c in range(8):
            key = (key << 8) & M64
            ch = int(rec["ch"][c])
            if ch != NULL:
                key = (key + _mask(pool[lev + 1][ch])) & M64
        return key
    for c in range(8):
        o = key
        h = (o << (c + 1)) & M64
        ch = int(rec["ch"][c])
        if ch != NULL:
            h = node_hash(pool, lev + 1, ch, depth - 1)
        key = (((o << 1) & M64) ^ h) ^ o
    return key


def diff_subtrees(pool, lev, a, b, abort_at, acc):
    """diffSubtrees(lev, lev, A, B, abort_at, acc, leaves): returns the new
    (acc, leaves delta) with the reference's early exits."""
    L = len(pool)
    leaves = 0
    ma, mb = _mask(pool[lev][a]), _mask(pool[lev][b])
    if lev == L - 1:
        d = bin(ma ^ mb).count("1")
        acc += d
        if d > 4:
            acc += abort_at + 1
        return acc, 1
    for i in range(8):
        ea, eb = (ma >> i) & 1, (mb >> i) & 1
        if ea != eb:
            if lev == L - 2:
                child = int(pool[lev]["ch"][a if ea else b][i])
                d = bin(_mask(pool[lev + 1][child])).count("1")
                leaves += 1
                acc += d
                if d > 4:
                    acc += abort_at + 1
                    return acc, leaves
                continue
            acc += abort_at
            return acc, leaves
        if not ea:
            continue
        acc, lv = diff_subtrees(pool, lev + 1, int(pool[lev]["ch"][a][i]), int(pool[lev]["ch"][b][i]), abort_at, acc)
        leaves += lv
        if acc >= abort_at:
            return acc, leaves
    return acc, leaves


def candidate_edges(pool, rc, lev, diff_factor, included, reps_below=None):
    """toLossyDag's candidate edges of level `lev` of a sorted DAG: sorted
    list of (src, tgt, weight as float32)."""
    L = len(pool)
    depth = max(L - lev - 2, 1)
    keys = [node_hash(pool, lev, i, depth) for i in range(len(pool[lev]))]
    groups = {}
    for i, k in enumerate(keys):
        groups.setdefault(k, []).append(i)
    # std::round (halves away from zero) of the double product (:901)
    max_diff = int(math.floor((L - lev) ** 2 * float(np.float32(diff_factor)) + 0.5))
    edges = []
    for a in range(len(pool[lev])):
        if rc[lev][a] > included:
            continue
        if reps_below is not None:
            m = _mask(pool[lev][a])
            if any(reps_below[pool[lev]["ch"][a][c]] for c in range(8) if (m >> c) & 1):
                continue
        probes = [keys[a] ^ (1 << bit) for bit in range(64)] if lev == L - 2 else [keys[a]]
        for k in probes:
            for b in groups.get(k, []):
                if b >= a or rc[lev][b] > included:
                    continue
                if lev == L - 2:
                    edges.append((a, b, np.float32(1.0)))
                    continue
                acc, leaves = diff_subtrees(pool, lev, a, b, max_diff + 1, 0)
                if acc <= max_diff and np.float32(acc) < np.float32(4.0 * leaves):
                    w = np.float32(1.0) - np.float32(acc) / (np.float32(max_diff) + np.float32(1.0))
                    edges.append((a, b, np.float32(w)))
    edges.sort(key=lambda e: (e[0], e[1]))
    return edges
