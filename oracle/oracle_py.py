"""ctypes wrapper of the restated CPU oracle (oracle/build/liboracle.so) and
readers for the reference dump format.  TEST INFRASTRUCTURE: imported only by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker; the product never uses it.
"""
import ctypes
import os
import struct

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
REC = np.dtype([("hdr", "<u4"), ("ch", "<u4", (8,)), ("cl", "u1", (8,)), ("inv", "u1"), ("pad", "u1", (3,))])


class _OraStats(ctypes.Structure):
    _fields_ = [
        ("n_total_voxels", ctypes.c_uint64),
        ("n_nodes_svo", ctypes.c_uint64),
        ("n_nodes_last_lev_svo", ctypes.c_uint64),
        ("n_nodes_dag", ctypes.c_uint64),
        ("n_nodes_sdag", ctypes.c_uint64),
        ("n_nodes", ctypes.c_uint64),
        ("n_cross_level_merged", ctypes.c_uint64),
        ("n_missing_correspondences", ctypes.c_uint64),
        ("levels", ctypes.c_uint32),
        ("state", ctypes.c_uint32),
    ]


_VP, _U32, _U64, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
_SIGS = {
    "ora_create": (_VP, []),
    "ora_destroy": (None, [_VP]),
    "ora_clone": (_VP, [_VP]),
    "ora_build_svo": (_I, [_VP, _VP, _U64, _VP, _U32]),
    "ora_build_dag_chunked": (_I, [_VP, _VP, _U64, _VP, _U32, _U32, _I]),
    "ora_build_from_bricks": (_I, [_VP, _U32, _VP]),
    "ora_lossy_exact": (_I, [_VP, _U32, _U32, ctypes.c_double, ctypes.POINTER(_U64)]),
    "ora_refcount_order": (_I, [_VP, _U64, _VP]),
    "ora_ssvdag_traverse": (_I, [_VP, _U64, _VP, _U64, _VP, _U32, _U32, _VP, ctypes.c_float, _VP, _U64, _VP]),
    "ora_ssvdag_raycast": (_I, [_VP, _U64, _VP, _U64, _VP, _U32, _U32, _VP, ctypes.c_float, _VP, _VP, _U32, _U32,
                                _U32, _U32, ctypes.c_float, ctypes.c_float, ctypes.c_float, _VP]),
    "ora_flood_fill": (_I, [_VP, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "ora_get_outside": (_I, [_VP, _U32, _VP]),
    "ora_to_dag": (_I, [_VP]),
    "ora_to_sdag": (_I, [_VP]),
    "ora_to_sdag_ex": (_I, [_VP, _I]),
    "ora_init_child_levels": (_I, [_VP]),
    "ora_merge_across_levels": (_I, [_VP]),
    "ora_level_count": (_U64, [_VP, _U32]),
    "ora_get_level": (_I, [_VP, _U32, _VP]),
    "ora_get_stats": (_I, [_VP, ctypes.POINTER(_OraStats)]),
    "ora_tri_box": (_I, [_VP, ctypes.c_double, _VP]),
    # seeded scene generators (the same source as the product's host library)
    "svdag_synth_terrain_count": (_U64, [_U32]),
    "svdag_synth_terrain": (_I, [_U32, _U32, ctypes.c_double, _U64, _VP]),
    "svdag_synth_boxes": (_I, [_VP, _VP, _U64, _VP]),
}
_lib = None


def load():
    global _lib
    if _lib is None:
        p = os.path.join(ORACLE_DIR, "build", "liboracle.so")
        if not os.path.exists(p):
            raise RuntimeError("oracle/build/liboracle.so not built")
        lib = ctypes.CDLL(p)
        for k, (r, a) in _SIGS.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _lib = lib
    return _lib


def terrain(grid=2048, octaves=8, height=0.3, seed=7):
    """The seeded fBm terrain (float[9] per triangle), generated inside the
    oracle library: the CPU legs need no product library for their input."""
    L = load()
    out = np.empty((L.svdag_synth_terrain_count(grid), 9), np.float32)
    assert L.svdag_synth_terrain(grid, octaves, height, seed, out.ctypes.data) == 0
    return out


def boxes(lo, hi):
    L = load()
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    out = np.empty((lo.shape[0] * 12, 9), np.float32)
    assert L.svdag_synth_boxes(lo.ctypes.data, hi.ctypes.data, lo.shape[0], out.ctypes.data) == 0
    return out


def city(grid=4096, n_boxes=200000, levels=15, seed=15, octaves=8, height=0.3):
    """The depth-15 city scene (terrain + boxes), as the product's generator
    builds it; the box placement is the package's numpy code (no native
    library is loaded by importing it)."""
    import svdag_gb300 as sv  # pure Python at import time

    t = terrain(grid, octaves, height, seed)
    lo, hi = sv.city_box_extents(t, grid, n_boxes, levels, seed)
    return np.concatenate([t, boxes(lo, hi)])


class OracleOctree:
    def __init__(self, _h=None):
        self.L = load()
        self.h = _h if _h is not None else self.L.ora_create()

    def __del__(self):
        try:
            if self.h:
                self.L.ora_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def clone(self):
        return OracleOctree(self.L.ora_clone(self.h))

    def buildSVO(self, tris, levels, bbox=(0, 0, 0, 1, 1, 1)):
        tris = np.ascontiguousarray(tris, np.float32)
        bb = np.array(bbox, np.float64)
        assert self.L.ora_build_svo(self.h, tris.ctypes.data, tris.shape[0], bb.ctypes.data, levels) == 0

    def buildDAG(self, tris, levels, step_level, bbox=(0, 0, 0, 1, 1, 1), threads=0):
        tris = np.ascontiguousarray(tris, np.float32)
        bb = np.array(bbox, np.float64)
        assert self.L.ora_build_dag_chunked(self.h, tris.ctypes.data, tris.shape[0], bb.ctypes.data, levels,
                                            step_level, threads) == 0

    def buildFromBricks(self, depth, bricks):
        """Node pools of a voxel-brick grid (Morton order), DAG state."""
        bricks = np.ascontiguousarray(bricks, np.uint8)
        assert bricks.size == 8 ** (depth - 1)
        assert self.L.ora_build_from_bricks(self.h, depth, bricks.ctypes.data) == 0

    def lossyExact(self, min_above=3, max_above=5, max_error=0.01):
        """Lossy LSVDAG, exact-proposer form; returns the number of merged nodes."""
        m = ctypes.c_uint64()
        assert self.L.ora_lossy_exact(self.h, min_above, max_above, max_error, ctypes.byref(m)) == 0
        return m.value

    def hiddenGeometryFloodfill(self):
        """Outside masks of the SVO (list of u8 arrays, one per level) and the
        counts (empty cells reached, surface voxels marked); None when the
        start corner cell is set."""
        e, s = ctypes.c_uint64(), ctypes.c_uint64()
        r = self.L.ora_flood_fill(self.h, ctypes.byref(e), ctypes.byref(s))
        if r == -3:
            return None
        assert r == 0, r
        masks = []
        for l in range(self.stats()["levels"]):
            m = np.zeros(self.L.ora_level_count(self.h, l), np.uint8)
            self.L.ora_get_outside(self.h, l, m.ctypes.data)
            masks.append(m)
        return masks, e.value, s.value

    def toDAG(self):
        assert self.L.ora_to_dag(self.h) == 0

    def toSDAG(self, skip_symmetry=False):
        assert self.L.ora_to_sdag_ex(self.h, 1 if skip_symmetry else 0) == 0

    def initChildLevels(self):
        assert self.L.ora_init_child_levels(self.h) == 0

    def mergeAcrossAllLevels(self):
        assert self.L.ora_merge_across_levels(self.h) == 0

    def stats(self):
        s = _OraStats()
        self.L.ora_get_stats(self.h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in _OraStats._fields_}

    def level(self, l):
        n = self.L.ora_level_count(self.h, l)
        a = np.zeros(n, REC)
        if n:
            self.L.ora_get_level(self.h, l, a.ctypes.data)
        return a

    def pool(self):
        return [self.level(l) for l in range(self.stats()["levels"])]


def tri_box(center, half, tri):
    c = np.array(center, np.float64)
    t = np.ascontiguousarray(tri, np.float32)
    return bool(load().ora_tri_box(c.ctypes.data, half, t.ctypes.data))


def read_pool(path):
    """Reads a pool file written by ref_dump (layout in oracle/ref_dump.cpp)."""
    with open(path, "rb") as f:
        b = f.read()
    assert b[:4] == b"SVDP"
    ver, levels, state = struct.unpack_from("<III", b, 4)
    nvox, nn = struct.unpack_from("<QQ", b, 16)
    off = 32
    out = []
    for _ in range(levels):
        (n,) = struct.unpack_from("<Q", b, off)
        off += 8
        out.append(np.frombuffer(b, REC, n, off).copy())
        off += 48 * n
    return {"levels": levels, "state": state, "nvoxels": nvox, "nnodes": nn, "pool": out}


def pool_digest(pool):
    """SHA-256 over the concatenated level records (hdr, children, childLevels,
    invariant) -- the form the golden fixtures store."""
    import hashlib

    h = hashlib.sha256()
    for lev in pool:
        h.update(np.uint64(len(lev)).tobytes())
        h.update(np.ascontiguousarray(lev).tobytes())
    return h.hexdigest()


def read_ssvdag(path):
    """Fields of a .ssvdag file (EncodedSSVDAG::save layout)."""
    raw = open(path, "rb").read()
    o = 0
    bbox = np.frombuffer(raw, np.float32, 6, o); o += 24
    root_side = float(np.frombuffer(raw, np.float32, 1, o)[0]); o += 4
    levels, n_nodes = np.frombuffer(raw, np.uint32, 2, o); o += 8
    n = int(np.frombuffer(raw, np.uint32, 1, o)[0]); o += 4
    inner = np.frombuffer(raw, np.uint16, n, o).copy(); o += 2 * n
    n = int(np.frombuffer(raw, np.uint32, 1, o)[0]); o += 4
    leaves = np.frombuffer(raw, np.uint8, n, o).copy(); o += n
    n = int(np.frombuffer(raw, np.uint32, 1, o)[0]); o += 4
    offs = np.frombuffer(raw, np.uint32, n, o).copy()
    return {"bbox": bbox.copy(), "root_side": root_side, "levels": int(levels), "n_nodes": int(n_nodes),
            "inner": inner, "leaves": leaves, "level_offsets": offs}


def refcount_order(counts):
    """EncodedSSVDAG::encode's per-level order: std::sort of (index, count)
    pairs by count, descending (libstdc++, as the reference)."""
    c = np.ascontiguousarray(counts, np.uint32)
    out = np.empty(c.size, np.uint32)
    assert load().ora_refcount_order(c.ctypes.data, c.size, out.ctypes.data) == 0
    return out


def ssvdag_traverse(f, pts):
    """EncodedSSVDAG::traverse restated: depth reached per query point
    (-1 outside the box, -2 where a pointer leads outside the arrays)."""
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.empty(pts.shape[0], np.int32)
    inner, leaves, offs = f["inner"], f["leaves"], f["level_offsets"]
    rc = load().ora_ssvdag_traverse(inner.ctypes.data, inner.size, leaves.ctypes.data, leaves.size, offs.ctypes.data,
                                    offs.size, f["levels"], f["bbox"].ctypes.data, f["root_side"], pts.ctypes.data,
                                    pts.shape[0], out.ctypes.data)
    assert rc in (0, -2), rc
    return out

# one ray-cast pixel (the 32-byte hit record)
HIT = np.dtype([("t", "<f4"), ("level", "<i4"), ("iterations", "<i4"), ("node", "<i4"), ("voxel", "<i4", (3,)),
                ("normal", "<u4")])


def ssvdag_raycast(f, cam):
    """The viewer's SSVDAG ray traversal restated on the CPU: one hit record
    per pixel (row y = 0 at the bottom).  `cam` holds view_inv, proj_inv
    (column-major 16 floats), width, height, max_iters, draw_level,
    projection_factor, t_min, t_max.  Returns (hits, status): status -2 when
    a ray met a pointer outside the arrays."""
    inner, leaves, offs = f["inner"], f["leaves"], f["level_offsets"]
    bb = np.ascontiguousarray(f["bbox"], np.float32)
    vi = np.ascontiguousarray(cam["view_inv"], np.float32).ravel()
    pi = np.ascontiguousarray(cam["proj_inv"], np.float32).ravel()
    out = np.zeros(cam["width"] * cam["height"], HIT)
    rc = load().ora_ssvdag_raycast(inner.ctypes.data, inner.size, leaves.ctypes.data, leaves.size, offs.ctypes.data,
                                   offs.size, f["levels"], bb.ctypes.data, f["root_side"], vi.ctypes.data,
                                   pi.ctypes.data, cam["width"], cam["height"], cam["max_iters"], cam["draw_level"],
                                   cam["projection_factor"], cam["t_min"], cam["t_max"], out.ctypes.data)
    assert rc in (0, -2), rc
    return out, rc
