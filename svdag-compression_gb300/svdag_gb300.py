"""Python mirror of the GeomOctree build surface over the sm_103a C ABI.

``Octree`` follows the reference's GeomOctree call surface
(src/symvox/geom_octree.hpp:106-157): ``buildSVO`` / ``toDAG`` /
``initChildLevels`` / ``toSDAG`` / ``mergeAcrossAllLevels`` and the getters.
All compute runs in libsvdag_gpu.so on the GPU; there is no CPU fallback and
loading fails loudly when the library or a device is missing.

Node pools are returned per level as numpy structured arrays with the
48-byte record layout ``REC`` (hdr, children[8], childLevels[8], invariant).
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG_DIR, "lib")
NULL_NODE = 0xFFFFFFFE

REC = np.dtype([("hdr", "<u4"), ("ch", "<u4", (8,)), ("cl", "u1", (8,)), ("inv", "u1"), ("pad", "u1", (3,))])

STATES = {0: "S_EMPTY", 1: "S_SVO", 2: "S_DAG", 3: "S_SDAG"}


class SvdagError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("svdag status %d: %s" % (status, message))
        self.status = status


class _Stats(ctypes.Structure):
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
        ("svo_ms", ctypes.c_double),
        ("dag_ms", ctypes.c_double),
        ("sdag_ms", ctypes.c_double),
        ("csv_ms", ctypes.c_double),
        ("gpu_launches", ctypes.c_uint64),
        ("frontier_pairs", ctypes.c_uint64),
        ("sat_fallbacks", ctypes.c_uint64),
    ]


# Every symbol include/svdag_gpu.h declares, with its ctypes signature.
_VP, _U32, _U64, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
GPU_SYMBOLS = {
    "svdag_create": (_I, [ctypes.POINTER(_VP), _I, _VP]),
    "svdag_destroy": (_I, [_VP]),
    "svdag_clone": (_I, [_VP, ctypes.POINTER(_VP)]),
    "svdag_clone_on": (_I, [_VP, _VP, ctypes.POINTER(_VP)]),
    "svdag_last_error": (ctypes.c_char_p, [_VP]),
    "svdag_status_string": (ctypes.c_char_p, [_I]),
    "svdag_synchronize": (_I, [_VP]),
    "svdag_set_persistent_blocks": (_I, [_VP, _U32]),
    "svdag_upload_triangles": (_I, [_VP, _VP, _U64]),
    "svdag_set_device_triangles": (_I, [_VP, _VP, _U64]),
    "svdag_voxelize": (_I, [_VP, _U32, _VP]),
    "svdag_build_dag": (_I, [_VP, _U32, _U32, _VP]),
    "svdag_reduce_dag": (_I, [_VP]),
    "svdag_sort_by_effective_refcount": (_I, [_VP]),
    "svdag_lossy_candidates": (_I, [_VP, _U32, ctypes.c_float, _I, _VP, _VP, _VP, _VP, _U64, ctypes.POINTER(_U64)]),
    "svdag_tri_box_children": (_I, [_VP, _VP, _VP, _VP, _U64, _VP, ctypes.POINTER(_U64)]),
    "svdag_init_child_levels": (_I, [_VP]),
    "svdag_reduce_sdag": (_I, [_VP]),
    "svdag_reduce_sdag_ex": (_I, [_VP, _U32]),
    "svdag_voxelize_ex": (_I, [_VP, _U32, _VP, _U32]),
    "svdag_download_leaf_centers": (_I, [_VP, _VP, _U64, ctypes.POINTER(_U64)]),
    "svdag_cross_level_merge": (_I, [_VP]),
    "svdag_level_count": (_I, [_VP, _U32, ctypes.POINTER(_U64)]),
    "svdag_download_level": (_I, [_VP, _U32, _VP, _VP, _VP, _VP]),
    "svdag_get_stats": (_I, [_VP, ctypes.POINTER(_Stats)]),
    "svdag_level_device_ptrs": (_I, [_VP, _U32, _VP, _VP, _VP, _VP]),
    "svdag_import_begin": (_I, [_VP, _U32, _VP, ctypes.c_double, _U64]),
    "svdag_import_level": (_I, [_VP, _U32, _U64, _VP, _VP]),
    "svdag_profile_enable": (_I, [_VP, _I]),
    "svdag_profile_report": (_I, [_VP, ctypes.c_char_p, _U64]),
    "svdag_reduce_dag_noalloc": (_I, [_VP]),
    "svdag_device_alloc_count": (_U64, []),
    "svdag_flood_fill": (_I, [_VP, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "svdag_download_outside_masks": (_I, [_VP, _U32, _VP]),
    "svdag_synth_noise_bricks": (_I, [_VP, _U32, _U64, ctypes.c_double, _VP, ctypes.POINTER(ctypes.c_float)]),
    "svdag_import_bricks": (_I, [_VP, _U32, _VP]),
    "svdag_batch_create": (_I, [ctypes.POINTER(_VP), _I, _VP]),
    "svdag_batch_destroy": (_I, [_VP]),
    "svdag_batch_last_error": (ctypes.c_char_p, [_VP]),
    "svdag_batch_clear": (_I, [_VP]),
    "svdag_batch_add_chunk": (_I, [_VP, _U32, _VP]),
    "svdag_batch_chunk_count": (_I, [_VP, ctypes.POINTER(_U32)]),
    "svdag_batch_build": (_I, [_VP, _U32]),
    "svdag_batch_result": (_I, [_VP, _U32, _U32, ctypes.POINTER(_VP)]),
    "svdag_batch_set_tuning": (_I, [_VP, _VP]),
    "svdag_batch_get_tuning": (_I, [_VP, _VP]),
    "svdag_batch_autotune": (_I, [_VP, _U32, _U32]),
    "svdag_batch_get_stats": (_I, [_VP, _VP]),
    "svdag_lossy_dag": (_I, [_VP, _VP, _VP]),
    "svdag_encode": (_I, [_VP, _U32, _VP, _U64, ctypes.POINTER(_U64)]),
    "svdag_encode_ssvdag": (_I, [_VP, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U32)]),
    "svdag_download_ssvdag": (_I, [_VP, _VP, _VP, _VP]),
    "svdag_refcount_order": (_I, [_VP, _VP, _U64, _VP]),
    "svdag_ssvdag_traverse": (_I, [_VP, _U64, _VP, _U64, _VP, _U32, _U32, _VP, ctypes.c_float, _VP, _U64, _VP]),
    "svdag_ssvdag_upload": (_I, [_VP, _U64, _VP, _U64, _VP, _U32, _U32, _VP, ctypes.c_float, ctypes.POINTER(_VP)]),
    "svdag_ssvdag_free": (_I, [_VP]),
    "svdag_ssvdag_raycast": (_I, [_VP, _VP, _VP, _VP, _I]),
    "svdag_mlp_create": (_I, [ctypes.POINTER(_VP), _I, _U64]),
    "svdag_mlp_destroy": (_I, [_VP]),
    "svdag_mlp_param_count": (_U64, []),
    "svdag_mlp_get_params": (_I, [_VP, _VP]),
    "svdag_mlp_set_params": (_I, [_VP, _VP]),
    "svdag_mlp_loss_grad": (_I, [_VP, _VP, _VP, _VP, _U32, _VP, _VP]),
    "svdag_mlp_embed": (_I, [_VP, _VP, _U32, _VP]),
}


class LossyParams(ctypes.Structure):
    _fields_ = [("levels_above_min", ctypes.c_uint32), ("levels_above_max", ctypes.c_uint32),
                ("max_error", ctypes.c_double), ("proposer", ctypes.c_uint32), ("top_k", ctypes.c_uint32),
                ("train_pairs", ctypes.c_uint64), ("train_epochs", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("train_batch", ctypes.c_uint32), ("train_lr", ctypes.c_float)]


class _LossyStats(ctypes.Structure):
    _fields_ = [("nodes_before", ctypes.c_uint64), ("nodes_after", ctypes.c_uint64), ("candidates", ctypes.c_uint64),
                ("pairs_evaluated", ctypes.c_uint64), ("edges", ctypes.c_uint64), ("merged", ctypes.c_uint64),
                ("ms", ctypes.c_double), ("propose_ms", ctypes.c_double), ("train_ms", ctypes.c_double),
                ("final_loss", ctypes.c_float)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("table_factor", ctypes.c_double), ("threads", ctypes.c_uint32), ("streams", ctypes.c_uint32)]


class _BatchStats(ctypes.Structure):
    _fields_ = [("dag_ms", ctypes.c_double), ("reduce_ms", ctypes.c_double), ("gpu_launches", ctypes.c_uint64),
                ("table_retries", ctypes.c_uint64)]

HOST_SYMBOLS = {
    "svdag_synth_icosphere_count": (_U64, [_U32]),
    "svdag_synth_icosphere": (_I, [_U32, ctypes.c_double, ctypes.c_double, _U64, _VP]),
    "svdag_synth_terrain_count": (_U64, [_U32]),
    "svdag_synth_terrain": (_I, [_U32, _U32, ctypes.c_double, _U64, _VP]),
    "svdag_synth_boxes": (_I, [_VP, _VP, _U64, _VP]),
    "svdag_write_obj": (_I, [ctypes.c_char_p, _VP, _U64, _I]),
    "svdag_write_encoded": (_I, [ctypes.c_char_p, _I, _U32, _VP, _VP, _VP, ctypes.c_float, _U64, _I]),
    "svdag_scene_load_obj": (_I, [ctypes.c_char_p, _U32, _I, _I, ctypes.POINTER(_VP)]),
    "svdag_scene_triangle_count": (_U64, [_VP]),
    "svdag_scene_triangles": (_VP, [_VP]),
    "svdag_scene_bbox": (_I, [_VP, _VP]),
    "svdag_scene_free": (None, [_VP]),
}

FORMATS = {"svdag": 0, "ussvdag": 1, "ssvdag": 2}

_gpu = None
_host = None


def _bind(lib, table):
    for name, (res, args) in table.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def gpu_library_path():
    return os.path.join(LIB_DIR, "libsvdag_gpu.so")


def load_gpu():
    """Loads libsvdag_gpu.so (raises if it was not built)."""
    global _gpu
    if _gpu is None:
        p = gpu_library_path()
        if not os.path.exists(p):
            raise SvdagError(-1, "libsvdag_gpu.so not built (run __graft_entry__.build())")
        _gpu = _bind(ctypes.CDLL(p), GPU_SYMBOLS)
    return _gpu


def load_host():
    global _host
    if _host is None:
        p = os.path.join(LIB_DIR, "libsvdag_host.so")
        if not os.path.exists(p):
            raise SvdagError(-1, "libsvdag_host.so not built (run __graft_entry__.build())")
        _host = _bind(ctypes.CDLL(p), HOST_SYMBOLS)
    return _host


# --------------------------------------------------------------------------
# seeded synthetic scenes (host)

def icosphere(subdiv=5, radius=0.4, amp=0.08, seed=1234):
    h = load_host()
    n = h.svdag_synth_icosphere_count(subdiv)
    out = np.empty((n, 9), np.float32)
    if h.svdag_synth_icosphere(subdiv, radius, amp, seed, out.ctypes.data) != 0:
        raise SvdagError(-1, "icosphere synthesis failed")
    return out


def terrain(grid=2048, octaves=8, height=0.3, seed=7):
    h = load_host()
    n = h.svdag_synth_terrain_count(grid)
    out = np.empty((n, 9), np.float32)
    if h.svdag_synth_terrain(grid, octaves, height, seed, out.ctypes.data) != 0:
        raise SvdagError(-1, "terrain synthesis failed")
    return out


def boxes(lo, hi):
    h = load_host()
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    n = lo.shape[0]
    out = np.empty((n * 12, 9), np.float32)
    h.svdag_synth_boxes(lo.ctypes.data, hi.ctypes.data, n, out.ctypes.data)
    return out


def city(grid=4096, n_boxes=200000, levels=15, seed=15, octaves=8, height=0.3):
    """A procedural city on an fBm terrain: the terrain (grid x grid, skirts)
    followed by `n_boxes` seeded boxes with footprints of 8-256 voxels and
    log-normal heights (median 64 voxels) at a resolution of 2^levels,
    standing on the terrain (base 2 voxels below the lowest of the four
    terrain vertices around the box centre)."""
    t = terrain(grid, octaves, height, seed)
    lo, hi = city_box_extents(t, grid, n_boxes, levels, seed)
    return np.concatenate([t, boxes(lo, hi)])


def city_box_extents(t, grid, n_boxes, levels, seed):
    """The city's box corners (lo, hi: float arrays of n_boxes x 3) placed on
    the terrain triangles `t` (numpy only)."""
    n = grid
    cells = t[: 2 * (n - 1) ** 2].reshape(n - 1, n - 1, 2, 9)
    hgt = np.empty((n, n), np.float32)  # [j, i] -> y at grid vertex (i, j)
    hgt[:-1, :-1] = cells[:, :, 0, 1]   # a = (i, j)
    hgt[:-1, -1] = cells[:, -1, 0, 4]   # b = (i+1, j)
    hgt[-1, :-1] = cells[-1, :, 1, 7]   # d = (i, j+1)
    hgt[-1, -1] = cells[-1, -1, 0, 7]   # c = (i+1, j+1)
    rng = np.random.default_rng(seed)
    vox = 1.0 / (1 << levels)
    fx = rng.uniform(8, 256, n_boxes) * vox
    fz = rng.uniform(8, 256, n_boxes) * vox
    hy = rng.lognormal(np.log(64.0), 0.5, n_boxes) * vox
    cx = rng.uniform(fx / 2, 1 - fx / 2)
    cz = rng.uniform(fz / 2, 1 - fz / 2)
    gi = np.minimum((cx * (n - 1)).astype(np.int64), n - 2)
    gj = np.minimum((cz * (n - 1)).astype(np.int64), n - 2)
    base = np.minimum(np.minimum(hgt[gj, gi], hgt[gj, gi + 1]), np.minimum(hgt[gj + 1, gi], hgt[gj + 1, gi + 1]))
    base = np.maximum(base - 2 * vox, 0.0)
    lo = np.stack([cx - fx / 2, base, cz - fz / 2], axis=1)
    hi = np.stack([cx + fx / 2, np.minimum(base + hy, 1.0), cz + fz / 2], axis=1)
    return lo, hi


def write_obj(path, tris, pin_unit_cube=True):
    h = load_host()
    tris = np.ascontiguousarray(tris, np.float32)
    if h.svdag_write_obj(path.encode(), tris.ctypes.data, tris.shape[0], 1 if pin_unit_cube else 0) != 0:
        raise SvdagError(-1, "cannot write " + path)


UNIT_BOX = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)


def write_encoded(path, fmt, pool, n_nodes, state, bbox=UNIT_BOX, root_side=1.0):
    """Writes a node pool (list of REC arrays) in one of the reference's file
    formats: "svdag", "ussvdag" or "ssvdag" (also .esvdag from a DAG)."""
    h = load_host()
    pool = [np.ascontiguousarray(l, REC) for l in pool]
    counts = (ctypes.c_uint64 * len(pool))(*[len(l) for l in pool])
    ptrs = (ctypes.c_void_p * len(pool))(*[l.ctypes.data for l in pool])
    bb = (ctypes.c_float * 6)(*bbox)
    r = h.svdag_write_encoded(path.encode(), FORMATS[fmt], len(pool), counts, ptrs, bb, root_side, n_nodes, state)
    if r != 0:
        raise SvdagError(r, "cannot encode %s to %s" % (fmt, path))


# --------------------------------------------------------------------------
class Octree:
    """GPU octree with the GeomOctree build surface."""

    def __init__(self, device=0, stream=None, _handle=None, _owner=None):
        self._lib = load_gpu()
        self._owner = _owner  # a Batch whose result view this is (not destroyed here)
        if _handle is not None:
            self._h = _handle
        else:
            h = ctypes.c_void_p()
            self._check(self._lib.svdag_create(ctypes.byref(h), device, stream), None)
            self._h = h
        self._tris_ref = None

    def _check(self, status, h=-1):
        if status != 0:
            hh = self._h if h == -1 else h
            msg = self._lib.svdag_last_error(hh).decode() if hh else self._lib.svdag_status_string(status).decode()
            raise SvdagError(status, msg or self._lib.svdag_status_string(status).decode())

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owner", None) is None:
                self._lib.svdag_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # scene input
    def upload_triangles(self, tris):
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        self._check(self._lib.svdag_upload_triangles(self._h, tris.ctypes.data, tris.shape[0]))
        self._lib.svdag_synchronize(self._h)

    def set_device_triangles(self, dev_ptr, n_tris, keepalive=None):
        self._tris_ref = keepalive
        self._check(self._lib.svdag_set_device_triangles(self._h, ctypes.c_void_p(dev_ptr), n_tris))

    # GeomOctree surface
    def buildSVO(self, levels, bbox=UNIT_BOX, leaves_centers=False):
        """GeomOctree::buildSVO; with leaves_centers, returns its leavesCenters
        list (the fp64 centre of every leaf-level node, in node order) as an
        (n, 3) float64 array."""
        bb = (ctypes.c_double * 6)(*bbox)
        if not leaves_centers:
            self._check(self._lib.svdag_voxelize(self._h, levels, bb))
            return None
        self._check(self._lib.svdag_voxelize_ex(self._h, levels, bb, 1))
        n = _U64()
        self._check(self._lib.svdag_download_leaf_centers(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 3), np.float64)
        if n.value:
            self._check(self._lib.svdag_download_leaf_centers(self._h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def buildDAG(self, levels, step_level, bbox=UNIT_BOX):
        """GeomOctree::buildDAG: chunked build, DAG state, reference node order."""
        bb = (ctypes.c_double * 6)(*bbox)
        self._check(self._lib.svdag_build_dag(self._h, levels, step_level, bb))

    def import_bricks(self, depth, bricks):
        """Node pools of a voxel-brick chunk (a torch uint8 CUDA tensor of
        8^(depth-1) Morton-ordered bricks), DAG state."""
        self._check(self._lib.svdag_import_bricks(self._h, depth, ctypes.c_void_p(bricks.data_ptr())))

    def hiddenGeometryFloodfill(self):
        """Outside masks of the SVO (GeomOctree::hiddenGeometryFloodfill):
        one u8 array per level, and the counts (empty cells reached, surface
        voxels marked)."""
        e, s = _U64(), _U64()
        self._check(self._lib.svdag_flood_fill(self._h, ctypes.byref(e), ctypes.byref(s)))
        masks = []
        for l in range(self.stats()["levels"]):
            n = _U64()
            self._check(self._lib.svdag_level_count(self._h, l, ctypes.byref(n)))
            m = np.zeros(n.value, np.uint8)
            if n.value:
                self._check(self._lib.svdag_download_outside_masks(self._h, l, m.ctypes.data))
            masks.append(m)
        return masks, e.value, s.value

    def toDAG(self):
        self._check(self._lib.svdag_reduce_dag(self._h))

    def triBoxChildren(self, tris, centers, half_sides):
        """testTriBox of the 8 children of each (triangle, node) pair on the
        GPU (svdag_tri_box_children): (u8 masks, fp64 fallback count)."""
        tris = np.ascontiguousarray(tris, np.float32)
        centers = np.ascontiguousarray(centers, np.float64)
        half_sides = np.ascontiguousarray(half_sides, np.float64)
        n = tris.shape[0]
        assert centers.shape == (n, 3) and half_sides.shape == (n,)
        out = np.zeros(n, np.uint8)
        fb = _U64()
        self._check(self._lib.svdag_tri_box_children(self._h, tris.ctypes.data, centers.ctypes.data,
                                                     half_sides.ctypes.data, n, out.ctypes.data, ctypes.byref(fb)))
        return out, fb.value

    def encode(self, fmt="svdag"):
        """The EncodedSVDAG ("svdag") or EncodedUSSVDAG ("ussvdag") word
        stream, encoded on the GPU (svdag_encode)."""
        f = {"svdag": 0, "ussvdag": 1}[fmt]
        n = ctypes.c_uint64()
        self._check(self._lib.svdag_encode(self._h, f, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.uint32)
        self._check(self._lib.svdag_encode(self._h, f, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def encode_ssvdag(self):
        """EncodedSSVDAG::encode on the GPU (svdag_encode_ssvdag): the inner
        u16 words, the leaf bytes and the level offsets of the .ssvdag file."""
        ni, nl, no = _U64(), _U64(), _U32()
        self._check(self._lib.svdag_encode_ssvdag(self._h, ctypes.byref(ni), ctypes.byref(nl), ctypes.byref(no)))
        inner = np.empty(ni.value, np.uint16)
        leaves = np.empty(nl.value, np.uint8)
        offs = np.empty(no.value, np.uint32)
        self._check(self._lib.svdag_download_ssvdag(self._h, inner.ctypes.data, leaves.ctypes.data, offs.ctypes.data))
        return inner, leaves, offs

    def save_ssvdag(self, path, bbox=UNIT_BOX, root_side=1.0):
        """The .ssvdag file of this octree (EncodedSSVDAG::save layout)."""
        inner, leaves, offs = self.encode_ssvdag()
        head = np.array(bbox, np.float32).tobytes() + np.array([root_side], np.float32).tobytes()
        head += np.array([self.getLevels(), self.stats()["n_nodes"] & 0xFFFFFFFF], np.uint32).tobytes()
        with open(path, "wb") as f:
            f.write(head)
            for a in (inner, leaves, offs):
                f.write(np.array([a.size], np.uint32).tobytes())
                f.write(a.tobytes())

    def save_encoded(self, path, fmt="svdag", bbox=UNIT_BOX, root_side=1.0):
        """Writes the file the reference's saver writes for this stream."""
        words = self.encode(fmt)
        head = np.array(bbox, np.float32).tobytes() + np.array([root_side], np.float32).tobytes()
        head += np.array([self.getLevels(), self.stats()["n_nodes"] & 0xFFFFFFFF, words.size, words.size],
                         np.uint32).tobytes()
        with open(path, "wb") as f:
            f.write(head)
            f.write(words.tobytes())

    LOSSY = {"exact": 0, "learned": 1, "untrained": 2}

    def lossy(self, proposer="exact", min_above=3, max_above=5, max_error=0.01, top_k=0, train_pairs=0,
              epochs=0, seed=1, train_batch=0, lr=0.0):
        """Lossy LSVDAG on a DAG (svdag_lossy_dag); returns its statistics."""
        p = LossyParams(min_above, max_above, max_error, self.LOSSY[proposer], top_k, train_pairs, epochs, seed,
                        train_batch, lr)
        s = _LossyStats()
        self._check(self._lib.svdag_lossy_dag(self._h, ctypes.byref(p), ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _LossyStats._fields_}

    def sortByEffectiveRefCount(self):
        """GeomOctree::sortByEffectiveRefCount on the GPU."""
        self._check(self._lib.svdag_sort_by_effective_refcount(self._h))

    def lossyCandidates(self, level, diff_factor=1.0, included_ref_count=1, reps_below=None):
        """The reference toLossyDag's candidate edges at `level` (see
        svdag_lossy_candidates): (src, tgt, weight) arrays sorted by (src, tgt)."""
        reps = None if reps_below is None else np.ascontiguousarray(reps_below, np.uint8)
        rp = reps.ctypes.data if reps is not None else None
        cnt = _U64()
        self._check(self._lib.svdag_lossy_candidates(self._h, level, diff_factor, included_ref_count, rp, None, None,
                                                     None, 0, ctypes.byref(cnt)))
        n = cnt.value
        src, tgt, w = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(n, np.float32)
        if n:
            self._check(self._lib.svdag_lossy_candidates(self._h, level, diff_factor, included_ref_count, rp,
                                                         src.ctypes.data, tgt.ctypes.data, w.ctypes.data, n,
                                                         ctypes.byref(cnt)))
        return src, tgt, w

    def toDAG_noalloc(self):
        """toDAG with the library's static device scratch (no allocation);
        raises SvdagError (SVDAG_ERR_OVERFLOW) when a level does not fit."""
        self._check(self._lib.svdag_reduce_dag_noalloc(self._h))

    def initChildLevels(self):
        self._check(self._lib.svdag_init_child_levels(self._h))

    def toSDAG(self, skip_symmetry=False):
        """GeomOctree::toSDAG(false, skipSymmetry)."""
        self._check(self._lib.svdag_reduce_sdag_ex(self._h, 1 if skip_symmetry else 0))

    def mergeAcrossAllLevels(self):
        self._check(self._lib.svdag_cross_level_merge(self._h))
        return self.stats()["n_cross_level_merged"]

    def importDAG(self, pool, bbox=UNIT_BOX, root_side=1.0, n_total_voxels=0):
        """GeomOctree(NodeData, bbox, rootSide, levels, stats): a DAG from host
        pools (list of REC arrays, or (hdr, children) pairs per level)."""
        bb = (ctypes.c_float * 6)(*bbox)
        self._check(self._lib.svdag_import_begin(self._h, len(pool), bb, root_side, n_total_voxels))
        for l, lev in enumerate(pool):
            if isinstance(lev, np.ndarray) and lev.dtype == REC:
                hdr = np.ascontiguousarray(lev["hdr"])
                ch = np.ascontiguousarray(lev["ch"])
            else:
                hdr = np.ascontiguousarray(lev[0], np.uint32)
                ch = np.ascontiguousarray(lev[1], np.uint32)
            self._check(self._lib.svdag_import_level(self._h, l, len(hdr), hdr.ctypes.data, ch.ctypes.data))

    def set_persistent_blocks(self, blocks):
        """Cap the reduction kernels' grids at `blocks` SMs (0 = no cap), so
        that they share the GPU with work on other streams; clones inherit it."""
        self._check(self._lib.svdag_set_persistent_blocks(self._h, int(blocks)))

    def clone(self, stream=None):
        """Device-side copy (GeomOctree's copy constructor); on `stream` (a
        cudaStream_t handle) when given."""
        h = ctypes.c_void_p()
        if stream is None:
            self._check(self._lib.svdag_clone(self._h, ctypes.byref(h)))
        else:
            self._check(self._lib.svdag_clone_on(self._h, stream, ctypes.byref(h)))
        return Octree(_handle=h)

    # results
    def stats(self):
        s = _Stats()
        self._check(self._lib.svdag_get_stats(self._h, ctypes.byref(s)))
        d = {k: getattr(s, k) for k, _ in _Stats._fields_}
        d["state_name"] = STATES.get(d["state"], "?")
        return d

    def getLevels(self):
        return self.stats()["levels"]

    def level_count(self, level):
        n = ctypes.c_uint64()
        self._check(self._lib.svdag_level_count(self._h, level, ctypes.byref(n)))
        return n.value

    def level(self, level):
        n = self.level_count(level)
        hdr = np.zeros(n, np.uint32)
        ch = np.zeros((n, 8), np.uint32)
        cl = np.zeros((n, 8), np.uint8)
        inv = np.zeros(n, np.uint8)
        if n:
            self._check(self._lib.svdag_download_level(self._h, level, hdr.ctypes.data, ch.ctypes.data,
                                                       cl.ctypes.data, inv.ctypes.data))
        rec = np.zeros(n, REC)
        rec["hdr"], rec["ch"], rec["cl"], rec["inv"] = hdr, ch, cl, inv
        return rec

    def pool(self):
        return [self.level(l) for l in range(self.getLevels())]

    # per-kernel device timing
    def profile(self, enable=True):
        self._check(self._lib.svdag_profile_enable(self._h, 1 if enable else 0))

    def profile_report(self):
        """{kernel name: (launches, total_ms)} since the last report."""
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._lib.svdag_profile_report(self._h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.rsplit(";", 2)
            out[name] = (int(n), float(ms))
        return out

    def handle(self):
        return self._h.value


# --------------------------------------------------------------------------
# voxel-brick chunks

def device_alloc_count():
    """Stream-ordered device allocations the library has made in this process
    (svdag_device_alloc_count)."""
    return int(load_gpu().svdag_device_alloc_count())


def noise_bricks(depth, seed, fill, device=0):
    """Seeded synthetic chunk: a torch uint8 CUDA tensor of 8^(depth-1)
    Morton-ordered bricks with about `fill` of the voxels set."""
    import torch

    t = torch.empty(8 ** (depth - 1), dtype=torch.uint8, device="cuda:%d" % device)
    lib = load_gpu()
    thr = ctypes.c_float()
    st = torch.cuda.current_stream(device).cuda_stream
    r = lib.svdag_synth_noise_bricks(ctypes.c_void_p(st), depth, seed, fill, ctypes.c_void_p(t.data_ptr()),
                                     ctypes.byref(thr))
    if r != 0:
        raise SvdagError(r, "noise bricks failed")
    torch.cuda.synchronize(device)
    return t


class Batch:
    """Batched build of voxel-brick chunks (svdag_batch_*)."""

    RESULT = {"dag": 0, "sdag": 1, "csvdag": 2}

    def __init__(self, device=0, stream=None):
        self._lib = load_gpu()
        h = ctypes.c_void_p()
        r = self._lib.svdag_batch_create(ctypes.byref(h), device, stream)
        if r != 0:
            raise SvdagError(r, "batch create failed")
        self._h = h
        self._keep = []

    def _check(self, status):
        if status != 0:
            raise SvdagError(status, self._lib.svdag_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.svdag_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_chunk(self, depth, bricks):
        self._check(self._lib.svdag_batch_add_chunk(self._h, depth, ctypes.c_void_p(bricks.data_ptr())))
        self._keep.append(bricks)

    def clear(self):
        self._check(self._lib.svdag_batch_clear(self._h))
        self._keep = []

    def build(self, sdag=True, csvdag=True):
        self._check(self._lib.svdag_batch_build(self._h, (1 if sdag else 0) | (2 if csvdag else 0)))

    def result(self, chunk, kind="dag"):
        v = ctypes.c_void_p()
        self._check(self._lib.svdag_batch_result(self._h, chunk, self.RESULT[kind], ctypes.byref(v)))
        return Octree(_handle=v, _owner=self)

    def tuning(self):
        t = BatchTuning()
        self._check(self._lib.svdag_batch_get_tuning(self._h, ctypes.byref(t)))
        return {"table_factor": t.table_factor, "threads": t.threads, "streams": t.streams}

    def set_tuning(self, table_factor=2.0, threads=256, streams=4):
        t = BatchTuning(table_factor, threads, streams)
        self._check(self._lib.svdag_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, sdag=True, csvdag=True, max_trials=12):
        self._check(self._lib.svdag_batch_autotune(self._h, (1 if sdag else 0) | (2 if csvdag else 0), max_trials))

    def stats(self):
        s = _BatchStats()
        self._check(self._lib.svdag_batch_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _BatchStats._fields_}


class Mlp:
    """The lossy proposer's network on host buffers (svdag_mlp_*)."""

    def __init__(self, seed=1, device=0):
        self._lib = load_gpu()
        h = ctypes.c_void_p()
        r = self._lib.svdag_mlp_create(ctypes.byref(h), device, seed)
        if r != 0:
            raise SvdagError(r, "mlp create failed")
        self._h = h
        self.n_params = int(self._lib.svdag_mlp_param_count())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.svdag_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        out = np.empty(self.n_params, np.float32)
        assert self._lib.svdag_mlp_get_params(self._h, out.ctypes.data) == 0
        return out

    def set_params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert self._lib.svdag_mlp_set_params(self._h, w.ctypes.data) == 0

    def loss_grad(self, xa, xb, t):
        xa = np.ascontiguousarray(xa, np.float32)
        xb = np.ascontiguousarray(xb, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_float()
        g = np.empty(self.n_params, np.float32)
        r = self._lib.svdag_mlp_loss_grad(self._h, xa.ctypes.data, xb.ctypes.data, t.ctypes.data, t.shape[0],
                                          ctypes.byref(loss), g.ctypes.data)
        if r != 0:
            raise SvdagError(r, "mlp loss_grad failed")
        return loss.value, g

    def embed(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty((x.shape[0], 64), np.float32)
        r = self._lib.svdag_mlp_embed(self._h, x.ctypes.data, x.shape[0], out.ctypes.data)
        if r != 0:
            raise SvdagError(r, "mlp embed failed")
        return out


def ssvdag_traverse(f, pts):
    """GPU point queries of an encoded SSVDAG (fields as read from a .ssvdag
    file: inner, leaves, level_offsets, levels, bbox, root_side)."""
    lib = load_gpu()
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.empty(pts.shape[0], np.int32)
    bb = np.ascontiguousarray(f["bbox"], np.float32)
    r = lib.svdag_ssvdag_traverse(f["inner"].ctypes.data, f["inner"].size, f["leaves"].ctypes.data, f["leaves"].size,
                                  f["level_offsets"].ctypes.data, f["level_offsets"].size, f["levels"], bb.ctypes.data,
                                  f["root_side"], pts.ctypes.data, pts.shape[0], out.ctypes.data)
    if r != 0:
        raise SvdagError(r, "ssvdag traverse failed")
    return out


def refcount_order(counts, device=0):
    """The order EncodedSSVDAG::encode gives one level's nodes: the indices of
    (index, count) pairs after the reference's std::sort by count, descending
    (src/symvox/encoded_ssvdag.cpp:266-276), computed on the GPU.  `counts`:
    host array of u32 pointer counts; returns the u32 order on the host."""
    import torch

    c = np.ascontiguousarray(counts, np.uint32)
    n = c.size
    dev = "cuda:%d" % device
    d_counts = torch.from_numpy(c.view(np.int32)).to(dev)
    d_order = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    lib = load_gpu()
    st = torch.cuda.current_stream(device).cuda_stream
    r = lib.svdag_refcount_order(ctypes.c_void_p(st), ctypes.c_void_p(d_counts.data_ptr()), n,
                                 ctypes.c_void_p(d_order.data_ptr()))
    if r != 0:
        raise SvdagError(r, "refcount order failed")
    return d_order[:n].cpu().numpy().view(np.uint32)


# --------------------------------------------------------------------------
# ray casting of encoded SSVDAGs

# one pixel's result (svdag_ray_hit)
HIT = np.dtype([("t", "<f4"), ("level", "<i4"), ("iterations", "<i4"), ("node", "<i4"), ("voxel", "<i4", (3,)),
                ("normal", "<u4")])


class _Camera(ctypes.Structure):
    _fields_ = [
        ("view_inv", ctypes.c_float * 16),
        ("proj_inv", ctypes.c_float * 16),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("max_iters", ctypes.c_uint32),
        ("draw_level", ctypes.c_uint32),
        ("projection_factor", ctypes.c_float),
        ("t_min", ctypes.c_float),
        ("t_max", ctypes.c_float),
    ]


def camera(eye, target, width, height, levels, up=(0.0, 1.0, 0.0), fovy_deg=60.0, near=0.01, far=100.0,
           pixel_tolerance=1.0, max_iters=300):
    """A perspective camera as the viewer sets one up: gluLookAt /
    gluPerspective matrices inverted (column-major floats), the viewer's
    default 60-degree field of view, 300 iterations, full draw level, and
    OctreeDDARenderer::getProjectionFactor for the pixel tolerance."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    sd = np.cross(f, up)
    sd /= np.linalg.norm(sd)
    u = np.cross(sd, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = sd, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    fovy = np.float32(fovy_deg * 3.14159265359 / 180.0)
    g = 1.0 / np.tan(float(fovy) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0] = g / (width / height)
    proj[1, 1] = g
    proj[2, 2] = (far + near) / (near - far)
    proj[2, 3] = 2 * far * near / (near - far)
    proj[3, 2] = -1.0
    inv2tan = np.float32(1.0) / (np.float32(2.0) * np.float32(np.tan(np.float32(0.5) * fovy)))
    tol = np.float32(pixel_tolerance) / np.float32(height)
    return {"view_inv": np.linalg.inv(view).T.astype(np.float32).ravel(),
            "proj_inv": np.linalg.inv(proj).T.astype(np.float32).ravel(),
            "width": int(width), "height": int(height), "max_iters": int(max_iters), "draw_level": int(levels),
            "projection_factor": float(inv2tan / tol), "t_min": 0.0, "t_max": 1e30}


def _camera_struct(cam):
    c = _Camera()
    c.view_inv[:] = [float(x) for x in np.asarray(cam["view_inv"], np.float32).ravel()]
    c.proj_inv[:] = [float(x) for x in np.asarray(cam["proj_inv"], np.float32).ravel()]
    for k in ("width", "height", "max_iters", "draw_level", "projection_factor", "t_min", "t_max"):
        setattr(c, k, cam[k])
    return c


class Ssvdag:
    """An encoded SSVDAG (the arrays of a .ssvdag file, as read_ssvdag
    returns them) resident on the current CUDA device."""

    def __init__(self, f):
        self._lib = load_gpu()
        self.h = _VP()
        bb = np.ascontiguousarray(f["bbox"], np.float32)
        self.levels = int(f["levels"])
        r = self._lib.svdag_ssvdag_upload(f["inner"].ctypes.data, f["inner"].size, f["leaves"].ctypes.data,
                                          f["leaves"].size, f["level_offsets"].ctypes.data, f["level_offsets"].size,
                                          f["levels"], bb.ctypes.data, f["root_side"], ctypes.byref(self.h))
        if r != 0:
            raise SvdagError(r, "ssvdag upload failed")

    def close(self):
        if self.h:
            self._lib.svdag_ssvdag_free(self.h)
            self.h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def raycast(self, cam):
        """One hit record per pixel (row y = 0 at the bottom), host array."""
        out = np.zeros(cam["width"] * cam["height"], HIT)
        c = _camera_struct(cam)
        r = self._lib.svdag_ssvdag_raycast(self.h, ctypes.byref(c), None, out.ctypes.data, 0)
        if r != 0:
            raise SvdagError(r, "ssvdag raycast failed")
        return out

    def raycast_device(self, cam, hits_ptr, stream_ptr=None):
        """Ray cast into a device buffer of width * height * 32 bytes."""
        c = _camera_struct(cam)
        r = self._lib.svdag_ssvdag_raycast(self.h, ctypes.byref(c), stream_ptr, hits_ptr, 1)
        if r != 0:
            raise SvdagError(r, "ssvdag raycast failed")


def write_depth_pgm(path, hits, width, height):
    """The hit distances as a 16-bit binary PGM (nearest white, misses
    black), top row first -- the headless stand-in for the viewer's window."""
    t = hits["t"].reshape(height, width)[::-1]
    ok = t > 0
    img = np.zeros((height, width), np.uint16)
    if ok.any():
        lo, hi = float(t[ok].min()), float(t[ok].max())
        img[ok] = (65535 - (t[ok] - lo) / max(hi - lo, 1e-30) * 60000).astype(np.uint16)
    with open(path, "wb") as fh:
        fh.write(b"P5\n%d %d\n65535\n" % (width, height))
        fh.write(img.astype(">u2").tobytes())


def load_obj(path, threads=0, use_bincache=False, write_bincache=False):
    """Scene::loadObj on `threads` host threads (0: all cores): the triangle
    soup (n, 9) float32 and the scene bounding box (6 floats)."""
    lib = load_host()
    h = _VP()
    r = lib.svdag_scene_load_obj(os.fsencode(path), threads, int(use_bincache), int(write_bincache), ctypes.byref(h))
    if r != 0:
        raise SvdagError(r, "cannot load %s" % path)
    try:
        n = lib.svdag_scene_triangle_count(h)
        tris = np.zeros((n, 9), np.float32)
        if n:
            ctypes.memmove(tris.ctypes.data, lib.svdag_scene_triangles(h), 36 * n)
        bb = np.zeros(6, np.float32)
        lib.svdag_scene_bbox(h, bb.ctypes.data)
    finally:
        lib.svdag_scene_free(h)
    return tris, bb
