/*
 * svdag_gpu.h -- C ABI of the GB300 (sm_103a) SVDAG construction path.
 *
 * Drop-in replacement for the compute of SymVox's GeomOctree build path:
 * voxelization into an SVO, bottom-up reduction to an SVDAG, the
 * symmetry-aware SSVDAG reduction and the cross-level CSVDAG merge.  Results
 * (node pools per level, counts, statistics) are bit-identical to the
 * reference's; only the place the work runs changes.
 *
 * Conventions
 *   - Every entry point returns an int status (SVDAG_OK == 0).  On failure
 *     svdag_last_error() gives a one-line reason.  The reference prints and
 *     returns on a wrong octree state (src/symvox/geom_octree.cpp:464-469,
 *     553-563); here that case is SVDAG_ERR_INVALID_STATE.
 *   - A context owns one CUDA stream and all device memory of one octree.
 *     It is not thread-safe: use one context per host thread, as the
 *     reference uses one GeomOctree per OpenMP thread
 *     (src/symvox/geom_octree.cpp:339).
 *   - Node records use the reference's node fields in fixed-width form:
 *       hdr       = childrenBitmask | mirX<<8 | mirY<<16 | mirZ<<24
 *       children  = 8 x u32 per node, 0xFFFFFFFE for no child
 *                   (Octree::nullNode, src/symvox/octree.cpp:22)
 *       childLevels = 8 x u8 per node (low byte of the reference's value,
 *                   0xFF when never initialised)
 *       invariant = u8 invariantBitmask (bit0 X, bit1 Y, bit2 Z)
 *     Child index c = 4x + 2y + z (src/symvox/octree.hpp:33-42).
 */
#ifndef SVDAG_GPU_H
#define SVDAG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum svdag_status {
  SVDAG_OK = 0,
  SVDAG_ERR_INVALID_ARG = 1,
  SVDAG_ERR_INVALID_STATE = 2,
  SVDAG_ERR_CUDA = 3,
  SVDAG_ERR_OOM = 4,
  SVDAG_ERR_OVERFLOW = 5,
  SVDAG_ERR_TIMEOUT = 6,
  SVDAG_ERR_NO_DEVICE = 7
};

/* GeomOctree::State (src/symvox/geom_octree.hpp:36-41) */
enum svdag_state { SVDAG_S_EMPTY = 0, SVDAG_S_SVO = 1, SVDAG_S_DAG = 2, SVDAG_S_SDAG = 3 };

typedef struct svdag_ctx svdag_ctx;

/* GeomOctree::Stats subset (src/symvox/geom_octree.hpp:43-56) plus device
 * times of each phase measured with CUDA events on the context stream. */
typedef struct svdag_stats {
  uint64_t n_total_voxels;
  uint64_t n_nodes_svo;
  uint64_t n_nodes_last_lev_svo;
  uint64_t n_nodes_dag;
  uint64_t n_nodes_sdag;
  uint64_t n_nodes;                 /* current node count (reference _nNodes) */
  uint64_t n_cross_level_merged;
  uint64_t n_missing_correspondences;
  uint32_t levels;
  uint32_t state;                   /* enum svdag_state */
  double svo_ms, dag_ms, sdag_ms, csv_ms;
  uint64_t gpu_launches;            /* kernels launched by this context */
  uint64_t frontier_pairs;          /* (triangle, node) visits of the last voxelization */
  uint64_t sat_fallbacks;           /* box predicates decided in fp64 (fp32 filter undecided) */
} svdag_stats;

/* Lifetime.  `stream` is a cudaStream_t to run on, or NULL for a new one. */
int svdag_create(svdag_ctx** out, int device, void* stream);
int svdag_destroy(svdag_ctx* ctx);
/* Device-side deep copy (same device and stream): lets one DAG feed both the
 * SSVDAG and the CSVDAG reductions, as GeomOctree's copy constructor does
 * (src/symvox/geom_octree.cpp:40-45). */
int svdag_clone(const svdag_ctx* src, svdag_ctx** out);
/* The same copy on `stream` (a cudaStream_t, or NULL for a new one), so that
 * two clones of one DAG -- the SSVDAG and the CSVDAG reductions -- can run
 * concurrently from two host threads. */
int svdag_clone_on(const svdag_ctx* src, void* stream, svdag_ctx** out);
const char* svdag_last_error(const svdag_ctx* ctx);
const char* svdag_status_string(int status);
int svdag_synchronize(svdag_ctx* ctx);

/* The reductions (toDAG, toSDAG, mergeAcrossAllLevels) each run as one
 * persistent cooperative kernel of at most one block per SM; a cooperative
 * launch starts only when its whole grid fits, so a full-GPU reduction waits
 * for (and then excludes) other work on the GPU.  This caps the context's
 * reduction grids at `blocks` SMs (0 = no cap, the default), leaving the
 * other SMs to work on other streams -- e.g. the next scene's voxelization
 * while this one's SSVDAG and CSVDAG reductions run.  Clones inherit it.
 * (No reference counterpart: a GPU scheduling knob.) */
int svdag_set_persistent_blocks(svdag_ctx* ctx, unsigned blocks);

/* Scene input: triangles as float[9] each (v0 v1 v2, xyz), the layout of
 * Scene::getTrianglePtr (src/symvox/scene.hpp:90).  upload copies from host
 * memory; set_device borrows a device buffer that must outlive the build. */
int svdag_upload_triangles(svdag_ctx* ctx, const float* host_tris, uint64_t n_tris);
int svdag_set_device_triangles(svdag_ctx* ctx, const float* device_tris, uint64_t n_tris);

/* GeomOctree::buildSVO(levels, bbox) (src/symvox/geom_octree.cpp:171-280):
 * bbox = {minx, miny, minz, maxx, maxy, maxz} in double, 1 <= levels <= 21. */
int svdag_voxelize(svdag_ctx* ctx, uint32_t levels, const double bbox[6]);
/* The same; with SVDAG_VOXELIZE_LEAF_CENTERS the build keeps buildSVO's
 * leavesCenters (geom_octree.cpp:245-246: the fp64 centre each leaf-level
 * node was created with, in node order; none for levels == 1), read with
 * svdag_download_leaf_centers until the next voxelization (count = the
 * leaf level's node count; capacity in centres, 3 doubles each; a capacity
 * below the count is SVDAG_ERR_OVERFLOW; NULL xyz only counts). */
enum { SVDAG_VOXELIZE_LEAF_CENTERS = 1 };
int svdag_voxelize_ex(svdag_ctx* ctx, uint32_t levels, const double bbox[6], uint32_t flags);
int svdag_download_leaf_centers(svdag_ctx* ctx, double* xyz, uint64_t capacity, uint64_t* count);
/* GeomOctree::buildDAG(levels, stepLevel, bbox) (src/symvox/geom_octree.cpp:289-435):
 * the chunked build svbuilder runs for numBuildSteps > 0
 * (src/svbuilder/main.cpp:158-175) -- a top SVO of stepLevel+1 levels, one
 * sub-octree (buildSVO + toDAG) per top-level voxel, joined in the
 * reference's order and reduced by one toDAG; leaves the octree in DAG state
 * with the reference's node order.  1 <= stepLevel < levels - 1. */
int svdag_build_dag(svdag_ctx* ctx, uint32_t levels, uint32_t step_level, const double bbox[6]);
/* testTriBox (src/symvox/test_triangle_box.cpp:105-184), as buildSVO calls
 * it for the 8 children of a visited node (geom_octree.cpp:222-262), for n
 * arbitrary (triangle, node) pairs: triangle i = tris[9i..9i+8], node centre
 * centers[3i..3i+2], child half side half_sides[i] (children centred at
 * centre +- half side per axis, child index 4x+2y+z).  Bit ci of masks[i] is
 * set when child ci overlaps the triangle.  The decisions come from the same
 * device code and the same decision sequence as the voxelizer's (certified
 * fp32 filter, fp64 fallback); fallbacks (may be NULL) receives the number of
 * predicates decided in fp64.  Host buffers; synchronous. */
int svdag_tri_box_children(svdag_ctx* ctx, const float* tris, const double* centers, const double* half_sides,
                           uint64_t n, uint8_t* masks, uint64_t* fallbacks);
/* GeomOctree::toDAG (src/symvox/geom_octree.cpp:462-548).  toDAG and toSDAG
 * rewrite the parent levels in place as they go: when either fails on the
 * device (SVDAG_ERR_OVERFLOW: hash probe limit; SVDAG_ERR_TIMEOUT: a grid
 * barrier of the persistent kernel ran out), the octree is left EMPTY and
 * must be rebuilt. */
int svdag_reduce_dag(svdag_ctx* ctx);
/* GeomOctree::sortByEffectiveRefCount (src/symvox/geom_octree_extension.cpp:
 * 521-620): every level of a DAG reordered by effective reference count
 * (root paths to the node, 32-bit unsigned sums), descending, in exactly the
 * order the reference's unstable std::sort gives, children renamed.  The
 * first step of toLossyDag (:887). */
int svdag_sort_by_effective_refcount(svdag_ctx* ctx);
/* The candidate edges toLossyDag (src/symvox/geom_octree_extension.cpp:
 * 904-1049) builds at `level` of a DAG in effective-reference-count order
 * (svdag_sort_by_effective_refcount), before its MCL clustering: for every
 * node A whose effective count is at most included_ref_count and that is not
 * a parent of a cluster representative of the level below (reps_below: one
 * byte per node of level + 1, non-zero = representative; NULL = none), each
 * earlier node B with such a count and the same node hash (computeNodeHash
 * at depth max(levels - level - 2, 1)) -- at levels - 2, a hash one bit away,
 * weight 1 -- whose subtree difference (diffSubtrees, with its abort rules)
 * is within round((levels - level)^2 * diff_factor) and below 4 per compared
 * leaf, weight 1 - diff / (max + 1).  Edges (src = A, tgt = B, weight) are
 * written sorted by (src, tgt); *count receives their number.  With
 * capacity 0 and NULL arrays the call only counts; a capacity below the
 * count is SVDAG_ERR_OVERFLOW.  1 <= level <= levels - 2. */
int svdag_lossy_candidates(svdag_ctx* ctx, uint32_t level, float diff_factor, int included_ref_count,
                           const uint8_t* reps_below, uint32_t* src, uint32_t* tgt, float* weight, uint64_t capacity,
                           uint64_t* count);
/* GeomOctree::initChildLevels (src/symvox/geom_octree_extension.cpp:21-30) */
int svdag_init_child_levels(svdag_ctx* ctx);
/* GeomOctree::toSDAG(false, false) (src/symvox/geom_octree.cpp:551-697).  On
 * an SVO (the reference's direct "SVO -> SDAG", :554-556) the result is the
 * one toDAG then toSDAG give -- the compiled reference's direct pass gives the
 * same pools -- and nNodesDAG is left as it was. */
int svdag_reduce_sdag(svdag_ctx* ctx);
/* GeomOctree::toSDAG(false, skipSymmetry): flags 0 is svdag_reduce_sdag;
 * SVDAG_SDAG_SKIP_SYMMETRY is the reference's pointer-compression-only form
 * (geom_octree.cpp:596-601): every non-empty node kept in order, no
 * invariance bits, no mirror lookups (a DAG's pools stay as they are; empty
 * nodes of imported pools and of an SVO are dropped, a pointer to one becomes
 * 0; an SVO's duplicates stay). */
enum { SVDAG_SDAG_SKIP_SYMMETRY = 1 };
int svdag_reduce_sdag_ex(svdag_ctx* ctx, uint32_t flags);
/* GeomOctree::mergeAcrossAllLevels (src/symvox/geom_octree_extension.cpp:1192-1544) */
int svdag_cross_level_merge(svdag_ctx* ctx);

/* GeomOctree(const NodeData&, bbox, rootSide, levels, stats)
 * (src/symvox/geom_octree.cpp:49-60): replaces the context's octree with host
 * node pools in DAG state -- the route a decoded .svdag input takes
 * (src/svbuilder/main.cpp:97-101).  import_begin sizes the tree; each level is
 * then given by import_level (children may be NULL on the leaf level). */
int svdag_import_begin(svdag_ctx* ctx, uint32_t levels, const float bbox[6], double root_side,
                       uint64_t n_total_voxels);
int svdag_import_level(svdag_ctx* ctx, uint32_t level, uint64_t count, const uint32_t* hdr,
                       const uint32_t* children);

/* Results.  Host buffers sized by svdag_level_count; any pointer may be NULL
 * to skip that field.  children/child_levels take 8 entries per node. */
int svdag_level_count(const svdag_ctx* ctx, uint32_t level, uint64_t* count);
int svdag_download_level(svdag_ctx* ctx, uint32_t level, uint32_t* hdr, uint32_t* children,
                         uint8_t* child_levels, uint8_t* invariant);
int svdag_get_stats(const svdag_ctx* ctx, svdag_stats* out);
/* Device pointers of one level's arrays (valid until the next build call on
 * the context); children is NULL on the leaf level. */
int svdag_level_device_ptrs(const svdag_ctx* ctx, uint32_t level, const uint32_t** hdr,
                            const uint32_t** children, const uint8_t** child_levels,
                            const uint8_t** invariant);

/* EncodedSVDAG::encode (src/symvox/encoded_svdag.cpp:105-199; DAG or CSVDAG
 * after initChildLevels) and EncodedUSSVDAG::encode (encoded_ussvdag.cpp:
 * 86-170; SDAG) on the GPU: the u32 stream that follows the file header.
 * host_words may be NULL to query the size.  The file is: bbox min, max
 * (6 floats), rootSide (float), levels (u32), nNodes (u32), the word count
 * twice (the reference's "first leaf pointer" field holds it), the words. */
enum { SVDAG_FORMAT_SVDAG = 0, SVDAG_FORMAT_USSVDAG = 1 };
int svdag_encode(svdag_ctx* ctx, uint32_t format, uint32_t* host_words, uint64_t capacity, uint64_t* n_words);

/* EncodedSSVDAG::encode (src/symvox/encoded_ssvdag.cpp:194-466) on the GPU
 * (DAG or SDAG state, not cross-level merged): the arrays of a .ssvdag file,
 * byte-identical to the reference's -- the level order is the one the
 * reference's std::sort over the pointer counts leaves (reproduced on the
 * GPU, see svdag_refcount_order), the packing runs on the GPU; nothing goes
 * through the host.  svdag_encode_ssvdag encodes and
 * reports the sizes (u16 inner words, leaf bytes, level offsets); the
 * result stays in the context until svdag_download_ssvdag copies it to host
 * buffers of those sizes (any may be NULL to skip it).  The file is: bbox
 * (6 floats), rootSide (float), levels (u32), nNodes (u32), then u32 count +
 * data for the inner words, the leaf bytes and the level offsets. */
int svdag_encode_ssvdag(svdag_ctx* ctx, uint64_t* n_inner_words, uint64_t* n_leaf_bytes, uint32_t* n_level_offsets);
int svdag_download_ssvdag(svdag_ctx* ctx, uint16_t* inner, uint8_t* leaves, uint32_t* level_offsets);

/* The per-level node order of EncodedSSVDAG::encode
 * (src/symvox/encoded_ssvdag.cpp:259-276): the (index, count) pairs
 * (i, counts[i]), sorted by std::sort with "count(a) > count(b)", exactly as
 * libstdc++'s (GCC 13) introsort orders them -- equal counts included, whose
 * order that unstable sort decides.  order[k] = index of the k-th pair.
 * Device buffers of n u32 each; runs on `stream` (0 = default) and returns
 * when the order is written.  n <= 2^31. */
int svdag_refcount_order(void* stream, const uint32_t* device_counts, uint64_t n, uint32_t* device_order);

/* EncodedSSVDAG::traverse (src/symvox/encoded_ssvdag.cpp:527-574) on the
 * GPU, one point query per thread: the depth each point reaches in an encoded
 * SSVDAG (the arrays of a .ssvdag file), `levels` when its voxel is set, -1
 * outside the box, -2 where a pointer leads outside the arrays (the call
 * then returns SVDAG_ERR_INVALID_ARG).  Host buffers; points as x, y, z
 * floats. */
int svdag_ssvdag_traverse(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                          const uint32_t* level_offsets, uint32_t n_level_offsets, uint32_t levels,
                          const float bbox[6], float root_side, const float* points, uint64_t n_points,
                          int32_t* depth);

/* Ray casting of an encoded SSVDAG: the viewer's DDA traversal
 * (shaders/octree_dda.frag.glsl:539-581, trace_ray, SSVDAG variant, as
 * OctreeDDARenderer feeds it, src/svviewer/octree_dda_renderer.cpp:199-223,
 * 391-422) into a headless buffer, one ray per pixel, pixel (x, y) at index
 * y * width + x with y = 0 the bottom row (gl_FragCoord).
 * svdag_ssvdag_upload copies the arrays of a .ssvdag file to the current
 * device (n_leaves a multiple of 8). */
typedef struct svdag_ssvdag svdag_ssvdag;
int svdag_ssvdag_upload(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                        const uint32_t* level_offsets, uint32_t n_level_offsets, uint32_t levels,
                        const float bbox[6], float root_side, svdag_ssvdag** out);
int svdag_ssvdag_free(svdag_ssvdag* s);

typedef struct svdag_camera {
  float view_inv[16];       /* inverse view matrix, column-major (glUniformMatrix4fv, no transpose) */
  float proj_inv[16];       /* inverse projection matrix, column-major */
  uint32_t width, height;   /* screenRes */
  uint32_t max_iters;       /* maxIters (the viewer's default: 300) */
  uint32_t draw_level;      /* drawLevel (the viewer's default: the level count) */
  float projection_factor;  /* projectionFactor (OctreeDDARenderer::getProjectionFactor) */
  float t_min, t_max;       /* the ray's t range in world units (the viewer: 0, 1e30) */
} svdag_camera;

/* One pixel: trace_ray's result -- t = hit distance in world units, or -1
 * (inside the box, no hit), -2 (past t_max), -3 (max_iters reached), -4
 * (outside the box), -5 (a pointer outside the arrays); level = the shader
 * level of the hit; iterations; node = node index of the hit (-1 none) --
 * plus the hit cell's grid coordinates at that level and the entry face
 * normal -stepDir as three signed bytes (x in the low byte). */
typedef struct svdag_ray_hit {
  float t;
  int32_t level, iterations, node;
  int32_t voxel[3];
  uint32_t normal;
} svdag_ray_hit;

/* hits: width * height records, in device memory when device_buffer != 0
 * (then on `stream`, or the handle's own stream when NULL), else host
 * memory.  Returns when the buffer is written; SVDAG_ERR_INVALID_ARG when a
 * ray met a pointer outside the arrays (its record has t = -5). */
int svdag_ssvdag_raycast(svdag_ssvdag* s, const svdag_camera* cam, void* stream, svdag_ray_hit* hits,
                         int device_buffer);

/* GeomOctree::hiddenGeometryFloodfill (src/symvox/geom_octree_extension.cpp:
 * 1651-1891) on an SVO (state SVO, before toDAG): each node's outsideMask --
 * bit c set when child slot c is an empty cell face-connected through empty
 * cells to the start cell (slot 7 of the deepest node on the child-7 path),
 * a set voxel sharing a face with such a cell, or a child node with any
 * outside bit.  n_outside_empty counts the empty cells reached (the start
 * included), n_outside_surface the set voxels marked; either may be NULL.
 * SVDAG_ERR_INVALID_STATE when the start cell is set (the reference aborts)
 * or the octree is not an SVO.  The masks are read per level with
 * svdag_download_outside_masks (one byte per node) while the SVO is
 * unchanged; toDAG and the other reductions do not use them. */
int svdag_flood_fill(svdag_ctx* ctx, uint64_t* n_outside_empty, uint64_t* n_outside_surface);
int svdag_download_outside_masks(svdag_ctx* ctx, uint32_t level, uint8_t* masks);

/* Per-kernel device timing (no counterpart in the reference, whose Stats
 * hold phase times only, src/symvox/geom_octree.hpp:54).  While enabled,
 * every kernel launch of the context is bracketed by CUDA events on its
 * stream.  The report is text, one line per kernel name:
 *   "<kernel>;<launches>;<total_ms>\n"
 * and reading it clears the accumulated records. */
int svdag_profile_enable(svdag_ctx* ctx, int enable);
int svdag_profile_report(svdag_ctx* ctx, char* buf, uint64_t capacity);
/* Number of stream-ordered device allocations (cudaMallocAsync) this library
 * has made in the process, over all contexts and threads; no counterpart in
 * the reference.  A diagnostic: the difference across a call shows whether
 * that call allocated device memory. */
uint64_t svdag_device_alloc_count(void);

/* ---- Voxel-brick chunks (no counterpart in the reference, which voxelizes
 * triangles only; a voxel grid enters it as node pools through
 * GeomOctree(const NodeData&, ...), src/symvox/geom_octree.cpp:49-60).
 *
 * A chunk of depth d (2..11) is a dense grid of 2^d voxels per side, given
 * as 8^(d-1) bricks (one byte = 2^3 voxels, bit 4x+2y+z) in Morton order
 * (x the most significant bit of each coordinate triple), in device memory
 * aligned to 8 bytes.  Its node pools: the non-empty bricks in Morton order
 * on level d-1, on each level above the non-empty cells of 8 consecutive
 * entries of the level below (child k = entry 8j+k), the root always present.
 *
 * Seeded synthetic chunk: 3D value noise (lattice period 16 voxels) below a
 * threshold chosen so that about `fill` of the voxels are set; writes the
 * threshold used when `threshold` is not NULL. */
int svdag_synth_noise_bricks(void* stream, uint32_t depth, uint64_t seed, double fill, uint8_t* device_bricks,
                             float* threshold);
/* The plain per-chunk form: the chunk's node pools into `ctx` (DAG state, as
 * the NodeData constructor leaves them); svdag_reduce_dag / reduce_sdag /
 * cross_level_merge then run on them. */
int svdag_import_bricks(svdag_ctx* ctx, uint32_t depth, const uint8_t* device_bricks);

/* The batched form: many chunks (of any depths) reduced together, height by
 * height (every chunk's leaves first), one launch per step for all chunks;
 * then toSDAG and the cross-level merge of each chunk on several streams.
 * Each chunk's results equal the plain form's (toDAG / toSDAG /
 * mergeAcrossAllLevels of its node pools).  Chunks are borrowed: their bricks
 * must stay valid until the build returns.  Result views are owned by the
 * batch and valid until the next build, clear or destroy: read them with
 * svdag_level_count / svdag_download_level / svdag_get_stats, or
 * svdag_clone them to work on; do not destroy them or run phases on them. */
typedef struct svdag_batch svdag_batch;
enum { SVDAG_BATCH_SDAG = 1, SVDAG_BATCH_CSVDAG = 2 };
enum { SVDAG_BATCH_RESULT_DAG = 0, SVDAG_BATCH_RESULT_SDAG = 1, SVDAG_BATCH_RESULT_CSVDAG = 2 };
typedef struct svdag_batch_tuning {
  double table_factor; /* hash slots per key of a height (rounded up to a power of two), 1.25..16: per cell
                          until a height has been seen, then per expected distinct key (twice the
                          largest share of distinct keys among the cells seen at that height) */
  uint32_t threads;    /* block size of the per-height kernels, 64..1024, multiple of 32 */
  uint32_t streams;    /* chunks reduced concurrently in the SSVDAG / CSVDAG stage, 1..64 */
} svdag_batch_tuning;
typedef struct svdag_batch_stats {
  double dag_ms;       /* wall time of the batched toDAG stage of the last build */
  double reduce_ms;    /* wall time of the SSVDAG / CSVDAG stage */
  uint64_t gpu_launches;
  uint64_t table_retries; /* heights redone with a full-size hash table after the
                             estimated one proved too small (all builds) */
} svdag_batch_stats;
int svdag_batch_create(svdag_batch** out, int device, void* stream);
int svdag_batch_destroy(svdag_batch* batch);
const char* svdag_batch_last_error(const svdag_batch* batch);
int svdag_batch_clear(svdag_batch* batch);
int svdag_batch_add_chunk(svdag_batch* batch, uint32_t depth, const uint8_t* device_bricks);
int svdag_batch_chunk_count(const svdag_batch* batch, uint32_t* n);
/* flags: SVDAG_BATCH_SDAG and / or SVDAG_BATCH_CSVDAG (the DAG is always built) */
int svdag_batch_build(svdag_batch* batch, uint32_t flags);
int svdag_batch_result(svdag_batch* batch, uint32_t chunk, uint32_t kind, svdag_ctx** view);
int svdag_batch_set_tuning(svdag_batch* batch, const svdag_batch_tuning* tuning);
int svdag_batch_get_tuning(const svdag_batch* batch, svdag_batch_tuning* tuning);
/* Times full builds of the current chunks under candidate settings
 * (coordinate search, at most max_trials builds), keeps the fastest setting
 * and leaves its results in place. */
int svdag_batch_autotune(svdag_batch* batch, uint32_t flags, uint32_t max_trials);
int svdag_batch_get_stats(const svdag_batch* batch, svdag_batch_stats* out);

/* ---- Lossy LSVDAG (project-defined; the reference's toLossyDag,
 * src/symvox/geom_octree_extension.cpp:797-1179, clusters with the external
 * MCL binary, which is not available, and its candidate order depends on
 * OpenMP scheduling).  On a DAG: candidates are the referenced nodes of
 * levels L-1-levels_above_max .. L-1-levels_above_min (top-down) outside
 * subtrees already kept as merge targets; a merge i -> j is allowed when the
 * exact voxel Hamming distance of the two subtrees is at most
 * floor(max_error * 8^(L-level)), the voxels of the subtree's cube; each candidate joins the
 * lowest-index leader among its allowed partners below it, else leads;
 * unreachable nodes are then dropped and toDAG merges new duplicates.  The
 * proposer picks which pairs get the exact check: all pairs whose voxel
 * counts permit the bound (SVDAG_LOSSY_EXACT), the top_k partners by the
 * distance of embeddings from an MLP trained on the GPU on train_pairs exact
 * distances of the scene (SVDAG_LOSSY_LEARNED), or the same network left
 * untrained (SVDAG_LOSSY_UNTRAINED, for comparison).  Every accepted merge
 * is checked exactly, whatever the proposer. */
enum { SVDAG_LOSSY_EXACT = 0, SVDAG_LOSSY_LEARNED = 1, SVDAG_LOSSY_UNTRAINED = 2 };
typedef struct svdag_lossy_params {
  uint32_t levels_above_min; /* 3 */
  uint32_t levels_above_max; /* 5 */
  double max_error;          /* 0.01 */
  uint32_t proposer;
  uint32_t top_k;            /* learned: proposals per candidate, at most 512 (0 = 384) */
  uint64_t train_pairs;      /* learned: training pairs (0 = 2,000,000) */
  uint32_t train_epochs;     /* learned: passes over them (0 = 1) */
  uint64_t seed;
  uint32_t train_batch;      /* learned: pairs per training step, a multiple of 64 in [256, 65536] (0 = 8192) */
  float train_lr;            /* learned: Adam learning rate (0 = 2e-3) */
} svdag_lossy_params;
typedef struct svdag_lossy_stats {
  uint64_t nodes_before, nodes_after, candidates, pairs_evaluated, edges, merged;
  double ms, propose_ms, train_ms;
  float final_loss;
} svdag_lossy_stats;
int svdag_lossy_dag(svdag_ctx* ctx, const svdag_lossy_params* params, svdag_lossy_stats* out);

/* The proposer's network on host buffers (512 -> 256 -> 256 -> 64, ReLU;
 * parameters W1[512x256], b1, W2[256x256], b2, W3[256x64], b3 row-major,
 * concatenated).  loss_grad: siamese loss mean(|f(a) - f(b)|^2 - t)^2 over n
 * pairs and the gradient of every parameter. */
typedef struct svdag_mlp svdag_mlp;
int svdag_mlp_create(svdag_mlp** out, int device, uint64_t seed);
int svdag_mlp_destroy(svdag_mlp* mlp);
uint64_t svdag_mlp_param_count(void);
int svdag_mlp_get_params(svdag_mlp* mlp, float* host_params);
int svdag_mlp_set_params(svdag_mlp* mlp, const float* host_params);
int svdag_mlp_loss_grad(svdag_mlp* mlp, const float* x_a, const float* x_b, const float* t, uint32_t n, float* loss,
                        float* grads);
int svdag_mlp_embed(svdag_mlp* mlp, const float* x, uint32_t n, float* out);

/* toDAG without allocating (no counterpart in the reference, whose toDAG,
 * src/symvox/geom_octree.cpp:462-548, works in host containers).
 *
 * Same result as svdag_reduce_dag, but every temporary (hash table, scan
 * sums, compacted level) lives in one file-scope __device__ array of
 * SVDAG_NOALLOC_SCRATCH_BYTES per device, and each reduced level is copied
 * back into the front of the buffers it already has.  No cudaMalloc,
 * cudaMallocAsync, cudaFree or allocating library call is made.  For callers
 * that must not allocate device memory in the middle of their work: a
 * renderer or streaming system that has already committed the GPU's memory
 * to its own pools (an allocation there fails with out-of-memory, or grows
 * a pool the caller accounts for), or a caller whose memory budget is
 * enforced outside the CUDA allocator.
 *
 * Limit: every inner level (not the root, not the leaves) must fit the
 * scratch.  Levels of up to SVDAG_NOALLOC_MAX_LEVEL_NODES nodes always fit;
 * somewhat larger ones may.  A tree that does not fit is rejected with
 * SVDAG_ERR_OVERFLOW before any work is queued, the octree unchanged and
 * svdag_last_error() naming the level; svdag_reduce_dag has no such limit.
 *
 * The array is shared by every context on a device: calls whose work
 * overlaps in time (two threads, or two streams in flight at once) race on
 * it and corrupt each other; serialise them.  Its contents need not be zero:
 * each call clears what it reads first.  The first call on a device looks
 * the array up (cudaGetSymbolAddress, which can load the module and commit
 * its 64 MiB); make that first call before any stream capture begins, and
 * before the caller commits the GPU's memory to its own pools -- if the
 * array cannot be committed then, the call returns SVDAG_ERR_OOM.  The
 * device address is kept for the life of the process; after a
 * cudaDeviceReset it is stale, so do not call this entry point again in that
 * process.  Like svdag_reduce_dag, the call synchronises its stream once per
 * level and on return.  Per-kernel profiling (svdag_profile_enable) does not
 * cover it.
 *
 * On success the octree is left as svdag_reduce_dag leaves it, except that
 * the SVO's outside masks (svdag_flood_fill), which no longer apply, are
 * released by the next other call on the context or by svdag_destroy
 * instead of at once.  If the hash table's probe limit is hit (only a
 * pathological key set can do it) the levels have already been rewritten
 * when the error is read: the call returns SVDAG_ERR_OVERFLOW with the
 * octree in state SVDAG_S_EMPTY, to be rebuilt. */
#define SVDAG_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define SVDAG_NOALLOC_MAX_LEVEL_NODES 1048576ull
int svdag_reduce_dag_noalloc(svdag_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* SVDAG_GPU_H */
