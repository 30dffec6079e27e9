// CPU oracle for the SVDAG construction path: a restatement of the
// reference's GeomOctree algorithms (voxelization, SVO->DAG, DAG->SDAG,
// cross-level merge, chunked build).  TEST INFRASTRUCTURE ONLY: the tests,
// the smoke check and the CPU-baseline leg of the benchmark call it as the
// checker; the product path never links or calls it.
//
// Node records are exchanged in the same 48-byte layout the reference dump
// harness writes (ref_dump.cpp):
//   u32 hdr = mask | mirX<<8 | mirY<<16 | mirZ<<24, u32 children[8],
//   u8 childLevels[8], u8 invariant, u8 pad[3]
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_octree ora_octree;

typedef struct ora_stats {
  uint64_t n_total_voxels;
  uint64_t n_nodes_svo, n_nodes_last_lev_svo;
  uint64_t n_nodes_dag, n_nodes_sdag;
  uint64_t n_nodes;           /* current node count (reference _nNodes) */
  uint64_t n_cross_level_merged;
  uint64_t n_missing_correspondences;
  uint32_t levels;
  uint32_t state;             /* 0 empty, 1 SVO, 2 DAG, 3 SDAG (geom_octree.hpp:36-41) */
} ora_stats;

ora_octree* ora_create(void);
void ora_destroy(ora_octree* o);
ora_octree* ora_clone(const ora_octree* o);

/* GeomOctree::buildSVO (geom_octree.cpp:171-280). bbox = {minx,miny,minz,maxx,maxy,maxz}. */
int ora_build_svo(ora_octree* o, const float* tris, uint64_t n_tris, const double bbox[6], uint32_t levels);
/* GeomOctree::buildDAG (geom_octree.cpp:289-435), OpenMP over chunks; n_threads<=0 = all. */
int ora_build_dag_chunked(ora_octree* o, const float* tris, uint64_t n_tris, const double bbox[6],
                          uint32_t levels, uint32_t step_level, int n_threads);
/* voxel bricks (8^(depth-1) masks, Morton order) -> node pools in the DAG
 * state, the GeomOctree(NodeData, ...) route (geom_octree.cpp:49-60) */
int ora_build_from_bricks(ora_octree* o, uint32_t depth, const uint8_t* bricks);
/* lossy LSVDAG, exact-proposer form (project-defined; see the .cpp) */
int ora_lossy_exact(ora_octree* o, uint32_t min_above, uint32_t max_above, double max_err, uint64_t* merged);
/* the per-level node order of EncodedSSVDAG::encode (encoded_ssvdag.cpp:259-276):
 * std::sort of (index, count) pairs by count, descending */
int ora_refcount_order(const uint32_t* counts, uint64_t n, uint32_t* order);
/* EncodedSSVDAG::traverse (encoded_ssvdag.cpp:527-574): depth reached per point */
int ora_ssvdag_traverse(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                        const uint32_t* level_off, uint32_t n_level_off, uint32_t levels, const float bbox[6],
                        float root_side, const float* pts, uint64_t n, int32_t* out);
/* the viewer's SSVDAG ray traversal (shaders/octree_dda.frag.glsl:539-581),
 * one 32-byte hit record per pixel (ssvdag_raycast.cpp) */
int ora_ssvdag_raycast(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                       const uint32_t* level_off, uint32_t n_level_off, uint32_t levels, const float bbox[6],
                       float root_side, const float view_inv[16], const float proj_inv[16], uint32_t width,
                       uint32_t height, uint32_t max_iters, uint32_t draw_level, float projection_factor,
                       float t_min, float t_max, void* hits);
/* GeomOctree::hiddenGeometryFloodfill (geom_octree_extension.cpp:1651-1891)
 * on an SVO: outside masks per node; -3 when the start corner cell is set */
int ora_flood_fill(ora_octree* o, uint64_t* n_empty, uint64_t* n_surface);
int ora_get_outside(const ora_octree* o, uint32_t level, uint8_t* out);
int ora_to_dag(ora_octree* o);                 /* geom_octree.cpp:462-548 */
int ora_to_sdag(ora_octree* o);                /* geom_octree.cpp:551-697 (greedy, symmetry on) */
int ora_to_sdag_ex(ora_octree* o, int skip_symmetry); /* the same, skipSymmetry (:596-601) when non-zero */
int ora_init_child_levels(ora_octree* o);      /* geom_octree_extension.cpp:21-30 */
int ora_merge_across_levels(ora_octree* o);    /* geom_octree_extension.cpp:1192-1544 */

uint64_t ora_level_count(const ora_octree* o, uint32_t level);
int ora_get_level(const ora_octree* o, uint32_t level, uint8_t* rec48);
int ora_get_stats(const ora_octree* o, ora_stats* s);

/* Single fp64 SAT test (test_triangle_box.cpp:105-184), exposed for unit tests. */
int ora_tri_box(const double center[3], double half_side, const float tri[9]);

#ifdef __cplusplus
}
#endif
