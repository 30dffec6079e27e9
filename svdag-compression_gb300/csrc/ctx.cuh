// Internal state of one SVDAG build context and the phase entry points the
// C ABI (api.cu) dispatches to.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "common.cuh"

namespace svdag {

// One octree level in HBM, structure-of-arrays.
//   hdr[n]      : mask | mirX<<8 | mirY<<16 | mirZ<<24
//   ch[8n]      : child ids (kNull when absent); empty on the leaf level
//   inv[n]      : invariant mask (SDAG only; empty otherwise)
//   clev[8n]    : child levels (CSVDAG only; empty otherwise)
//   ctr[3n]     : fp64 node centre (SVO build only)
//   nbox[8n]    : fp32 child-box centres of the node (SVO build only)
//   outm[n]     : outside mask of the hidden-geometry flood fill (SVO only)
struct Level {
  uint64_t n = 0;
  DBuf<uint32_t> hdr;
  DBuf<uint32_t> ch;
  DBuf<uint8_t> inv;
  DBuf<uint8_t> clev;
  DBuf<double> ctr;
  DBuf<float> nbox;
  DBuf<uint8_t> outm;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Exec ex;
  uint64_t launches = 0;

  const float* tris = nullptr;
  uint64_t n_tris = 0;
  DBuf<float> owned_tris;

  uint32_t levels = 0;
  int state = SVDAG_S_EMPTY;
  bool child_levels_init = false;  // initChildLevels called (clev = lev+1 implicitly)
  std::vector<Level> lev;
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  double root_side = 0.0;

  svdag_stats st{};
  std::string last_error;

  // buildSVO's leavesCenters (geom_octree.cpp:245-246): the fp64 centre of
  // every leaf-level node, in node order, kept by svdag_voxelize_ex on request
  bool keep_leaf_centers = false;
  DBuf<double> leaf_ctr;
  uint64_t leaf_ctr_n = 0;

  // Outside masks taken off the levels by svdag_reduce_dag_noalloc, which
  // may not free device memory: released by a later call on the context
  // (every entry point that can allocate) or by svdag_destroy.
  std::vector<DBuf<uint8_t>> retired;

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Profiler prof;

  // the last SSVDAG encoding (svdag_encode_ssvdag), read by
  // svdag_download_ssvdag: inner words per level, leaf bricks
  std::vector<DBuf<uint16_t>> ss_inner;
  std::vector<uint64_t> ss_words;
  DBuf<uint64_t> ss_leaves;
  uint64_t ss_bricks = 0;
};

// Phases (each throws svdag::Error on failure).
// tri_list (optional, device, ascending ids): voxelize only these triangles
void phase_voxelize(Ctx& c, uint32_t levels, const double bbox[6], const uint32_t* tri_list = nullptr,
                    uint64_t n_list = 0);
// GeomOctree::buildDAG: chunked build joined and reduced to a DAG
void phase_build_dag(Ctx& c, uint32_t levels, uint32_t step_level, const double bbox[6]);
void phase_reduce_dag(Ctx& c);
void phase_reduce_sdag(Ctx& c);
// toSDAG with skipSymmetry: pointer compression only (reduce.cu)
void phase_reduce_sdag_skip_symmetry(Ctx& c);
void phase_cross_level_merge(Ctx& c);
// GeomOctree::hiddenGeometryFloodfill: outside masks of an SVO (floodfill.cu).
void phase_flood_fill(Ctx& c, uint64_t* n_empty, uint64_t* n_surface);
// Reference-count order of a level, exactly as the reference's std::sort of
// (index, count) pairs leaves it (refsort.cu): order[k] = k-th node.
void refcount_order(const Exec& ex, const uint32_t* counts, uint64_t n, uint32_t* order);
// testTriBox of the 8 children of n (triangle, node) pairs, host buffers in
// and out (voxelize.cu).
void tri_box_children(Ctx& c, const float* tris, const double* centers, const double* half_sides, uint64_t n,
                      uint8_t* masks, uint64_t* fallbacks);
// The reference's lossy candidate stage (lossy_ref.cu).
void phase_sort_by_effective_refcount(Ctx& c);
void lossy_candidate_edges(Ctx& c, uint32_t level, float diff_factor, int included, const uint8_t* reps_below,
                           std::vector<uint32_t>& src, std::vector<uint32_t>& tgt, std::vector<float>& weight);
// toDAG with every temporary in caller-provided device scratch (no allocation).
void phase_reduce_dag_scratch(Ctx& c, uint8_t* scratch, uint64_t capacity);

// Voxel-brick chunks (batch.cu).
float synth_noise_bricks(cudaStream_t st, uint32_t depth, uint64_t seed, double fill, uint8_t* out);
void phase_import_bricks(Ctx& c, uint32_t depth, const uint8_t* bricks);

}  // namespace svdag

struct svdag_ctx {
  svdag::Ctx c;
};

namespace svdag {

struct BatchChunk {
  uint32_t depth;
  const uint8_t* bricks;  // device, borrowed
};
struct BatchResult {
  std::unique_ptr<svdag_ctx> dag, sdag, csv;
};
struct BatchTuning {
  double table_factor = 2.0;  // hash slots per cell of a height (power of two above)
  unsigned threads = 256;     // block size of the per-height kernels
  int streams = 4;            // concurrent per-chunk reductions
};
struct Batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Exec ex;
  uint64_t launches = 0;
  std::vector<BatchChunk> chunks;
  std::vector<BatchResult> results;
  BatchTuning tuning;
  std::vector<uint64_t> worker_launches;
  std::vector<cudaStream_t> streams;
  std::string last_error;
  double dag_ms = 0, reduce_ms = 0;
  // Largest share of distinct keys among the cells of each height seen by
  // earlier waves and builds (0 = none yet): later tables of that height are
  // sized for twice that share; a table that proves too small is rebuilt at
  // full size (table_retries counts those).
  std::vector<double> distinct_share;
  uint64_t table_retries = 0;
};
void batch_build_dags(Batch& B);
void batch_reduce(Batch& B, bool sdag, bool csv);

}  // namespace svdag

struct svdag_batch {
  svdag::Batch b;
};
