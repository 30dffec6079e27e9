// GeomOctree facade over the GPU C ABI (see octree_host.hpp).
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "octree_host.hpp"
#include "scene.hpp"

namespace svdag {

void GeomOctree::check(int status) const {
  if (status == SVDAG_OK) return;
  throw std::runtime_error(std::string("svdag: ") + svdag_status_string(status) + ": " +
                           (ctx_ ? svdag_last_error(ctx_) : ""));
}

GeomOctree::GeomOctree(Scene* scene, int device) : scene_(scene) { check(svdag_create(&ctx_, device, nullptr)); }

GeomOctree::GeomOctree(const GeomOctree& o) : scene_(o.scene_), rootSide_(o.rootSide_) {
  std::memcpy(bbox_, o.bbox_, sizeof(bbox_));
  check(svdag_clone(o.ctx_, &ctx_));
}

GeomOctree::~GeomOctree() {
  if (ctx_) svdag_destroy(ctx_);
}

void GeomOctree::buildSVO(unsigned levels, const double bb[6], bool /*internalCall*/,
                          std::vector<std::array<double, 3>>* leavesCenters) {
  if (!scene_) throw std::runtime_error("GeomOctree::buildSVO: no scene");
  check(svdag_upload_triangles(ctx_, scene_->triangles().data(), scene_->nTriangles()));
  check(svdag_voxelize_ex(ctx_, levels, bb, leavesCenters ? SVDAG_VOXELIZE_LEAF_CENTERS : 0));
  if (leavesCenters) {
    uint64_t n = 0;
    check(svdag_download_leaf_centers(ctx_, nullptr, 0, &n));
    leavesCenters->resize(n);
    if (n) check(svdag_download_leaf_centers(ctx_, leavesCenters->front().data(), n, &n));
  }
  // Octree bbox and root side as resizeSceneBbox (octree.hpp:101-105)
  float b[6];
  for (int k = 0; k < 6; ++k) b[k] = float(bb[k]);
  resizeSceneBbox(b);
  invalidate();
}

void GeomOctree::buildDAG(unsigned levels, unsigned stepLevel, const double bb[6]) {
  if (!scene_) throw std::runtime_error("GeomOctree::buildDAG: no scene");
  check(svdag_upload_triangles(ctx_, scene_->triangles().data(), scene_->nTriangles()));
  check(svdag_build_dag(ctx_, levels, stepLevel, bb));
  float b[6];
  for (int k = 0; k < 6; ++k) b[k] = float(bb[k]);
  resizeSceneBbox(b);
  invalidate();
}

void GeomOctree::toDAG() {
  check(svdag_reduce_dag(ctx_));
  invalidate();
}

void GeomOctree::toSDAG(bool /*internalCall*/, bool skipSymmetry) {
  check(svdag_reduce_sdag_ex(ctx_, skipSymmetry ? SVDAG_SDAG_SKIP_SYMMETRY : 0));
  invalidate();
}

unsigned GeomOctree::mergeAcrossAllLevels() {
  check(svdag_cross_level_merge(ctx_));
  invalidate();
  return unsigned(getStats().nCrossLevelMerged);
}

uint64_t GeomOctree::toLossyDag(float, float, int) {
  svdag_lossy_params p{};
  p.levels_above_min = 3;
  p.levels_above_max = 5;
  p.max_error = 0.01;
  p.proposer = SVDAG_LOSSY_EXACT;
  p.seed = 1;
  svdag_lossy_stats st{};
  check(svdag_lossy_dag(ctx_, &p, &st));
  invalidate();
  return st.merged;
}

uint64_t GeomOctree::hiddenGeometryFloodfill() {
  uint64_t empty = 0, surface = 0;
  check(svdag_flood_fill(ctx_, &empty, &surface));
  invalidate();
  outside_ = true;
  return empty ? empty - 1 : 0;
}

void GeomOctree::initChildLevels() {
  check(svdag_init_child_levels(ctx_));
  invalidate();
}

void GeomOctree::importDAG(const NodeData& d, const float bbox[6], double rootSide, uint64_t nVoxels) {
  check(svdag_import_begin(ctx_, unsigned(d.size()), bbox, rootSide, nVoxels));
  for (size_t l = 0; l < d.size(); ++l) {
    std::vector<uint32_t> hdr(d[l].size()), ch(8 * d[l].size());
    for (size_t i = 0; i < d[l].size(); ++i) {
      const Node& n = d[l][i];
      hdr[i] = uint32_t(n.childrenBitmask) | uint32_t(n.childrenMirroredBitmask[0]) << 8 |
               uint32_t(n.childrenMirroredBitmask[1]) << 16 | uint32_t(n.childrenMirroredBitmask[2]) << 24;
      std::memcpy(&ch[8 * i], n.children, 32);
    }
    check(svdag_import_level(ctx_, unsigned(l), d[l].size(), hdr.data(), ch.data()));
  }
  std::memcpy(bbox_, bbox, sizeof(bbox_));
  rootSide_ = rootSide;
  invalidate();
}

void GeomOctree::resizeSceneBbox(const float b[6]) {
  std::memcpy(bbox_, b, sizeof(bbox_));
  float s[3];
  for (int k = 0; k < 3; ++k) s[k] = ((b[3 + k] - b[k]) * 0.5f) * 2.0f;
  float r = s[0] > s[1] ? s[0] : s[1];
  rootSide_ = double(r > s[2] ? r : s[2]);
}

const NodeData& GeomOctree::getNodeData() const {
  if (cached_) return data_;
  const unsigned L = getLevels();
  data_.assign(L, std::vector<Node>());
  for (unsigned l = 0; l < L; ++l) {
    uint64_t n = 0;
    check(svdag_level_count(ctx_, l, &n));
    std::vector<uint32_t> hdr(n), ch(8 * n);
    std::vector<uint8_t> cl(8 * n), inv(n);
    if (n) check(svdag_download_level(ctx_, l, hdr.data(), ch.data(), cl.data(), inv.data()));
    std::vector<Node>& out = data_[l];
    out.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
      Node& d = out[i];
      d.childrenBitmask = uint8_t(hdr[i]);
      d.childrenMirroredBitmask[0] = uint8_t(hdr[i] >> 8);
      d.childrenMirroredBitmask[1] = uint8_t(hdr[i] >> 16);
      d.childrenMirroredBitmask[2] = uint8_t(hdr[i] >> 24);
      std::memcpy(d.children, &ch[8 * i], 32);
      for (int c = 0; c < 8; ++c) d.childLevels[c] = (cl[8 * i + c] == 0xFF) ? 0xFFFFFFFFu : cl[8 * i + c];
      d.invariantBitmask = inv[i];
    }
    if (outside_ && n) {
      std::vector<uint8_t> om(n);
      check(svdag_download_outside_masks(ctx_, l, om.data()));
      for (uint64_t i = 0; i < n; ++i) out[i].outsideMask = om[i];
    }
  }
  cached_ = true;
  return data_;
}

Stats GeomOctree::getStats() const {
  svdag_stats s;
  check(svdag_get_stats(ctx_, &s));
  Stats r;
  r.nTotalVoxels = s.n_total_voxels;
  r.nNodesSVO = s.n_nodes_svo;
  r.nNodesLastLevSVO = s.n_nodes_last_lev_svo;
  r.nNodesDAG = s.n_nodes_dag;
  r.nNodesSDAG = s.n_nodes_sdag;
  r.simulatedEncodedSVOSize = (s.n_nodes_svo - s.n_nodes_last_lev_svo) * 4;
  r.nCrossLevelMerged = s.n_cross_level_merged;
  r.nMissingCorrespondences = s.n_missing_correspondences;
  r.buildSVOTime = s.svo_ms;
  r.toDAGTime = s.dag_ms;
  r.toSDAGTime = s.sdag_ms;
  r.crossMergeTime = s.csv_ms;
  return r;
}

State GeomOctree::getState() const {
  svdag_stats s;
  check(svdag_get_stats(ctx_, &s));
  return State(s.state);
}

unsigned GeomOctree::getLevels() const {
  svdag_stats s;
  check(svdag_get_stats(ctx_, &s));
  return s.levels;
}

uint64_t GeomOctree::getNVoxels() const { return getStats().nTotalVoxels; }

uint64_t GeomOctree::getNNodes() const {
  svdag_stats s;
  check(svdag_get_stats(ctx_, &s));
  return s.n_nodes;
}

}  // namespace svdag
