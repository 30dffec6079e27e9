// Host-side mirror of SymVox's GeomOctree build surface over the GPU C ABI
// (include/svdag_gpu.h), plus the reference's node record and the encoders
// of its output files.
//
// GeomOctree keeps the reference's method names and meaning
// (src/symvox/geom_octree.hpp:106-157); geometry arguments are plain arrays
// instead of SpaceLand types.  The node pool lives on the GPU and is copied
// into the reference's NodeData form on the first getNodeData() after a build
// step, so encoders and other consumers read it exactly as in the reference.
#pragma once

#include <stdint.h>

#include <array>
#include <string>
#include <vector>

#include "svdag_gpu.h"

namespace svdag {

constexpr uint32_t kNullNode = 0xFFFFFFFEu;  // Octree::nullNode (src/symvox/octree.cpp:22)

// Octree::Node + GeomOctree::Node fields (src/symvox/octree.hpp:57-85,
// src/symvox/geom_octree.hpp:59-96).
struct Node {
  uint32_t children[8];
  uint8_t childrenBitmask = 0;
  uint32_t childLevels[8];
  uint8_t childrenMirroredBitmask[3] = {0, 0, 0};
  uint8_t invariantBitmask = 0;
  uint8_t outsideMask = 0;
  Node() {
    for (int c = 0; c < 8; ++c) { children[c] = kNullNode; childLevels[c] = 0xFFFFFFFFu; }
  }
  bool existsChild(int c) const { return (childrenBitmask >> c) & 1u; }
  bool existsChildPointer(int c) const { return children[c] != kNullNode; }
  bool getChildMirrorBit(int axis, int c) const { return (childrenMirroredBitmask[axis] >> c) & 1u; }
  unsigned getNChildren() const { return unsigned(__builtin_popcount(childrenBitmask)); }
};

typedef std::vector<std::vector<Node>> NodeData;

enum State { S_EMPTY = 0, S_SVO = 1, S_DAG = 2, S_SDAG = 3 };

struct Stats {
  uint64_t nTotalVoxels = 0, nNodesSVO = 0, nNodesDAG = 0, nNodesSDAG = 0;
  uint64_t nNodesLastLevSVO = 0, nNodesLastLevDAG = 0, nNodesLastLevSDAG = 0;
  uint64_t simulatedEncodedSVOSize = 0, nCrossLevelMerged = 0, nMissingCorrespondences = 0;
  double buildSVOTime = 0, toDAGTime = 0, toSDAGTime = 0, crossMergeTime = 0;  // milliseconds
};

class Scene;

class GeomOctree {
 public:
  explicit GeomOctree(Scene* scene = nullptr, int device = 0);
  GeomOctree(const GeomOctree& other);  // device-side deep copy
  GeomOctree& operator=(const GeomOctree&) = delete;
  ~GeomOctree();

  void setScene(Scene* s) { scene_ = s; }
  // buildSVO(levels, bbox) (geom_octree.cpp:171-280); bbox = {min xyz, max xyz}
  // With leavesCenters, also the reference's list of leaf-node centres
  // (geom_octree.cpp:245-246), in node order; internalCall only silences the
  // reference's log.  putMaterialIdInLeaves is not supported.
  void buildSVO(unsigned levels, const double bbox[6], bool internalCall = false,
                std::vector<std::array<double, 3>>* leavesCenters = nullptr);
  // buildDAG(levels, stepLevel, bbox) (geom_octree.cpp:289-435): chunked
  // build, same node order as the reference.
  void buildDAG(unsigned levels, unsigned stepLevel, const double bbox[6]);
  void toDAG();
  // toSDAG(internalCall, skipSymmetry) (geom_octree.cpp:551-697); internalCall
  // only silences the reference's log
  void toSDAG(bool internalCall = false, bool skipSymmetry = false);
  unsigned mergeAcrossAllLevels();
  // toLossyDag(lossyInflation, allowedLossyDiffFactor, includedNodeRefCount)
  // (geom_octree_extension.cpp:797-1179).  The reference clusters its
  // candidate edges with the external MCL program, which this build does not
  // have; here the DAG goes through the project's lossy LSVDAG on the GPU
  // (svdag_lossy_dag: exact proposals for the nodes 3-5 levels above the
  // leaves, a merge accepted within 1 % of the subtree cube's voxels).  The
  // reference's three parameters are parsed for the output names only.
  // Returns the number of merged nodes.
  uint64_t toLossyDag(float lossyInflation, float allowedLossyDiffFactor, int includedNodeRefCount);
  void initChildLevels();
  // hiddenGeometryFloodfill (geom_octree_extension.cpp:1651-1891) on the SVO:
  // fills each node's outsideMask (read through getNodeData until the next
  // build step); returns the reference's count of empty leaves reached
  // besides the start cell.  Throws when the start corner cell is set.
  uint64_t hiddenGeometryFloodfill();
  // GeomOctree(NodeData, bbox, rootSide, levels, stats) (geom_octree.cpp:49-60)
  void importDAG(const NodeData& data, const float bbox[6], double rootSide, uint64_t nVoxels);

  const NodeData& getNodeData() const;
  Stats getStats() const;
  State getState() const;
  unsigned getLevels() const;
  uint64_t getNVoxels() const;
  uint64_t getNNodes() const;
  const float* getSceneBBox() const { return bbox_; }
  float getRootSide() const { return float(rootSide_); }
  double getRootSideD() const { return rootSide_; }
  // resizeSceneBbox (octree.hpp:101-105)
  void resizeSceneBbox(const float bbox[6]);
  svdag_ctx* handle() const { return ctx_; }

 private:
  void check(int status) const;
  void invalidate() {
    cached_ = false;
    outside_ = false;
  }
  bool outside_ = false;  // outside masks of the current SVO are on the device
  Scene* scene_ = nullptr;
  svdag_ctx* ctx_ = nullptr;
  float bbox_[6] = {0, 0, 0, 0, 0, 0};
  double rootSide_ = 0;
  mutable NodeData data_;
  mutable bool cached_ = false;
};

// ---------------------------------------------------------------------------
// Output files, byte-compatible with the reference's savers.

// EncodedSVDAG (src/symvox/encoded_svdag.cpp:76-199): absolute u32 pointers,
// child levels honoured (CSVDAG).
struct EncodedSVDAG {
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  float rootSide = 0;
  uint32_t levels = 0;
  uint64_t nNodes = 0;
  uint32_t firstLeafPtr = 0;
  std::vector<uint32_t> data;
  bool encode(const NodeData& d, const float bbox[6], float rootSide, uint64_t nNodes, State st);
  // the same stream built on the GPU from the octree's device pools (svdag_encode)
  bool encode(const GeomOctree& o);
  bool save(const std::string& path) const;
  size_t getDataSize() const { return data.size() * 4; }
  // EncodedSVDAG::load / decode (encoded_svdag.cpp:44-74, 217-281): the
  // stream back into per-level nodes (same-level pointers only, as the
  // reference's decoder).
  bool load(const std::string& path);
  NodeData decode() const;
};

// EncodedUSSVDAG (src/symvox/encoded_ussvdag.cpp:60-170): SVDAG layout with the
// three mirror masks packed into the node header word.
struct EncodedUSSVDAG {
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  float rootSide = 0;
  uint32_t levels = 0;
  uint64_t nNodes = 0;
  uint32_t firstLeafPtr = 0;
  std::vector<uint32_t> data;
  bool encode(const NodeData& d, const float bbox[6], float rootSide, uint64_t nNodes, State st);
  // the same stream built on the GPU (svdag_encode)
  bool encode(const GeomOctree& o);
  bool save(const std::string& path) const;
  size_t getDataSize() const { return data.size() * 4; }
};

// EncodedSSVDAG (src/symvox/encoded_ssvdag.cpp:84-466): levels reordered by
// reference count, 4^3 leaf bricks, 16/32-bit pointers with mirror bits.
struct EncodedSSVDAG {
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  float rootSide = 0;
  uint32_t levels = 0;
  uint64_t nNodes = 0;
  std::vector<uint16_t> inner;
  std::vector<uint8_t> leaves;
  std::vector<uint32_t> levelOffsets;
  bool encode(const NodeData& d, const float bbox[6], float rootSide, uint64_t nNodes, State st);
  // the same arrays built on the GPU (svdag_encode_ssvdag; the ref-count
  // order is the same std::sort on the host)
  bool encode(const GeomOctree& o);
  bool save(const std::string& path) const;
  size_t getDataSize() const { return inner.size() * 2 + leaves.size() + levelOffsets.size() * 4; }
};

}  // namespace svdag
