// Triangle-soup scene loaded from ASCII OBJ with the reference's parsing
// rules and its binary cache (src/symvox/scene.cpp:51-416).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace svdag {

class Scene {
 public:
  Scene();
  // Scene::loadObj (scene.cpp:51-250): `v` lines (all of them grow the
  // bounding box, referenced or not), `f` lines as "%d//%d" tokens with
  // negative indices relative to the end; a binary cache "<file>.bincache"
  // is read when present and written after an ASCII parse.  The ASCII parse
  // runs on `threads` host threads (0: all cores): the file is cut at line
  // starts, each piece parsed on its own, and vertex numbering and negative
  // indices resolved from the pieces' vertex counts, so the result is the
  // same for every thread count.
  bool loadObj(const std::string& path, bool tryLoadBinCache = true, bool writeBinCache = true,
               unsigned threads = 0);
  // Triangle soup (Scene::buildTriVector, scene.cpp:394-416): 9 floats per
  // triangle, triangles with an out-of-range vertex index dropped.
  const std::vector<float>& triangles() const { return tris_; }
  uint64_t nTriangles() const { return tris_.size() / 9; }
  // Scene bounding box {min xyz, max xyz} (float, as Scene::getAABB)
  const float* bbox() const { return bbox_; }
  void setBBox(const float b[6]);
  void setTriangles(const float* t, uint64_t n);

 private:
  bool loadBinCache(const std::string& path);
  bool saveBinCache(const std::string& path) const;
  void buildTriVector(unsigned threads);
  std::vector<float> verts_;                 // xyz per vertex
  std::vector<uint64_t> tri_idx_;            // 3 vertex indices per triangle
  std::vector<uint64_t> tri_nidx_;           // 3 normal indices per triangle (cache layout only)
  std::vector<float> tris_;
  float bbox_[6];
};

}  // namespace svdag
