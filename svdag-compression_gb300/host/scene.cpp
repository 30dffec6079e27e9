// OBJ scene loading with the reference's rules (src/symvox/scene.cpp).
#include "scene.hpp"

#include <cfloat>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace svdag {

namespace {

// Scene::BinObjHeader and record layouts of the .bincache file
// (src/symvox/scene.hpp:107-116, scene.cpp:324-374) on LP64 hosts.
struct BinHeader {
  uint64_t nVertices, nNormals, nMaterials, nIndexedTris;
  float bboxMin[3], bboxMax[3];
};
struct BinMaterial {  // Scene::TMaterial: name[256], 3 colours, 2 floats
  char name[256];
  float diffuse[3], spec[3], ambient[3];
  float specCoef, transparency;
};
struct BinTri {  // Scene::TIndexedTri: size_t verticesIdx[3], normalsIdx[3], material
  uint64_t v[3], n[3], material;
};
static_assert(sizeof(BinHeader) == 56, "bincache header layout");
static_assert(sizeof(BinMaterial) == 300, "bincache material layout");
static_assert(sizeof(BinTri) == 56, "bincache triangle layout");

}  // namespace

Scene::Scene() {
  bbox_[0] = bbox_[1] = bbox_[2] = FLT_MAX;
  bbox_[3] = bbox_[4] = bbox_[5] = -FLT_MAX;
}

void Scene::setBBox(const float b[6]) { std::memcpy(bbox_, b, sizeof(bbox_)); }

void Scene::setTriangles(const float* t, uint64_t n) { tris_.assign(t, t + 9 * n); }

bool Scene::loadObj(const std::string& path, bool tryLoadBinCache, bool writeBinCache) {
  const std::string cache = path + ".bincache";
  if (tryLoadBinCache) {
    std::ifstream probe(cache);
    if (probe.good()) {
      probe.close();
      if (!loadBinCache(cache)) return false;
      buildTriVector();
      return true;
    }
  }
  FILE* fp = std::fopen(path.c_str(), "r");
  if (!fp) return false;
  verts_.clear();
  tri_idx_.clear();
  tri_nidx_.clear();
  bbox_[0] = bbox_[1] = bbox_[2] = FLT_MAX;
  bbox_[3] = bbox_[4] = bbox_[5] = -FLT_MAX;
  static char line[10000];
  while (std::fgets(line, sizeof(line), fp)) {
    if (line[0] == 'v') {
      if (line[1] == 'n' || line[1] == 't') continue;  // normals / texture coordinates are not used
      float p[3];
      if (std::sscanf(line + 1, "%f %f %f", &p[0], &p[1], &p[2]) != 3) continue;
      for (int k = 0; k < 3; ++k) {
        if (p[k] < bbox_[k]) bbox_[k] = p[k];
        if (p[k] > bbox_[3 + k]) bbox_[3 + k] = p[k];
      }
      verts_.insert(verts_.end(), p, p + 3);
    } else if (line[0] == 'f') {
      // tokens split on ' '; the last token loses its final character (the
      // newline), as the reference does
      std::vector<std::string> tok;
      char* save = nullptr;
      for (char* t = strtok_r(line + 1, " ", &save); t; t = strtok_r(nullptr, " ", &save)) tok.emplace_back(t);
      if (tok.empty()) continue;
      tok.back().resize(tok.back().size() - 1);
      if (tok.size() < 3) continue;
      auto parse = [&](const std::string& s, uint64_t& vi) {
        int iv = 0, in = 0;
        const int n = std::sscanf(s.c_str(), "%d//%d", &iv, &in);
        if (iv < 0) iv = int(verts_.size() / 3) + iv + 1;
        if (n >= 1) vi = uint64_t(int64_t(iv) - 1);
      };
      uint64_t v[3] = {~0ull, ~0ull, ~0ull};
      for (int i = 0; i < 3; ++i) parse(tok[i], v[i]);
      tri_idx_.insert(tri_idx_.end(), v, v + 3);
      if (tok.size() > 4) {  // the reference reads a second triangle only when more than 4 tokens remain
        uint64_t w[3] = {v[0], v[1], v[2]};
        for (int i = 0; i < 3; ++i) parse(tok[(i + 2) % 4], w[i]);
        tri_idx_.insert(tri_idx_.end(), w, w + 3);
      }
    }
  }
  std::fclose(fp);
  tri_nidx_.assign(tri_idx_.size(), 0);
  if (writeBinCache) saveBinCache(cache);
  buildTriVector();
  return true;
}

void Scene::buildTriVector() {
  tris_.clear();
  const uint64_t nv = verts_.size() / 3;
  for (size_t t = 0; t + 2 < tri_idx_.size(); t += 3) {
    if (tri_idx_[t] < nv && tri_idx_[t + 1] < nv && tri_idx_[t + 2] < nv)
      for (int k = 0; k < 3; ++k) tris_.insert(tris_.end(), &verts_[3 * tri_idx_[t + k]], &verts_[3 * tri_idx_[t + k]] + 3);
  }
}

bool Scene::saveBinCache(const std::string& path) const {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  BinHeader h{};
  h.nVertices = verts_.size() / 3;
  h.nNormals = 0;
  h.nMaterials = 1;
  h.nIndexedTris = tri_idx_.size() / 3;
  std::memcpy(h.bboxMin, bbox_, 12);
  std::memcpy(h.bboxMax, bbox_ + 3, 12);
  f.write(reinterpret_cast<const char*>(&h), sizeof(h));
  f.write(reinterpret_cast<const char*>(verts_.data()), std::streamsize(verts_.size() * 4));
  BinMaterial m{};
  std::snprintf(m.name, sizeof(m.name), "Voxelator Default Mat");
  for (int k = 0; k < 3; ++k) { m.ambient[k] = 0.1f; m.diffuse[k] = 0.9f; m.spec[k] = 0.2f; }
  f.write(reinterpret_cast<const char*>(&m), sizeof(m));
  for (size_t t = 0; t + 2 < tri_idx_.size(); t += 3) {
    BinTri bt{};
    for (int k = 0; k < 3; ++k) { bt.v[k] = tri_idx_[t + k]; bt.n[k] = tri_nidx_[t + k]; }
    f.write(reinterpret_cast<const char*>(&bt), sizeof(bt));
  }
  return bool(f);
}

bool Scene::loadBinCache(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  BinHeader h;
  if (!f.read(reinterpret_cast<char*>(&h), sizeof(h))) return false;
  std::memcpy(bbox_, h.bboxMin, 12);
  std::memcpy(bbox_ + 3, h.bboxMax, 12);
  verts_.resize(3 * h.nVertices);
  f.read(reinterpret_cast<char*>(verts_.data()), std::streamsize(verts_.size() * 4));
  f.seekg(std::streamoff(h.nNormals * 12 + h.nMaterials * sizeof(BinMaterial)), std::ios::cur);
  tri_idx_.resize(3 * h.nIndexedTris);
  tri_nidx_.resize(3 * h.nIndexedTris);
  for (uint64_t t = 0; t < h.nIndexedTris; ++t) {
    BinTri bt;
    if (!f.read(reinterpret_cast<char*>(&bt), sizeof(bt))) return false;
    for (int k = 0; k < 3; ++k) { tri_idx_[3 * t + k] = bt.v[k]; tri_nidx_[3 * t + k] = bt.n[k]; }
  }
  return true;
}

}  // namespace svdag
