// OBJ scene loading with the reference's rules (src/symvox/scene.cpp).
#include "scene.hpp"
#include "svdag_host.h"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
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

namespace {

constexpr size_t kLineCap = 10000;  // the reference's fgets buffer: records of at most 9999 characters

// One OBJ record (an fgets line) as the reference reads it
// (src/symvox/scene.cpp:98-233): a vertex, or a face giving one or two
// triangles.  Face corners keep the raw "%d//%d" index; a corner whose
// parse gives no index keeps the previous triangle's value (the reference
// reuses its TIndexedTri), which for the first triangle is no vertex.
struct Record {
  int kind = 0;  // 0 ignored, 1 vertex, 2 face
  float p[3];
  int ntri = 0;
  int iv[2][3];
  bool got[2][3];
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// Exact powers of ten in double (10^0 .. 10^22).
const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                           1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// A plain decimal [+-]digits[.digits][(e|E)[+-]digits] converted to the
// nearest float, or false to let the C library decide.  The value is
// m * 10^e with m < 2^53 and |e| <= 22, so one IEEE multiply or divide
// gives the double nearest to it (Clinger's fast path); rounding that
// double to float gives the float nearest to the decimal unless the double
// lies exactly halfway between two floats, which is left to the library
// too.  *end is set past the number.
bool fast_float(const char* p, const char** end, float* out) {
  while (is_space(*p)) ++p;
  bool neg = false;
  if (*p == '+' || *p == '-') neg = *p++ == '-';
  uint64_t m = 0;
  int digits = 0, exp10 = 0;
  bool any = false;
  for (; *p >= '0' && *p <= '9'; ++p) {
    any = true;
    if (m == 0 && *p == '0') continue;
    if (++digits > 18) return false;
    m = m * 10 + uint64_t(*p - '0');
  }
  if (*p == '.') {
    ++p;
    for (; *p >= '0' && *p <= '9'; ++p) {
      any = true;
      if (m == 0 && *p == '0') { --exp10; continue; }
      if (++digits > 18) return false;
      m = m * 10 + uint64_t(*p - '0');
      --exp10;
    }
  }
  if (!any) return false;
  if (*p == 'e' || *p == 'E') {
    const char* q = p + 1;
    bool eneg = false;
    if (*q == '+' || *q == '-') eneg = *q++ == '-';
    if (!(*q >= '0' && *q <= '9')) return false;
    int e = 0;
    for (; *q >= '0' && *q <= '9'; ++q) {
      if (e > 1000) return false;
      e = e * 10 + (*q - '0');
    }
    exp10 += eneg ? -e : e;
    p = q;
  }
  if (*p == 'x' || *p == 'X' || *p == 'p' || *p == 'P' || *p == 'n' || *p == 'N' || *p == 'i' || *p == 'I')
    return false;
  if (m >= (1ull << 53)) return false;
  double d = double(m);
  if (m != 0) {
    if (exp10 < -22 || exp10 > 22) return false;
    d = exp10 < 0 ? d / kPow10[-exp10] : d * kPow10[exp10];
  }
  // a float midpoint has exactly 25 significant bits: the 29 low mantissa
  // bits of the double are then 1 followed by zeros
  uint64_t bits;
  std::memcpy(&bits, &d, 8);
  if ((bits & ((1ull << 29) - 1)) == (1ull << 28)) return false;
  const float f = float(d);
  if (f == 0.f && d != 0.0) return false;  // below the float range: the library's rounding
  if (f - f != 0.f) return false;          // above it
  *out = neg ? -f : f;
  *end = p;
  return true;
}

// sscanf(s, "%f %f %f") == 3, with the common case parsed directly.
bool three_floats(const char* s, float p[3]) {
  const char* q = s;
  for (int k = 0; k < 3; ++k) {
    const char* e;
    if (!fast_float(q, &e, &p[k]) || (k < 2 && !is_space(*e))) {
      return std::sscanf(s, "%f %f %f", &p[0], &p[1], &p[2]) == 3;
    }
    q = e;
  }
  return true;
}

// sscanf(t, "%d//%d", &iv, ...) >= 1, with plain integers parsed directly.
bool face_index(const char* t, int& iv) {
  const char* p = t;
  while (is_space(*p)) ++p;
  bool neg = false;
  if (*p == '+' || *p == '-') neg = *p++ == '-';
  int64_t v = 0;
  int n = 0;
  for (; *p >= '0' && *p <= '9' && n < 10; ++p, ++n) v = v * 10 + (*p - '0');
  if (n == 0 || n >= 10 || (*p >= '0' && *p <= '9')) {
    int in = 0;
    iv = 0;
    return std::sscanf(t, "%d//%d", &iv, &in) >= 1;
  }
  iv = int(neg ? -v : v);
  return true;
}

void parse_record(char* line, Record& r) {
  r.kind = 0;
  if (line[0] == 'v') {
    if (line[1] == 'n' || line[1] == 't') return;  // normals / texture coordinates are not used
    if (!three_floats(line + 1, r.p)) return;
    r.kind = 1;
  } else if (line[0] == 'f') {
    // tokens split on ' '; the last token loses its final character (the
    // newline), as the reference does
    char* tok[5];
    size_t len[5];
    int nt = 0;
    char* save = nullptr;
    for (char* t = strtok_r(line + 1, " ", &save); t; t = strtok_r(nullptr, " ", &save)) {
      if (nt < 5) {
        tok[nt] = t;
        len[nt] = std::strlen(t);
      }
      ++nt;
      if (nt > 5) {
        // only the first four tokens are read; the count only decides
        // whether a second triangle exists, and the last token's trim only
        // matters when it is among the first four
      }
    }
    if (nt == 0) return;
    if (nt <= 5 && nt >= 1) tok[nt - 1][len[nt - 1] - 1] = '\0';
    if (nt < 3) return;
    auto parse = [](const char* t, int& iv) { return face_index(t, iv); };
    r.kind = 2;
    r.ntri = nt > 4 ? 2 : 1;
    for (int i = 0; i < 3; ++i) r.got[0][i] = parse(tok[i], r.iv[0][i]);
    if (r.ntri == 2)
      for (int i = 0; i < 3; ++i) r.got[1][i] = parse(tok[(i + 2) % 4], r.iv[1][i]);
  }
}

// A corner's vertex index given the vertex count at its line: negative
// indices count back from the end ("int(_vertices.size()) + idxV + 1").
struct Corner {
  int64_t v;    // resolved index, relative to the chunk's first vertex when rel
  uint8_t rel;
};

inline Corner corner(int iv, uint64_t nverts_local) {
  if (iv < 0) return {int64_t(nverts_local) + iv, 1};
  return {int64_t(iv) - 1, 0};
}

// Bounding-box update of AABox::merge: strict comparisons, so the first
// occurrence of an extreme value is the one kept.
inline void grow(float b[6], const float p[3]) {
  for (int k = 0; k < 3; ++k) {
    if (p[k] < b[k]) b[k] = p[k];
    if (p[k] > b[3 + k]) b[3 + k] = p[k];
  }
}

struct ChunkOut {
  std::vector<float> verts;
  std::vector<Corner> corners;  // 3 per triangle
  float bbox[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
};

// Records of [b, e) (b at a line start): fgets segmentation, each record
// copied into a NUL-terminated buffer and parsed.
void parse_chunk(const char* b, const char* e, ChunkOut& out) {
  std::vector<char> buf(kLineCap + 1);
  out.verts.reserve(size_t(e - b) / 24);
  out.corners.reserve(size_t(e - b) / 16);
  Record r;
  while (b < e) {
    const size_t span = std::min<size_t>(size_t(e - b), kLineCap - 1);
    const char* nl = static_cast<const char*>(std::memchr(b, '\n', span));
    const size_t n = nl ? size_t(nl - b) + 1 : span;
    std::memcpy(buf.data(), b, n);
    buf[n] = '\0';
    b += n;
    parse_record(buf.data(), r);
    if (r.kind == 1) {
      grow(out.bbox, r.p);
      out.verts.insert(out.verts.end(), r.p, r.p + 3);
    } else if (r.kind == 2) {
      const uint64_t nv = out.verts.size() / 3;
      Corner c0[3];
      for (int i = 0; i < 3; ++i) c0[i] = r.got[0][i] ? corner(r.iv[0][i], nv) : Corner{-1, 0};
      out.corners.insert(out.corners.end(), c0, c0 + 3);
      if (r.ntri == 2)
        for (int i = 0; i < 3; ++i) out.corners.push_back(r.got[1][i] ? corner(r.iv[1][i], nv) : c0[i]);
    }
  }
}

template <class F>
void parallel_for(unsigned threads, size_t n, F&& f) {
  if (threads <= 1 || n <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < std::min<size_t>(threads, n); ++t)
    pool.emplace_back([&] {
      for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
    });
  for (auto& th : pool) th.join();
}

}  // namespace

bool Scene::loadObj(const std::string& path, bool tryLoadBinCache, bool writeBinCache, unsigned threads) {
  const std::string cache = path + ".bincache";
  if (tryLoadBinCache) {
    std::ifstream probe(cache);
    if (probe.good()) {
      probe.close();
      if (!loadBinCache(cache)) return false;
      buildTriVector(threads);
      return true;
    }
  }
  if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
  // the file mapped read-only: the threads fault in their own pieces
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) return false;
  struct stat st;
  if (::fstat(fd, &st) != 0) {
    ::close(fd);
    return false;
  }
  const size_t n = size_t(st.st_size);
  const char* text = nullptr;
  void* map = nullptr;
  if (n) {
    map = ::mmap(nullptr, n, PROT_READ, MAP_PRIVATE, fd, 0);
    if (map == MAP_FAILED) {
      ::close(fd);
      return false;
    }
    text = static_cast<const char*>(map);
  }
  ::close(fd);
  // chunks start at line starts
  const size_t nchunks = threads == 1 ? 1 : std::max<size_t>(1, std::min<size_t>(size_t(threads) * 8, n / 65536 + 1));
  std::vector<size_t> cut(nchunks + 1, n);
  cut[0] = 0;
  for (size_t c = 1; c < nchunks; ++c) {
    size_t at = std::max(cut[c - 1], n / nchunks * c);
    const char* nl = at < n ? static_cast<const char*>(std::memchr(text + at, '\n', n - at)) : nullptr;
    cut[c] = nl ? size_t(nl - text) + 1 : n;
  }
  std::vector<ChunkOut> part(nchunks);
  parallel_for(threads, nchunks, [&](size_t c) { parse_chunk(text + cut[c], text + cut[c + 1], part[c]); });
  if (map) ::munmap(map, n);
  std::vector<uint64_t> vbase(nchunks + 1, 0), tbase(nchunks + 1, 0);
  bbox_[0] = bbox_[1] = bbox_[2] = FLT_MAX;
  bbox_[3] = bbox_[4] = bbox_[5] = -FLT_MAX;
  for (size_t c = 0; c < nchunks; ++c) {
    vbase[c + 1] = vbase[c] + part[c].verts.size() / 3;
    tbase[c + 1] = tbase[c] + part[c].corners.size() / 3;
    const float lo[3] = {part[c].bbox[0], part[c].bbox[1], part[c].bbox[2]};
    const float hi[3] = {part[c].bbox[3], part[c].bbox[4], part[c].bbox[5]};
    if (!part[c].verts.empty()) {
      grow(bbox_, lo);
      grow(bbox_, hi);
    }
  }
  verts_.resize(3 * vbase[nchunks]);
  tri_idx_.resize(3 * tbase[nchunks]);
  parallel_for(threads, nchunks, [&](size_t c) {
    std::copy(part[c].verts.begin(), part[c].verts.end(), verts_.begin() + 3 * vbase[c]);
    uint64_t* out = tri_idx_.data() + 3 * tbase[c];
    for (const Corner& k : part[c].corners) *out++ = k.rel ? uint64_t(int64_t(vbase[c]) + k.v) : uint64_t(k.v);
    ChunkOut().verts.swap(part[c].verts);
  });
  tri_nidx_.assign(tri_idx_.size(), 0);
  if (writeBinCache) saveBinCache(cache);
  buildTriVector(threads);
  return true;
}

void Scene::buildTriVector(unsigned threads) {
  if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
  const uint64_t nv = verts_.size() / 3;
  const uint64_t nt = tri_idx_.size() / 3;
  const size_t nb = std::max<size_t>(1, std::min<uint64_t>(uint64_t(threads) * 8, nt / 16384 + 1));
  std::vector<uint64_t> keep(nb + 1, 0);
  auto range = [&](size_t b) { return std::make_pair(nt * b / nb, nt * (b + 1) / nb); };
  auto ok = [&](uint64_t t) {
    return tri_idx_[3 * t] < nv && tri_idx_[3 * t + 1] < nv && tri_idx_[3 * t + 2] < nv;
  };
  parallel_for(threads, nb, [&](size_t b) {
    uint64_t k = 0;
    for (uint64_t t = range(b).first; t < range(b).second; ++t) k += ok(t);
    keep[b + 1] = k;
  });
  for (size_t b = 0; b < nb; ++b) keep[b + 1] += keep[b];
  tris_.resize(9 * keep[nb]);
  parallel_for(threads, nb, [&](size_t b) {
    float* o = tris_.data() + 9 * keep[b];
    for (uint64_t t = range(b).first; t < range(b).second; ++t)
      if (ok(t))
        for (int k = 0; k < 3; ++k, o += 3) std::memcpy(o, &verts_[3 * tri_idx_[3 * t + k]], 12);
  });
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

struct svdag_scene {
  svdag::Scene s;
};

extern "C" int svdag_scene_load_obj(const char* path, uint32_t threads, int use_bincache, int write_bincache,
                                    svdag_scene** out) {
  if (!path || !out) return 1;
  *out = nullptr;
  svdag_scene* h = new svdag_scene;
  if (!h->s.loadObj(path, use_bincache != 0, write_bincache != 0, threads)) {
    delete h;
    return 2;
  }
  *out = h;
  return 0;
}

extern "C" uint64_t svdag_scene_triangle_count(const svdag_scene* s) { return s ? s->s.nTriangles() : 0; }

extern "C" const float* svdag_scene_triangles(const svdag_scene* s) {
  return s && s->s.nTriangles() ? s->s.triangles().data() : nullptr;
}

extern "C" int svdag_scene_bbox(const svdag_scene* s, float bbox[6]) {
  if (!s || !bbox) return 1;
  std::memcpy(bbox, s->s.bbox(), 24);
  return 0;
}

extern "C" void svdag_scene_free(svdag_scene* s) { delete s; }
