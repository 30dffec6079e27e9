// Writers of the reference's output formats (.svdag, .ussvdag, .ssvdag /
// .esvdag), byte-compatible with the reference's savers so its viewer loads
// the files unchanged.  The layouts are fixed by the reference:
//   .svdag   src/symvox/encoded_svdag.cpp:76-199
//   .ussvdag src/symvox/encoded_ussvdag.cpp:60-170
//   .ssvdag  src/symvox/encoded_ssvdag.cpp:84-466
// The SSVDAG per-level order comes from std::sort (unstable) on reference
// counts; it is called here with the same comparator on the same input order,
// so libstdc++ produces the same permutation.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <utility>

#include "octree_host.hpp"

namespace svdag {
namespace {

void write_header(std::ofstream& f, const float bbox[6], float rootSide, uint32_t levels, uint64_t nNodes) {
  f.write(reinterpret_cast<const char*>(bbox), 12);
  f.write(reinterpret_cast<const char*>(bbox + 3), 12);
  f.write(reinterpret_cast<const char*>(&rootSide), 4);
  f.write(reinterpret_cast<const char*>(&levels), 4);
  const uint32_t nn = uint32_t(nNodes);  // the reference writes the low 4 bytes of a size_t
  f.write(reinterpret_cast<const char*>(&nn), 4);
}

// Absolute position of every node in the single pointer stream: inner nodes
// take 1 + popcount words, leaves 1 word.
uint32_t true_pointers(const NodeData& d, uint32_t levels, std::vector<uint32_t>& ptr) {
  uint32_t counter = 0;
  for (uint32_t lev = 0; lev < levels; ++lev)
    for (const Node& n : d[lev]) {
      ptr.push_back(counter);
      counter += (lev < levels - 1) ? n.getNChildren() + 1 : 1;
    }
  return counter;
}

uint8_t permute_mask(uint8_t m, bool x, bool y, bool z) {
  const int flip = (x ? 4 : 0) | (y ? 2 : 0) | (z ? 1 : 0);
  uint8_t r = 0;
  for (int c = 0; c < 8; ++c)
    if ((m >> c) & 1u) r |= uint8_t(1u << (c ^ flip));
  return r;
}

}  // namespace

bool EncodedSVDAG::encode(const NodeData& d, const float bb[6], float rs, uint64_t nn, State st) {
  if (st != S_DAG) return false;  // the reference refuses other states (encoded_svdag.cpp:109-112)
  std::memcpy(bbox, bb, sizeof(bbox));
  rootSide = rs;
  levels = uint32_t(d.size());
  nNodes = nn;
  data.clear();
  std::vector<uint32_t> ptr;
  firstLeafPtr = true_pointers(d, levels, ptr);
  // cumulative level sizes, for child pointers into other levels (CSVDAG)
  std::vector<uint64_t> acc(levels);
  uint64_t a = 0;
  for (uint32_t lev = 0; lev < levels; ++lev) { a += d[lev].size(); acc[lev] = a; }
  data.reserve(firstLeafPtr);
  for (uint32_t lev = 0; lev < levels; ++lev) {
    for (const Node& n : d[lev]) {
      data.push_back(uint32_t(n.childrenBitmask));
      if (data.size() >= firstLeafPtr) continue;  // leaves: mask word only
      for (int k = 7; k >= 0; --k) {
        if (n.children[k] == kNullNode) continue;
        const uint64_t off = (n.childLevels[k] == 0) ? 0 : acc[n.childLevels[k] - 1];
        const uint64_t g = uint64_t(n.children[k]) + off;
        // a CSVDAG pointer the reference leaves unresolved (0xFFFFFFFF) has no
        // target; it is written as 0xFFFFFFFF
        data.push_back(g < ptr.size() ? ptr[g] : 0xFFFFFFFFu);
      }
    }
  }
  return true;
}

namespace {
// The device-built stream of `o` in format f into `data`; false when the
// octree's state does not fit the format.
bool gpu_stream(const GeomOctree& o, uint32_t f, std::vector<uint32_t>& data) {
  uint64_t n = 0;
  if (svdag_encode(o.handle(), f, nullptr, 0, &n) != SVDAG_OK) return false;
  data.resize(n);
  return svdag_encode(o.handle(), f, data.data(), n, &n) == SVDAG_OK;
}
}  // namespace

bool EncodedSVDAG::encode(const GeomOctree& o) {
  if (o.getState() != S_DAG) return false;
  if (!gpu_stream(o, SVDAG_FORMAT_SVDAG, data)) return false;
  std::memcpy(bbox, o.getSceneBBox(), sizeof(bbox));
  rootSide = o.getRootSide();
  levels = o.getLevels();
  nNodes = o.getNNodes();
  firstLeafPtr = uint32_t(data.size());  // the reference writes the word count here
  return true;
}

bool EncodedUSSVDAG::encode(const GeomOctree& o) {
  if (o.getState() != S_SDAG) return false;
  if (!gpu_stream(o, SVDAG_FORMAT_USSVDAG, data)) return false;
  std::memcpy(bbox, o.getSceneBBox(), sizeof(bbox));
  rootSide = o.getRootSide();
  levels = o.getLevels();
  nNodes = o.getNNodes();
  firstLeafPtr = uint32_t(data.size());
  return true;
}

bool EncodedSSVDAG::encode(const GeomOctree& o) {
  if (o.getState() != S_SDAG && o.getState() != S_DAG) return false;  // encoded_ssvdag.cpp:218-221
  uint64_t ni = 0, nl = 0;
  uint32_t no = 0;
  if (svdag_encode_ssvdag(o.handle(), &ni, &nl, &no) != SVDAG_OK) return false;
  inner.resize(ni);
  leaves.resize(nl);
  levelOffsets.resize(no);
  if (svdag_download_ssvdag(o.handle(), inner.data(), leaves.data(), levelOffsets.data()) != SVDAG_OK) return false;
  std::memcpy(bbox, o.getSceneBBox(), sizeof(bbox));
  rootSide = o.getRootSide();
  levels = o.getLevels();
  nNodes = o.getNNodes();
  return true;
}

bool EncodedSVDAG::save(const std::string& path) const {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  write_header(f, bbox, rootSide, levels, nNodes);
  f.write(reinterpret_cast<const char*>(&firstLeafPtr), 4);
  const uint32_t count = uint32_t(data.size());
  f.write(reinterpret_cast<const char*>(&count), 4);
  f.write(reinterpret_cast<const char*>(data.data()), std::streamsize(4) * count);
  return bool(f);
}

bool EncodedSVDAG::load(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  uint32_t nn = 0, count = 0;
  f.read(reinterpret_cast<char*>(bbox), 12);
  f.read(reinterpret_cast<char*>(bbox + 3), 12);
  f.read(reinterpret_cast<char*>(&rootSide), 4);
  f.read(reinterpret_cast<char*>(&levels), 4);
  f.read(reinterpret_cast<char*>(&nn), 4);
  f.read(reinterpret_cast<char*>(&firstLeafPtr), 4);
  f.read(reinterpret_cast<char*>(&count), 4);
  nNodes = nn;
  data.resize(count);
  f.read(reinterpret_cast<char*>(data.data()), std::streamsize(4) * count);
  return bool(f) && levels >= 1;
}

NodeData EncodedSVDAG::decode() const {
  NodeData d(levels);
  // pass 1: walk the stream; a level ends where the smallest child pointer
  // of the level above begins; remember the pointer words before each node
  std::vector<uint64_t> level_start(levels, ~0ull);
  level_start[0] = 0;
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> ptrs_before(levels);  // (position, pointers before)
  uint32_t lev = 0;
  uint32_t nptr = 0;
  for (uint64_t i = 0; i < data.size(); ++i) {
    if (lev + 1 < levels && i == level_start[lev + 1]) { ++lev; nptr = 0; }
    Node n;
    n.childrenBitmask = uint8_t(data[i]);
    ptrs_before[lev].push_back(std::make_pair(uint32_t(i), nptr));
    if (lev + 1 < levels) {
      int k = 0;
      for (int c = 7; c >= 0; --c)
        if (n.existsChild(c)) {
          n.children[c] = data[i + 1 + k];
          ++k;
          if (n.children[c] < level_start[lev + 1]) level_start[lev + 1] = n.children[c];
        }
      i += k;
      nptr += k;
    }
    d[lev].push_back(n);
  }
  // pass 2: absolute positions -> per-level indices
  uint64_t start = 0;
  for (uint32_t l = 0; l + 1 < levels; ++l) {
    start += d[l].size();
    for (const Node& n : d[l]) start += n.getNChildren();
    const auto& pb = ptrs_before[l + 1];
    for (Node& n : d[l]) {
      for (int c = 0; c < 8; ++c) {
        if (!n.existsChild(c)) { n.children[c] = kNullNode; continue; }
        const uint32_t pos = n.children[c];
        auto it = std::lower_bound(pb.begin(), pb.end(), std::make_pair(pos, 0u),
                                   [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                                     return a.first < b.first;
                                   });
        const uint32_t before = (it != pb.end() && it->first == pos) ? it->second : 0u;
        n.children[c] = uint32_t(pos - start - before);
      }
    }
  }
  return d;
}

bool EncodedUSSVDAG::encode(const NodeData& d, const float bb[6], float rs, uint64_t nn, State st) {
  if (st != S_SDAG) return false;  // encoded_ussvdag.cpp:90-93
  std::memcpy(bbox, bb, sizeof(bbox));
  rootSide = rs;
  levels = uint32_t(d.size());
  nNodes = nn;
  data.clear();
  std::vector<uint32_t> ptr;
  firstLeafPtr = true_pointers(d, levels, ptr);
  uint64_t acc = 0;
  for (uint32_t lev = 0; lev < levels; ++lev) {
    acc += d[lev].size();
    for (const Node& n : d[lev]) {
      data.push_back(uint32_t(n.childrenMirroredBitmask[2]) << 24 | uint32_t(n.childrenMirroredBitmask[1]) << 16 |
                     uint32_t(n.childrenMirroredBitmask[0]) << 8 | uint32_t(n.childrenBitmask));
      if (data.size() >= firstLeafPtr) continue;
      for (int k = 7; k >= 0; --k)
        if (n.children[k] != kNullNode) data.push_back(ptr[uint64_t(n.children[k]) + acc]);
    }
  }
  return true;
}

bool EncodedUSSVDAG::save(const std::string& path) const {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  write_header(f, bbox, rootSide, levels, nNodes);
  f.write(reinterpret_cast<const char*>(&firstLeafPtr), 4);
  const uint32_t count = uint32_t(data.size());
  f.write(reinterpret_cast<const char*>(&count), 4);
  f.write(reinterpret_cast<const char*>(data.data()), std::streamsize(4) * count);
  return bool(f);
}

bool EncodedSSVDAG::encode(const NodeData& d, const float bb[6], float rs, uint64_t nn, State st) {
  if (st != S_SDAG && st != S_DAG) return false;  // encoded_ssvdag.cpp:218-221
  std::memcpy(bbox, bb, sizeof(bbox));
  rootSide = rs;
  levels = uint32_t(d.size());
  nNodes = nn;
  if (levels < 3) return false;
  inner.clear();
  leaves.clear();
  levelOffsets.clear();
  std::vector<std::vector<uint16_t>> enc(levels - 2);
  std::vector<std::pair<uint32_t, uint32_t>> hist;
  std::vector<uint32_t> indirection;
  for (int lev = int(levels) - 2; lev >= 0; --lev) {
    const std::vector<Node>& L = d[lev];
    if (L.size() > (1u << 30)) return false;  // the reference exits (encoded_ssvdag.cpp:251-254)
    hist.resize(L.size());
    for (uint32_t i = 0; i < L.size(); ++i) hist[i] = std::make_pair(i, 0u);
    if (lev > 0) {
      for (const Node& p : d[lev - 1])
        for (int c = 0; c < 8; ++c)
          if (p.existsChildPointer(c)) hist[p.children[c]].second++;
      std::sort(hist.begin(), hist.end(),
                [](std::pair<uint32_t, uint32_t> a, std::pair<uint32_t, uint32_t> b) { return a.second > b.second; });
    }
    std::vector<uint32_t> next(L.size());
    if (lev == int(levels) - 2) {
      // 4^3 leaf bricks: the 8 mirrored child masks, then voxel (x,y,z) of the
      // brick to bit x + 4y + 16z (encoded_ssvdag.cpp:280-351)
      leaves.resize(hist.size() * 8);
      for (uint32_t i = 0; i < hist.size(); ++i) {
        next[hist[i].first] = i;
        const Node& n = L[hist[i].first];
        uint8_t buf[8];
        for (int c = 7; c >= 0; --c) {
          if (n.existsChildPointer(c)) {
            const Node& cn = d[lev + 1][n.children[c]];
            buf[c] = permute_mask(cn.childrenBitmask, n.getChildMirrorBit(0, c), n.getChildMirrorBit(1, c),
                                  n.getChildMirrorBit(2, c));
          } else {
            buf[c] = 0;
          }
        }
        uint8_t out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int bit_out = 0;
        for (int z = 0; z < 4; ++z)
          for (int y = 0; y < 4; ++y)
            for (int x = 0; x < 4; ++x, ++bit_out) {
              const int byte_id = (x / 2) + (y / 2) * 2 + (z / 2) * 4;
              const int bit_id = (x % 2) + (y % 2) * 2 + (z % 2) * 4;
              const uint8_t v = (buf[byte_id] >> bit_id) & 1u;
              out[bit_out / 8] |= uint8_t(v << (bit_out % 8));
            }
        std::memcpy(&leaves[size_t(i) * 8], out, 8);
      }
    } else {
      // inner nodes: u16 header (2 bits per child: 01 16-bit pointer, 10/11
      // 32-bit pointer whose bit 29 is the low header bit), pointers carry
      // the three mirror bits on top (encoded_ssvdag.cpp:352-430)
      for (uint32_t i = 0; i < hist.size(); ++i) {
        const Node& n = L[hist[i].first];
        uint16_t tmp[20];
        tmp[0] = 0;
        int sz = 1;
        for (int c = 7; c >= 0; --c) {
          if (!n.existsChild(c)) continue;
          const uint32_t addr = indirection[n.children[c]];
          if (addr < (1u << 13)) {
            uint16_t p = uint16_t(addr);
            tmp[0] |= uint16_t(1u << (2 * c));
            if (n.getChildMirrorBit(0, c)) p |= 1u << 13;
            if (n.getChildMirrorBit(1, c)) p |= 1u << 14;
            if (n.getChildMirrorBit(2, c)) p |= 1u << 15;
            tmp[sz++] = p;
          } else if (addr < (1u << 30)) {
            uint32_t p = addr;
            if (p & (1u << 29)) {
              tmp[0] |= uint16_t(3u << (2 * c));
              p &= ~(1u << 29);
            } else {
              tmp[0] |= uint16_t(2u << (2 * c));
            }
            if (n.getChildMirrorBit(0, c)) p |= 1u << 29;
            if (n.getChildMirrorBit(1, c)) p |= 1u << 30;
            if (n.getChildMirrorBit(2, c)) p |= 1u << 31;
            tmp[sz++] = uint16_t(p >> 16);
            tmp[sz++] = uint16_t(p & 0xFFFFu);
          } else {
            std::fprintf(stderr, "EncodedSSVDAG: pointer %u exceeds 2^30\n", addr);
          }
        }
        next[hist[i].first] = uint32_t(enc[lev].size());
        enc[lev].insert(enc[lev].end(), tmp, tmp + sz);
      }
    }
    indirection.swap(next);
  }
  levelOffsets.resize(levels - 2);
  levelOffsets[0] = 0;
  for (size_t i = 1; i < levelOffsets.size(); ++i) levelOffsets[i] = uint32_t(enc[i - 1].size()) + levelOffsets[i - 1];
  for (auto& e : enc) inner.insert(inner.end(), e.begin(), e.end());
  return true;
}

bool EncodedSSVDAG::save(const std::string& path) const {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  write_header(f, bbox, rootSide, levels, nNodes);
  uint32_t count = uint32_t(inner.size());
  f.write(reinterpret_cast<const char*>(&count), 4);
  f.write(reinterpret_cast<const char*>(inner.data()), std::streamsize(2) * count);
  count = uint32_t(leaves.size());
  f.write(reinterpret_cast<const char*>(&count), 4);
  f.write(reinterpret_cast<const char*>(leaves.data()), count);
  count = uint32_t(levelOffsets.size());
  f.write(reinterpret_cast<const char*>(&count), 4);
  f.write(reinterpret_cast<const char*>(levelOffsets.data()), std::streamsize(4) * count);
  return bool(f);
}

}  // namespace svdag

// ---------------------------------------------------------------------------
// C entry for tests: encode pools given as 48-byte records per level
// (hdr u32, children 8 x u32, childLevels 8 x u8, invariant u8, pad 3).
extern "C" int svdag_write_encoded(const char* path, int format, uint32_t levels, const uint64_t* counts,
                                   const uint8_t* const* recs, const float bbox[6], float root_side, uint64_t n_nodes,
                                   int state) {
  using namespace svdag;
  NodeData d(levels);
  for (uint32_t l = 0; l < levels; ++l) {
    d[l].resize(counts[l]);
    for (uint64_t i = 0; i < counts[l]; ++i) {
      const uint8_t* r = recs[l] + 48 * i;
      Node& n = d[l][i];
      uint32_t hdr;
      std::memcpy(&hdr, r, 4);
      n.childrenBitmask = uint8_t(hdr);
      n.childrenMirroredBitmask[0] = uint8_t(hdr >> 8);
      n.childrenMirroredBitmask[1] = uint8_t(hdr >> 16);
      n.childrenMirroredBitmask[2] = uint8_t(hdr >> 24);
      std::memcpy(n.children, r + 4, 32);
      for (int c = 0; c < 8; ++c) n.childLevels[c] = (r[36 + c] == 0xFF) ? 0xFFFFFFFFu : r[36 + c];
      n.invariantBitmask = r[44];
    }
  }
  bool ok = false;
  switch (format) {
    case 0: { EncodedSVDAG e; ok = e.encode(d, bbox, root_side, n_nodes, State(state)) && e.save(path); break; }
    case 1: { EncodedUSSVDAG e; ok = e.encode(d, bbox, root_side, n_nodes, State(state)) && e.save(path); break; }
    case 2: { EncodedSSVDAG e; ok = e.encode(d, bbox, root_side, n_nodes, State(state)) && e.save(path); break; }
    default: ok = false;
  }
  return ok ? 0 : -1;
}
