// CPU oracle: a restatement of the reference SymVox / SVDAG-Compression
// build path.  TEST INFRASTRUCTURE ONLY (see svdag_oracle.h): it is the
// checker the CUDA path is compared against, never part of the product.
//
// Each function cites the reference lines it restates (paths relative to the
// reference project).  The data structures follow the reference's own
// (ordered maps, explicit DFS stack) so that its CPU timing is representative
// of the reference when it is used as the CPU baseline.
//
// Build with -ffp-contract=off: the fp64 triangle/box test must not be fused.
#include "svdag_oracle.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <stack>
#include <utility>
#include <vector>

namespace {

const uint32_t kNull = 0xFFFFFFFEu;  // Octree::nullNode (src/symvox/octree.cpp:22)

// GeomOctree::Node (src/symvox/octree.hpp:57-85, src/symvox/geom_octree.hpp:59-96)
struct Node {
  uint8_t mask;
  uint8_t mir[3];
  uint8_t inv;
  uint32_t ch[8];
  uint32_t clev[8];
  Node() : mask(0), inv(0) {
    mir[0] = mir[1] = mir[2] = 0;
    for (int c = 0; c < 8; ++c) { ch[c] = kNull; clev[c] = 0xFFFFFFFFu; }
  }
  bool has_ptr(int c) const { return ch[c] != kNull; }
  bool has_child(int c) const { return (mask >> c) & 1u; }
};

// Node::operator== / operator< (src/symvox/octree_node.cpp:39-86): the key is
// (childrenBitmask, children[0..7], childrenMirroredBitmask[0..2]).
inline bool key_eq(const Node& a, const Node& b) {
  if (a.mask != b.mask) return false;
  for (int c = 0; c < 8; ++c) if (a.ch[c] != b.ch[c]) return false;
  return a.mir[0] == b.mir[0] && a.mir[1] == b.mir[1] && a.mir[2] == b.mir[2];
}
struct KeyLess {
  bool operator()(const Node& a, const Node& b) const {
    if (a.mask != b.mask) return a.mask < b.mask;
    for (int c = 0; c < 8; ++c) if (a.ch[c] != b.ch[c]) return a.ch[c] < b.ch[c];
    for (int k = 0; k < 3; ++k) if (a.mir[k] != b.mir[k]) return a.mir[k] < b.mir[k];
    return false;
  }
};

// Node::mirror (src/symvox/octree_node.cpp:88-195): child index 4x+2y+z, an
// x mirror swaps c <-> c^4, y swaps c <-> c^2, z swaps c <-> c^1, for the
// mask, the three mirror masks and the child pointers; then the mirror bit of
// every mirrored axis is toggled for each child that has a pointer.  The
// result's invariant mask is 0 (the reference builds it in a fresh Node).
inline uint8_t permute_bits(uint8_t m, int flip) {
  uint8_t r = 0;
  for (int c = 0; c < 8; ++c) if ((m >> c) & 1u) r |= uint8_t(1u << (c ^ flip));
  return r;
}
Node mirror(const Node& n, bool x, bool y, bool z) {
  int flip = (x ? 4 : 0) | (y ? 2 : 0) | (z ? 1 : 0);
  Node r;
  if (flip == 0) return n;
  r.mask = permute_bits(n.mask, flip);
  for (int k = 0; k < 3; ++k) r.mir[k] = permute_bits(n.mir[k], flip);
  for (int c = 0; c < 8; ++c) r.ch[c] = n.ch[c ^ flip];
  r.inv = 0;
  for (int c = 0; c < 8; ++c) {
    if (r.has_ptr(c)) {
      if (x) r.mir[0] ^= uint8_t(1u << c);
      if (y) r.mir[1] ^= uint8_t(1u << c);
      if (z) r.mir[2] ^= uint8_t(1u << c);
    }
  }
  return r;
}

inline unsigned popc8(uint8_t m) { return unsigned(__builtin_popcount(m)); }

// ---------------------------------------------------------------------------
// Triangle / box overlap, fp64 (src/symvox/test_triangle_box.cpp:38-184).
// Every operation below is one IEEE double operation in the reference's order.

bool plane_box_overlap(const double n[3], const double v[3], double maxbox) {
  double vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    if (n[q] > 0.0) { vmin[q] = -maxbox - v[q]; vmax[q] = maxbox - v[q]; }
    else            { vmin[q] = maxbox - v[q];  vmax[q] = -maxbox - v[q]; }
  }
  double d = n[0] * vmin[0];
  d = d + n[1] * vmin[1];
  d = d + n[2] * vmin[2];
  if (d > 0.0) return false;
  double e = n[0] * vmax[0];
  e = e + n[1] * vmax[1];
  e = e + n[2] * vmax[2];
  if (e >= 0.0) return true;
  return false;
}

inline bool axis_reject(double pa, double pb, double fa, double fb, double h, bool b_first) {
  double mn, mx;
  // Z12 orders its pair as (p2 < p1); the other macros as (first < second).
  if (b_first) { if (pb < pa) { mn = pb; mx = pa; } else { mn = pa; mx = pb; } }
  else         { if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; } }
  double rad = (fa + fb) * h;
  return (mn > rad || mx < -rad);
}

bool tri_box(const double c[3], double h, const float* t) {
  double v0[3], v1[3], v2[3], e0[3], e1[3], e2[3];
  for (int k = 0; k < 3; ++k) {
    v0[k] = double(t[k]) - c[k];
    v1[k] = double(t[3 + k]) - c[k];
    v2[k] = double(t[6 + k]) - c[k];
  }
  for (int k = 0; k < 3; ++k) { e0[k] = v1[k] - v0[k]; e1[k] = v2[k] - v1[k]; e2[k] = v0[k] - v2[k]; }
  const int X = 0, Y = 1, Z = 2;
  double fex, fey, fez, a, b;
  // edge 0: X01, Y02, Z12
  fex = std::fabs(e0[X]); fey = std::fabs(e0[Y]); fez = std::fabs(e0[Z]);
  a = e0[Z]; b = e0[Y];
  if (axis_reject(a * v0[Y] - b * v0[Z], a * v2[Y] - b * v2[Z], fez, fey, h, false)) return false;
  a = e0[Z]; b = e0[X];
  if (axis_reject(-a * v0[X] + b * v0[Z], -a * v2[X] + b * v2[Z], fez, fex, h, false)) return false;
  a = e0[Y]; b = e0[X];
  if (axis_reject(a * v1[X] - b * v1[Y], a * v2[X] - b * v2[Y], fey, fex, h, true)) return false;
  // edge 1: X01, Y02, Z0
  fex = std::fabs(e1[X]); fey = std::fabs(e1[Y]); fez = std::fabs(e1[Z]);
  a = e1[Z]; b = e1[Y];
  if (axis_reject(a * v0[Y] - b * v0[Z], a * v2[Y] - b * v2[Z], fez, fey, h, false)) return false;
  a = e1[Z]; b = e1[X];
  if (axis_reject(-a * v0[X] + b * v0[Z], -a * v2[X] + b * v2[Z], fez, fex, h, false)) return false;
  a = e1[Y]; b = e1[X];
  if (axis_reject(a * v0[X] - b * v0[Y], a * v1[X] - b * v1[Y], fey, fex, h, false)) return false;
  // edge 2: X2, Y1, Z12
  fex = std::fabs(e2[X]); fey = std::fabs(e2[Y]); fez = std::fabs(e2[Z]);
  a = e2[Z]; b = e2[Y];
  if (axis_reject(a * v0[Y] - b * v0[Z], a * v1[Y] - b * v1[Z], fez, fey, h, false)) return false;
  a = e2[Z]; b = e2[X];
  if (axis_reject(-a * v0[X] + b * v0[Z], -a * v1[X] + b * v1[Z], fez, fex, h, false)) return false;
  a = e2[Y]; b = e2[X];
  if (axis_reject(a * v1[X] - b * v1[Y], a * v2[X] - b * v2[Y], fey, fex, h, true)) return false;
  // bounding-box overlap per axis (FINDMINMAX)
  for (int k = 0; k < 3; ++k) {
    double mn = v0[k], mx = v0[k];
    if (v1[k] < mn) mn = v1[k];
    if (v1[k] > mx) mx = v1[k];
    if (v2[k] < mn) mn = v2[k];
    if (v2[k] > mx) mx = v2[k];
    if (mn > h || mx < -h) return false;
  }
  // plane of the triangle: normal = e0 x e1
  double nrm[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
  return plane_box_overlap(nrm, v0, h);
}

}  // namespace

struct ora_octree {
  std::vector<std::vector<Node>> d;
  uint32_t levels = 0;
  int state = 0;  // 0 empty, 1 SVO, 2 DAG, 3 SDAG
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  double root_side = 0;
  uint64_t n_voxels = 0, n_nodes = 0;
  ora_stats st{};
  std::vector<std::vector<uint8_t>> outside;  // outsideMask per node after the flood fill
};

namespace {

// Octree::resizeSceneBbox / buildSVO prologue (src/symvox/octree.hpp:101-105,
// src/symvox/geom_octree.cpp:176-184): float box, root side = largest float side.
void set_box(ora_octree* o, const double bb[6]) {
  for (int k = 0; k < 6; ++k) o->bbox[k] = float(bb[k]);
  float s[3];
  for (int k = 0; k < 3; ++k) s[k] = ((o->bbox[3 + k] - o->bbox[k]) * 0.5f) * 2.0f;
  o->root_side = double(std::max(std::max(s[0], s[1]), s[2]));
}

// GeomOctree::cleanEmptyNodes (src/symvox/geom_octree.cpp:437-456)
void clean_empty(ora_octree* o) {
  for (int lev = int(o->levels) - 1; lev > 0; --lev) {
    std::vector<char> empty(o->d[lev].size());
    for (size_t i = 0; i < o->d[lev].size(); ++i) empty[i] = (o->d[lev][i].mask == 0);
    for (auto& p : o->d[lev - 1]) {
      for (int j = 0; j < 8; ++j) {
        if (p.ch[j] != kNull && p.ch[j] < empty.size() && empty[p.ch[j]]) {
          p.mask &= uint8_t(~(1u << j));
          p.ch[j] = kNull;
        }
      }
    }
  }
}

// GeomOctree::buildSVO (src/symvox/geom_octree.cpp:171-280)
void build_svo(ora_octree* o, const float* tris, uint64_t n_tris, const double bb[6], uint32_t levels) {
  set_box(o, bb);
  o->levels = levels;
  o->d.assign(levels, std::vector<Node>());
  o->d[0].push_back(Node());
  o->n_nodes = 0;
  o->n_voxels = 0;
  double root_c[3];
  for (int k = 0; k < 3; ++k) root_c[k] = (bb[k] + bb[3 + k]) * 0.5;
  struct Item { uint32_t id; uint32_t lev; double c[3]; };
  std::stack<Item> st;
  for (uint64_t t = 0; t < n_tris; ++t) {
    const float* tri = tris + 9 * t;
    Item root{0, 0, {root_c[0], root_c[1], root_c[2]}};
    st.push(root);
    while (!st.empty()) {
      Item it = st.top();
      st.pop();
      double k = o->root_side / double(1u << (it.lev + 2));  // getHalfSideD(lev+1)
      for (int i = 7; i >= 0; --i) {
        double cc[3] = {it.c[0] + ((i & 4) ? k : -k), it.c[1] + ((i & 2) ? k : -k), it.c[2] + ((i & 1) ? k : -k)};
        if (!tri_box(cc, k, tri)) continue;
        Node& node = o->d[it.lev][it.id];
        node.mask |= uint8_t(1u << i);
        if (node.ch[i] == kNull && it.lev < levels - 1) {
          node.ch[i] = uint32_t(o->d[it.lev + 1].size());
          o->d[it.lev + 1].emplace_back();
          o->n_nodes++;
        }
        if (it.lev + 1 < levels) {
          Item nx{o->d[it.lev][it.id].ch[i], it.lev + 1, {cc[0], cc[1], cc[2]}};
          st.push(nx);
        }
      }
    }
  }
  clean_empty(o);
  for (const auto& n : o->d[levels - 1]) o->n_voxels += popc8(n.mask);
  o->state = 1;
  o->st.n_nodes_svo = o->n_nodes;
  o->st.n_nodes_last_lev_svo = o->d[levels - 1].size();
  o->st.n_total_voxels = o->n_voxels;
}

// GeomOctree::toDAG (src/symvox/geom_octree.cpp:462-548)
int to_dag(ora_octree* o) {
  if (o->state != 1 && o->state != 2) return -1;
  o->n_nodes = 1;
  std::map<Node, uint32_t, KeyLess> seen;
  for (uint32_t lev = o->levels - 1; lev > 0; --lev) {
    std::vector<Node>& L = o->d[lev];
    std::vector<uint32_t> corr(L.size(), 0);
    std::vector<Node> uniq;
    seen.clear();
    for (size_t i = 0; i < L.size(); ++i) {
      const Node& n = L[i];
      if (n.mask == 0) continue;
      auto it = seen.find(n);
      if (it != seen.end()) {
        corr[i] = it->second;
      } else {
        uint32_t id = uint32_t(uniq.size());
        seen.emplace(n, id);
        corr[i] = id;
        uniq.push_back(n);
      }
    }
    L.swap(uniq);
    o->n_nodes += L.size();
    for (auto& p : o->d[lev - 1])
      for (int j = 0; j < 8; ++j)
        if (p.has_child(j)) p.ch[j] = corr[p.ch[j]];
  }
  o->state = 2;
  o->st.n_nodes_dag = o->n_nodes;
  return 0;
}

// GeomOctree::invertInvs (src/symvox/geom_octree.cpp:822-831)
void invert_invs(const ora_octree* o, Node& n, uint32_t lev, bool x, bool y, bool z) {
  for (int i = 0; i < 8; ++i) {
    if (!n.has_ptr(i)) continue;
    const Node& c = o->d[lev + 1][n.ch[i]];
    if (x && (c.inv & 1u)) n.mir[0] &= uint8_t(~(1u << i));
    if (y && (c.inv & 2u)) n.mir[1] &= uint8_t(~(1u << i));
    if (z && (c.inv & 4u)) n.mir[2] &= uint8_t(~(1u << i));
  }
}

// GeomOctree::toSDAG(false, skip_symmetry) (src/symvox/geom_octree.cpp:551-697).
// With skip_symmetry (:596-601, "pointer compression" only) every non-empty
// node is kept in order with no invariance bits and no lookups; a pointer to
// a dropped empty node keeps the default correspondence (id 0, no mirrors).
int to_sdag(ora_octree* o, bool skip_symmetry = false) {
  if (o->state != 1 && o->state != 2) return -1;
  struct Corr { uint8_t m; uint32_t id; };
  std::map<Node, uint32_t, KeyLess> seen;
  o->n_nodes = 0;
  // lookup order: identity, X, Y, Z, XY, XZ, YZ, XYZ (geom_octree.cpp:630-658)
  static const int axes[8] = {0, 4, 2, 1, 6, 5, 3, 7};
  for (uint32_t lev = o->levels - 1; lev > 0; --lev) {
    std::vector<Node>& L = o->d[lev];
    std::vector<Corr> corr(L.size(), Corr{0, 0});
    std::vector<Node> uniq;
    seen.clear();
    for (size_t i = 0; i < L.size(); ++i) {
      Node n = L[i];
      if (n.mask == 0) continue;
      if (skip_symmetry) {
        corr[i] = Corr{0, uint32_t(uniq.size())};
        uniq.push_back(n);
        continue;
      }
      if (key_eq(n, mirror(n, true, false, false))) n.inv |= 1u;
      if (key_eq(n, mirror(n, false, true, false))) n.inv |= 2u;
      if (key_eq(n, mirror(n, false, false, true))) n.inv |= 4u;
      Node var[8];
      var[0] = n;
      for (int k = 1; k < 8; ++k) {
        int a = axes[k];
        var[k] = mirror(n, a & 4, a & 2, a & 1);
        if (lev < o->levels - 1) invert_invs(o, var[k], lev, a & 4, a & 2, a & 1);
      }
      bool found = false;
      for (int k = 0; k < 8 && !found; ++k) {
        auto it = seen.find(var[k]);
        if (it != seen.end()) {
          // bit0 = X, bit1 = Y, bit2 = Z
          int a = axes[k];
          corr[i] = Corr{uint8_t(((a & 4) ? 1 : 0) | ((a & 2) ? 2 : 0) | ((a & 1) ? 4 : 0)), it->second};
          found = true;
        }
      }
      if (!found) {
        uint32_t id = uint32_t(uniq.size());
        seen.emplace(n, id);
        corr[i] = Corr{0, id};
        uniq.push_back(n);
      }
    }
    L.swap(uniq);
    o->n_nodes += L.size();
    for (auto& p : o->d[lev - 1]) {
      for (int j = 0; j < 8; ++j) {
        if (!p.has_ptr(j)) continue;
        Corr cr = corr[p.ch[j]];
        p.ch[j] = cr.id;
        if (cr.m & 1) p.mir[0] |= uint8_t(1u << j);
        if (cr.m & 2) p.mir[1] |= uint8_t(1u << j);
        if (cr.m & 4) p.mir[2] |= uint8_t(1u << j);
      }
    }
  }
  o->st.n_nodes_sdag = o->n_nodes;
  o->state = 3;
  return 0;
}

// GeomOctree::initChildLevels (src/symvox/geom_octree_extension.cpp:21-30)
void init_child_levels(ora_octree* o) {
  for (uint32_t lev = 0; lev < o->levels; ++lev)
    for (auto& n : o->d[lev])
      for (int c = 0; c < 8; ++c) n.clev[c] = lev + 1;
}

// Truncated-subtree equality "A equals the top of B" with correspondences of
// visited nodes (src/symvox/geom_octree_extension.cpp:238-290).  The map
// assignment overwrites, so a node reached twice keeps its last visit.
bool compare_subtrees(const ora_octree* o, uint32_t levA, uint32_t levB, const Node& a, const Node& b,
                      std::vector<std::map<uint32_t, std::pair<uint32_t, uint32_t>>>& visited) {
  if (a.mask != 0 && b.mask == 0) return false;
  if (levA == o->levels - 1) return a.mask == b.mask;
  for (int i = 0; i < 8; ++i) {
    if (a.has_child(i) != b.has_child(i)) return false;
    if (!a.has_child(i)) continue;
    const Node& ca = o->d[levA + 1][a.ch[i]];
    const Node& cb = o->d[levB + 1][b.ch[i]];
    visited[levA + 1][a.ch[i]] = std::make_pair(levB + 1, b.ch[i]);
    if (!compare_subtrees(o, levA + 1, levB + 1, ca, cb, visited)) return false;
  }
  return true;
}

inline uint64_t mix64(uint64_t x) {
  x ^= x >> 31; x *= 0x7FB5D329728EA185ull;
  x ^= x >> 27; x *= 0x81DADEF4BC2DD44Dull;
  x ^= x >> 33;
  return x;
}

// Depth-d structural fingerprint of every node at levels 1..levels-1: equal
// for nodes whose top d levels of masks agree.  Used only to shortlist
// candidates; equality is decided by compare_subtrees, exactly as the
// reference's hash multimap is only a shortlist (geom_octree_extension.cpp:34-74,
// 105-142, 1343-1348).
void depth_hashes(const ora_octree* o, uint32_t depth, std::vector<std::vector<uint64_t>>& h) {
  std::vector<std::vector<uint64_t>> prev(o->levels), cur(o->levels);
  for (uint32_t l = 0; l < o->levels; ++l) {
    prev[l].resize(o->d[l].size());
    for (size_t i = 0; i < o->d[l].size(); ++i) prev[l][i] = o->d[l][i].mask;
  }
  for (uint32_t dd = 1; dd <= depth; ++dd) {
    for (uint32_t l = 0; l < o->levels; ++l) {
      cur[l].assign(o->d[l].size(), 0);
      for (size_t i = 0; i < o->d[l].size(); ++i) {
        const Node& n = o->d[l][i];
        uint64_t x = mix64(0x1234567ull + n.mask);
        for (int c = 0; c < 8; ++c) {
          uint64_t v = 0x9E3779B97F4A7C15ull * uint64_t(c + 1);
          if (n.has_ptr(c) && l + 1 < o->levels) v ^= prev[n.clev[c]][n.ch[c]];
          x = mix64(x ^ v);
        }
        cur[l][i] = x;
      }
    }
    prev.swap(cur);
  }
  h.swap(prev);
}

// GeomOctree::mergeAcrossAllLevels (src/symvox/geom_octree_extension.cpp:1192-1544)
int merge_across_levels(ora_octree* o, uint64_t* n_missing) {
  const uint32_t L = o->levels;
  std::vector<std::multimap<uint64_t, uint32_t>> cand(L);
  std::vector<std::vector<uint64_t>> h;
  uint32_t cur_depth = L / 2;
  auto rebuild = [&](uint32_t depth) {
    depth_hashes(o, depth, h);
    for (uint32_t l = 0; l < L; ++l) cand[l].clear();
    // levels 1..L-1 only (buildMultiMap default range, geom_octree.hpp:146-148)
    for (uint32_t l = 1; l < L; ++l)
      for (uint32_t i = 0; i < o->d[l].size(); ++i) cand[l].insert(std::make_pair(h[l][i], i));
  };
  rebuild(cur_depth);

  std::set<uint32_t> check, next;
  // (a one-level tree has no level 1; the reference indexes past its levels
  // there, so the restatement merges nothing)
  if (L >= 2)
    for (uint32_t i = 0; i < o->d[1].size(); ++i) check.insert(i);
  std::vector<std::map<uint32_t, std::pair<uint32_t, uint32_t>>> corr(L), visited(L);
  for (uint32_t levA = 1; levA < L; ++levA) {
    uint32_t max_depth = L - levA - 1;
    if (max_depth < cur_depth) {
      cur_depth = max_depth;
      rebuild(cur_depth);
    }
    for (uint32_t idA : check) {
      const Node& a = o->d[levA][idA];
      uint64_t key = h[levA][idA];
      bool found = false;
      for (uint32_t levB = 0; levB < levA && !found; ++levB) {
        auto rng = cand[levB].equal_range(key);
        for (auto it = rng.first; it != rng.second; ++it) {
          uint32_t j = it->second;
          for (uint32_t l = 0; l < L; ++l) visited[l].clear();
          if (compare_subtrees(o, levA, levB, a, o->d[levB][j], visited)) {
            corr[levA][idA] = std::make_pair(levB, j);
            for (uint32_t l = 0; l < L; ++l) corr[l].insert(visited[l].begin(), visited[l].end());
            found = true;
            break;
          }
        }
      }
      if (!found)
        for (int i = 0; i < 8; ++i)
          if (a.has_child(i)) next.insert(a.ch[i]);
    }
    check.clear();
    check.swap(next);
  }

  uint64_t removed_total = 0, missing = 0;
  for (uint32_t l = 0; l < L; ++l) removed_total += corr[l].size();
  o->n_nodes = 1;
  for (uint32_t lev = L - 1; lev > 0; --lev) {
    std::vector<Node>& Lv = o->d[lev];
    std::vector<uint32_t> newidx(Lv.size(), 0xFFFFFFFFu);
    std::vector<Node> keep;
    for (uint32_t i = 0; i < Lv.size(); ++i) {
      if (corr[lev].count(i) == 0) { newidx[i] = uint32_t(keep.size()); keep.push_back(Lv[i]); }
    }
    Lv.swap(keep);
    o->n_nodes += Lv.size();
    for (auto& p : o->d[lev - 1]) {
      for (int j = 0; j < 8; ++j) {
        if (!p.has_child(j)) continue;
        auto it = corr[lev].find(p.ch[j]);
        if (it != corr[lev].end()) { p.clev[j] = it->second.first; p.ch[j] = it->second.second; }
        else p.ch[j] = newidx[p.ch[j]];
      }
    }
    for (uint32_t low = L - 2; low >= lev; --low) {
      for (auto& p : o->d[low]) {
        for (int j = 0; j < 8; ++j) {
          if (p.has_child(j) && p.clev[j] == lev) {
            if (newidx[p.ch[j]] == 0xFFFFFFFFu) ++missing;
            p.ch[j] = newidx[p.ch[j]];
          }
        }
      }
      if (low == 0) break;
    }
  }
  o->st.n_nodes_dag = o->n_nodes;
  o->st.n_cross_level_merged = removed_total;
  if (n_missing) *n_missing = missing;
  return 0;
}

// GeomOctree::buildDAG (src/symvox/geom_octree.cpp:289-435): a top SVO of
// step_level+1 levels, one sub-SVO + toDAG per top-level voxel (OpenMP,
// dynamic schedule), joined level by level with pointer offsets, then one
// toDAG over the whole tree.
void build_dag_chunked(ora_octree* o, const float* tris, uint64_t n_tris, const double bb[6], uint32_t levels,
                       uint32_t step_level, int n_threads) {
  const uint32_t top = step_level + 1;
  build_svo(o, tris, n_tris, bb, top);
  // centres of the top SVO's leaf nodes in creation order
  // (buildSVO's leavesCenters, geom_octree.cpp:245-246)
  std::vector<std::array<double, 3>> centers(o->d[top - 1].size());
  {
    // recompute by walking the top SVO from the root
    double rc[3];
    for (int k = 0; k < 3; ++k) rc[k] = (bb[k] + bb[3 + k]) * 0.5;
    struct W { uint32_t lev, id; double c[3]; };
    std::vector<W> stack{W{0, 0, {rc[0], rc[1], rc[2]}}};
    if (top == 1) centers[0] = {rc[0], rc[1], rc[2]};
    while (!stack.empty()) {
      W w = stack.back();
      stack.pop_back();
      if (w.lev + 1 >= top) continue;
      double k = o->root_side / double(1u << (w.lev + 2));
      const Node& n = o->d[w.lev][w.id];
      for (int i = 0; i < 8; ++i) {
        if (n.ch[i] == kNull) continue;
        double cc[3] = {w.c[0] + ((i & 4) ? k : -k), w.c[1] + ((i & 2) ? k : -k), w.c[2] + ((i & 1) ? k : -k)};
        if (w.lev + 1 == top - 1) centers[n.ch[i]] = {cc[0], cc[1], cc[2]};
        stack.push_back(W{w.lev + 1, n.ch[i], {cc[0], cc[1], cc[2]}});
      }
    }
  }
  const double lhs = o->root_side / double(1u << top);  // getHalfSideD(stepLevels-1)
  const size_t n_top = o->d[top - 1].size();
  std::vector<ora_octree*> sub(n_top * 8, nullptr);
  uint64_t svo_nodes = o->n_nodes, svo_last = 0, vox = o->n_voxels;
#pragma omp parallel for schedule(dynamic, 2) num_threads(n_threads > 0 ? n_threads : omp_get_max_threads()) reduction(+ : svo_nodes, svo_last, vox)
  for (long i = 0; i < long(n_top); ++i) {
    for (int j = 7; j >= 0; --j) {
      if (!((o->d[top - 1][i].mask >> j) & 1u)) continue;
      const auto& c = centers[i];
      double q[3] = {c[0] + ((j & 4) ? lhs : -lhs), c[1] + ((j & 2) ? lhs : -lhs), c[2] + ((j & 1) ? lhs : -lhs)};
      double sb[6];
      for (int k = 0; k < 3; ++k) { sb[k] = std::min(c[k], q[k]); sb[3 + k] = std::max(c[k], q[k]); }
      ora_octree* so = new ora_octree();
      build_svo(so, tris, n_tris, sb, levels - top);
      svo_nodes += so->n_nodes;
      svo_last += so->d[so->levels - 1].size();
      vox += so->n_voxels - 1;
      to_dag(so);
      sub[size_t(i) * 8 + j] = so;
    }
  }
  o->st.n_nodes_svo = svo_nodes;
  o->st.n_nodes_last_lev_svo = svo_last;
  o->st.n_total_voxels = vox;
  o->n_voxels = vox;
  o->d.resize(levels);
  o->levels = levels;
  for (size_t i = 0; i < n_top; ++i) {
    for (int j = 7; j >= 0; --j) {
      if (!((o->d[top - 1][i].mask >> j) & 1u)) continue;
      ora_octree* so = sub[i * 8 + j];
      o->d[top - 1][i].ch[j] = uint32_t(o->d[top].size());
      for (uint32_t k = top; k < levels; ++k) {
        if (k < levels - 1) {
          uint32_t off = uint32_t(o->d[k + 1].size());
          for (auto& n : so->d[k - top])
            for (int c = 0; c < 8; ++c)
              if (n.has_ptr(c)) n.ch[c] += off;
        }
        o->d[k].insert(o->d[k].end(), so->d[k - top].begin(), so->d[k - top].end());
      }
      delete so;
    }
  }
  o->state = 1;
  to_dag(o);
}

// GeomOctree::hiddenGeometryFloodfill (src/symvox/geom_octree_extension.cpp:
// 1651-1891) restated.  A traversal node is a cell: (depth, node of the
// level above, child slot); its parent cell follows from the SVO's single
// parent per node.  Neighbours are the leaf cells sharing a face
// (getNeighbourGrtrEqSz + getNeighboursSmSz, :1702-1775); the fill starts at
// the deepest cell on the child-7 path (:1788-1814) and, from every cell it
// reaches, marks each neighbour outside and continues through the empty ones
// (:1822-1843); then non-empty children with any outside bit are marked
// bottom-up (:1846-1860).
struct FloodFill {
  ora_octree* o;
  std::vector<std::vector<uint32_t>> par;   // parent node of each node
  std::vector<std::vector<uint8_t>> slot;   // its child slot in the parent
  struct Cell {
    int level;       // depth (0 = the root itself)
    uint32_t pidx;   // node at level - 1
    int c;           // child slot
    bool valid;
  };
  static Cell null_cell() { return Cell{-1, 0, 0, false}; }
  // getChildIndexForDirection (:1690-1699): directions NX NY NZ PX PY PZ
  static int dir_child(int dir, int i) {
    int c = i;
    if (dir % 3 == 1) c = i + 2 * (i / 2);
    else if (dir % 3 == 2) c = i * 2;
    if (dir == 3) c += 4;
    else if (dir == 4) c += 2;
    else if (dir == 5) c += 1;
    return c;
  }
  const Node& node_of(const Cell& t) const {  // getNode (:1678-1683)
    if (t.level == 0) return o->d[0][0];
    return o->d[t.level][o->d[t.level - 1][t.pidx].ch[t.c]];
  }
  uint32_t node_id(const Cell& t) const { return t.level == 0 ? 0 : o->d[t.level - 1][t.pidx].ch[t.c]; }
  bool is_leaf(const Cell& t) const {  // isLeaf (:1686-1692)
    if (uint32_t(t.level) == o->levels) return true;
    const Node& p = o->d[t.level - 1][t.pidx];
    if (p.has_ptr(t.c)) return node_of(t).mask == 0;
    return true;
  }
  Cell parent(const Cell& t) const {
    if (t.level <= 1) return Cell{0, 0, 0, true};
    return Cell{t.level - 1, par[t.level - 1][t.pidx], slot[t.level - 1][t.pidx], true};
  }
  Cell neighbour_ge(const Cell& t, int dir) const {  // getNeighbourGrtrEqSz
    if (t.level == 0) return null_cell();
    const int opp = (dir + 3) % 6;
    for (int i = 0; i < 4; ++i)
      if (t.c == dir_child(opp, i)) return Cell{t.level, t.pidx, dir_child(dir, i), true};
    const Cell pn = neighbour_ge(parent(t), dir);
    if (!pn.valid || is_leaf(pn)) return pn;
    const uint32_t pid = node_id(pn);
    for (int i = 0; i < 4; ++i)
      if (t.c == dir_child(dir, i)) return Cell{pn.level + 1, pid, dir_child(opp, i), true};
    return null_cell();
  }
  void neighbours_small(const Cell& nb, int dir, std::vector<Cell>& out) const {  // getNeighboursSmSz
    std::vector<Cell> st;
    if (nb.valid) st.push_back(nb);
    const int opp = (dir + 3) % 6;
    while (!st.empty()) {
      const Cell can = st.back();
      st.pop_back();
      if (is_leaf(can)) {
        out.push_back(can);
      } else {
        const uint32_t id = node_id(can);
        for (int i = 0; i < 4; ++i) st.push_back(Cell{can.level + 1, id, dir_child(opp, i), true});
      }
    }
  }
  bool bit(const Cell& t) const { return (o->outside[t.level - 1][t.pidx] >> t.c) & 1u; }
  void set_bit(const Cell& t) { o->outside[t.level - 1][t.pidx] |= uint8_t(1u << t.c); }

  int run(uint64_t* n_empty, uint64_t* n_surface) {
    const uint32_t L = o->levels;
    par.assign(L, {});
    slot.assign(L, {});
    o->outside.assign(L, {});
    for (uint32_t l = 0; l < L; ++l) {
      par[l].assign(o->d[l].size(), 0);
      slot[l].assign(o->d[l].size(), 0);
      o->outside[l].assign(o->d[l].size(), 0);
    }
    for (uint32_t l = 0; l + 1 < L; ++l)
      for (uint32_t i = 0; i < o->d[l].size(); ++i)
        for (int c = 0; c < 8; ++c)
          if (o->d[l][i].has_ptr(c)) {
            par[l + 1][o->d[l][i].ch[c]] = i;
            slot[l + 1][o->d[l][i].ch[c]] = uint8_t(c);
          }
    // the start cell: slot 7 of the deepest node on the child-7 path
    Cell start{1, 0, 7, true};
    uint32_t cur = 0;
    for (uint32_t lev = 0; lev < L; ++lev) {
      start = Cell{int(lev) + 1, cur, 7, true};
      if (!o->d[lev][cur].has_ptr(7)) break;
      cur = o->d[lev][cur].ch[7];
    }
    if (o->d[start.level - 1][start.pidx].has_child(7)) return -3;  // the reference aborts here
    std::vector<Cell> stack{start};
    set_bit(start);
    uint64_t empty = 1, surface = 0;
    std::vector<Cell> nbs;
    while (!stack.empty()) {
      const Cell t = stack.back();
      stack.pop_back();
      nbs.clear();
      for (int dir = 0; dir < 6; ++dir) neighbours_small(neighbour_ge(t, dir), dir, nbs);
      for (const Cell& nb : nbs) {
        if (bit(nb)) continue;
        set_bit(nb);
        if (!o->d[nb.level - 1][nb.pidx].has_child(nb.c)) {
          stack.push_back(nb);
          ++empty;
        } else {
          ++surface;
        }
      }
    }
    for (int lev = int(L) - 2; lev >= 0; --lev)
      for (uint32_t i = 0; i < o->d[lev].size(); ++i)
        for (int c = 0; c < 8; ++c)
          if (o->d[lev][i].has_ptr(c) && o->outside[lev + 1][o->d[lev][i].ch[c]] != 0)
            o->outside[lev][i] |= uint8_t(1u << c);
    if (n_empty) *n_empty = empty;
    if (n_surface) *n_surface = surface;
    return 0;
  }
};

}  // namespace

extern "C" {

int ora_flood_fill(ora_octree* o, uint64_t* n_empty, uint64_t* n_surface) {
  if (!o || o->state != 1 || o->levels < 1) return -1;
  FloodFill f{o, {}, {}};
  return f.run(n_empty, n_surface);
}

int ora_get_outside(const ora_octree* o, uint32_t level, uint8_t* out) {
  if (!o || level >= o->outside.size()) return -1;
  std::memcpy(out, o->outside[level].data(), o->outside[level].size());
  return 0;
}

ora_octree* ora_create(void) { return new ora_octree(); }
void ora_destroy(ora_octree* o) { delete o; }
ora_octree* ora_clone(const ora_octree* o) { return new ora_octree(*o); }

int ora_build_svo(ora_octree* o, const float* tris, uint64_t n_tris, const double bbox[6], uint32_t levels) {
  if (!o || levels < 1 || levels > 31) return -1;
  build_svo(o, tris, n_tris, bbox, levels);
  o->st.levels = levels;
  return 0;
}

int ora_build_dag_chunked(ora_octree* o, const float* tris, uint64_t n_tris, const double bbox[6], uint32_t levels,
                          uint32_t step_level, int n_threads) {
  if (!o || step_level == 0 || step_level + 1 >= levels) return -1;
  build_dag_chunked(o, tris, n_tris, bbox, levels, step_level, n_threads);
  o->st.levels = levels;
  return 0;
}

// Voxel-brick ingest.  The reference has no voxel-grid input; a grid enters
// it as node data through GeomOctree(const NodeData&, bbox, rootSide, levels,
// stats) (src/symvox/geom_octree.cpp:49-60), which stores the pools and sets
// the DAG state.  The pools restated here: bricks[8^(depth-1)] are 2^3 voxel
// masks (bit 4x+2y+z) in Morton order (x the most significant bit of each
// coordinate triple); level depth-1 holds the non-empty bricks in that order,
// and each level above the non-empty cells of 8 consecutive entries of the
// level below (child k = entry 8j+k), in Morton order; the root always exists.
int ora_build_from_bricks(ora_octree* o, uint32_t depth, const uint8_t* bricks) {
  if (!o || depth < 1 || depth > 11 || !bricks) return -1;
  o->levels = depth;
  o->d.assign(depth, std::vector<Node>());
  uint64_t cells = 1ull << (3 * (depth - 1));
  std::vector<uint32_t> idx(cells, kNull), up;
  o->n_voxels = 0;
  for (uint64_t i = 0; i < cells; ++i) {
    if (!bricks[i]) continue;
    Node n;
    n.mask = bricks[i];
    idx[i] = uint32_t(o->d[depth - 1].size());
    o->d[depth - 1].push_back(n);
    o->n_voxels += popc8(n.mask);
  }
  for (int l = int(depth) - 2; l >= 0; --l) {
    cells >>= 3;
    up.assign(cells, kNull);
    for (uint64_t j = 0; j < cells; ++j) {
      Node n;
      for (int k = 0; k < 8; ++k) {
        const uint32_t c = idx[8 * j + k];
        if (c == kNull) continue;
        n.mask |= uint8_t(1u << k);
        n.ch[k] = c;
      }
      if (!n.mask && l > 0) continue;
      up[j] = uint32_t(o->d[l].size());
      o->d[l].push_back(n);
    }
    idx.swap(up);
  }
  if (depth == 1 && o->d[0].empty()) o->d[0].push_back(Node());
  o->n_nodes = 0;
  for (const auto& L : o->d) o->n_nodes += L.size();
  o->state = 2;
  o->st = ora_stats{};
  o->st.levels = depth;
  o->st.n_total_voxels = o->n_voxels;
  o->st.n_nodes_dag = o->n_nodes;
  return 0;
}

// Lossy LSVDAG, the exact-proposer form of the GPU path (its definition is
// project-defined: the reference's toLossyDag, geom_octree_extension.cpp:
// 797-1179, needs the external MCL binary).  Levels L-1-max_above ..
// L-1-min_above top-down; candidates = reachable, not frozen; leaf bytes of
// each candidate's subtree in Morton order; an edge (a < b) when the XOR
// popcount is <= floor(max_err * 8^(L-lev)); leader rule in candidate
// order; parents redirected to leaders; leaders' subtrees frozen; finally
// unreachable nodes dropped and toDAG.
namespace {
void subtree_bytes(const ora_octree* o, uint32_t lev, uint32_t node, uint32_t k, uint64_t base, uint8_t* out) {
  if (k == 0) {
    out[base] = o->d[lev][node].mask;
    return;
  }
  const Node& n = o->d[lev][node];
  for (int d = 0; d < 8; ++d)
    if (n.has_child(d)) subtree_bytes(o, lev + 1, n.ch[d], k - 1, (base << 3) | uint64_t(d), out);
}
std::vector<std::vector<char>> reachable(const ora_octree* o) {
  std::vector<std::vector<char>> r(o->levels);
  for (uint32_t l = 0; l < o->levels; ++l) r[l].assign(o->d[l].size(), 0);
  if (!o->d[0].empty()) r[0][0] = 1;
  for (uint32_t l = 0; l + 1 < o->levels; ++l)
    for (size_t i = 0; i < o->d[l].size(); ++i)
      if (r[l][i])
        for (int c = 0; c < 8; ++c)
          if (o->d[l][i].has_child(c)) r[l + 1][o->d[l][i].ch[c]] = 1;
  return r;
}
}  // namespace

int ora_lossy_exact(ora_octree* o, uint32_t min_above, uint32_t max_above, double max_err, uint64_t* merged) {
  if (!o || o->state != 2 || min_above > max_above) return -1;
  const uint32_t L = o->levels;
  std::vector<std::vector<char>> frozen(L);
  for (uint32_t l = 0; l < L; ++l) frozen[l].assign(o->d[l].size(), 0);
  uint64_t nmerged = 0;
  for (uint32_t a = max_above + 1; a-- > min_above;) {
    if (a + 1 >= L) continue;
    const uint32_t lev = L - 1 - a;
    auto reach = reachable(o);
    std::vector<uint32_t> cand;
    for (uint32_t i = 0; i < o->d[lev].size(); ++i)
      if (reach[lev][i] && !frozen[lev][i]) cand.push_back(i);
    const uint32_t n = uint32_t(cand.size());
    if (n < 2) continue;
    const uint32_t k = L - 1 - lev;
    const uint64_t per = 1ull << (3 * k);
    std::vector<uint8_t> bytes(per * n, 0);
    std::vector<uint32_t> pop(n, 0);
    for (uint32_t c = 0; c < n; ++c) {
      const Node& nd = o->d[lev][cand[c]];
      uint8_t* out = bytes.data() + per * c;
      for (int d = 0; d < 8; ++d)
        if (nd.has_child(d)) subtree_bytes(o, lev + 1, nd.ch[d], k - 1, uint64_t(d), out);
      for (uint64_t s = 0; s < per; ++s) pop[c] += popc8(out[s]);
    }
    const uint32_t lim = uint32_t(max_err * double(1ull << (3 * (L - lev))));
    std::vector<std::vector<uint32_t>> below(n);
    for (uint32_t b = 0; b < n; ++b)
      for (uint32_t a2 = 0; a2 < b; ++a2) {
        const uint32_t gap = pop[a2] > pop[b] ? pop[a2] - pop[b] : pop[b] - pop[a2];
        if (gap > lim) continue;
        uint32_t dist = 0;
        const uint8_t* x = bytes.data() + per * a2;
        const uint8_t* y = bytes.data() + per * b;
        for (uint64_t s = 0; s < per && dist <= lim; ++s) dist += popc8(uint8_t(x[s] ^ y[s]));
        if (dist <= lim) below[b].push_back(a2);
      }
    const uint32_t kLeadO = 0xFFFFFFFEu;
    std::vector<uint32_t> state(n, 0xFFFFFFFFu);
    for (uint32_t i = 0; i < n; ++i) {
      uint32_t r = kLeadO;
      for (uint32_t j : below[i])
        if (state[j] == kLeadO) { r = j; break; }
      state[i] = r;
    }
    std::vector<uint32_t> node_to(o->d[lev].size(), 0xFFFFFFFFu);
    std::vector<char> lead(o->d[lev].size(), 0);
    for (uint32_t i = 0; i < n; ++i) {
      if (state[i] == kLeadO) lead[cand[i]] = 1;
      else { node_to[cand[i]] = cand[state[i]]; ++nmerged; }
    }
    for (auto& p : o->d[lev - 1])
      for (int c = 0; c < 8; ++c)
        if (p.has_child(c) && node_to[p.ch[c]] != 0xFFFFFFFFu) p.ch[c] = node_to[p.ch[c]];
    for (size_t i = 0; i < o->d[lev].size(); ++i)
      if (lead[i])
        for (int c = 0; c < 8; ++c)
          if (o->d[lev][i].has_child(c)) frozen[lev + 1][o->d[lev][i].ch[c]] = 1;
    for (uint32_t l = lev + 1; l + 1 < L; ++l)
      for (size_t i = 0; i < o->d[l].size(); ++i)
        if (frozen[l][i])
          for (int c = 0; c < 8; ++c)
            if (o->d[l][i].has_child(c)) frozen[l + 1][o->d[l][i].ch[c]] = 1;
  }
  // drop unreachable nodes, renumber
  auto reach = reachable(o);
  std::vector<std::vector<uint32_t>> nid(L);
  for (uint32_t l = 0; l < L; ++l) {
    nid[l].assign(o->d[l].size(), 0xFFFFFFFFu);
    uint32_t c = 0;
    for (size_t i = 0; i < o->d[l].size(); ++i)
      if (reach[l][i]) nid[l][i] = c++;
  }
  for (uint32_t l = 0; l < L; ++l) {
    std::vector<Node> keep;
    for (size_t i = 0; i < o->d[l].size(); ++i) {
      if (!reach[l][i]) continue;
      Node nd = o->d[l][i];
      for (int c = 0; c < 8; ++c) {
        if (l + 1 < L && nd.has_child(c)) nd.ch[c] = nid[l + 1][nd.ch[c]];
        else nd.ch[c] = kNull;
        nd.clev[c] = 0xFFFFFFFFu;
      }
      nd.inv = 0;
      keep.push_back(nd);
    }
    o->d[l].swap(keep);
  }
  o->state = 2;
  to_dag(o);
  if (merged) *merged = nmerged;
  return 0;
}

// The per-level node order of EncodedSSVDAG::encode
// (src/symvox/encoded_ssvdag.cpp:259-276): (index, count) pairs in index
// order, sorted by libstdc++'s std::sort with the reference's comparator.
int ora_refcount_order(const uint32_t* counts, uint64_t n, uint32_t* order) {
  std::vector<std::pair<uint32_t, uint32_t>> hist(n);
  for (uint64_t i = 0; i < n; ++i) hist[i] = std::make_pair(uint32_t(i), counts[i]);
  std::sort(hist.begin(), hist.end(),
            [](std::pair<uint32_t, uint32_t> a, std::pair<uint32_t, uint32_t> b) { return a.second > b.second; });
  for (uint64_t k = 0; k < n; ++k) order[k] = hist[k].first;
  return 0;
}

// EncodedSSVDAG::traverse (src/symvox/encoded_ssvdag.cpp:527-574) with
// getChild / getChildMask (:587-625) and getHalfSide (encoded_octree.hpp:68):
// the depth a point query reaches in an encoded SSVDAG (levels = voxel set).
// The leaf bricks are read in the encoder's default voxel-matrix order
// (:32, 317-345, xyz_to_byte_voxel :119-135), not as traverse() reads them
// (one byte per 2^3 sub-brick, the layout of the non-default mode).
// A pointer that leads outside the arrays ends that query with depth -2 and
// makes the call return -2.
int ora_ssvdag_traverse(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                        const uint32_t* level_off, uint32_t n_level_off, uint32_t levels, const float bbox[6],
                        float root_side, const float* pts, uint64_t n, int32_t* out) {
  if (levels < 3) return -1;
  int status = 0;
  auto code = [&](const uint16_t* nd, int c) { return (nd[0] >> (2 * c)) & 3u; };
  for (uint64_t q = 0; q < n; ++q) {
    float p[3] = {pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]};
    bool inside = true;
    for (int k = 0; k < 3; ++k) inside = inside && !(p[k] < bbox[k] || p[k] > bbox[3 + k]);
    if (!inside) { out[q] = -1; continue; }
    uint64_t idx = 0;
    uint32_t lev = 0;
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = (bbox[k] + bbox[3 + k]) * 0.5f;
    bool mx = false, my = false, mz = false;
    bool broken = false;
    while (lev < levels) {
      if (idx >= n_inner) { broken = true; break; }
      const uint16_t* nd = inner + idx;
      if (mx) p[0] = 2.f * c[0] - p[0];
      if (my) p[1] = 2.f * c[1] - p[1];
      if (mz) p[2] = 2.f * c[2] - p[2];
      int sel = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
      if (code(nd, sel) == 0) break;
      ++lev;
      float hs = root_side / float(1u << (lev + 1));
      for (int k = 0; k < 3; ++k) c[k] += (p[k] > c[k]) ? hs : -1.f * hs;
      uint64_t off = 1;
      for (int i = 7; i > sel; --i) off += code(nd, i) == 0 ? 0 : (code(nd, i) == 1 ? 1 : 2);
      const uint32_t cc = code(nd, sel);
      if (idx + off + (cc >= 2 ? 2 : 1) > n_inner) { broken = true; break; }
      uint32_t ch;
      if (cc == 1) {
        ch = nd[off];
        mx = (ch >> 13) & 1u; my = (ch >> 14) & 1u; mz = (ch >> 15) & 1u;
        ch &= ~(7u << 13);
      } else {
        // the high half is written first (encoded_ssvdag.cpp:395-403)
        ch = (uint32_t(nd[off]) << 16) | uint32_t(nd[off + 1]);
        mx = (ch >> 29) & 1u; my = (ch >> 30) & 1u; mz = (ch >> 31) & 1u;
        ch &= ~(7u << 29);
        ch |= (cc & 1u) << 29;
      }
      if (lev < levels - 2) {
        if (lev >= n_level_off) { broken = true; break; }
        idx = uint64_t(level_off[lev]) + ch;
      } else if (lev == levels - 2) {
        const uint64_t leaf = uint64_t(ch) * 8;
        if (leaf + 8 > n_leaves) { broken = true; break; }
        if (mx) p[0] = 2.f * c[0] - p[0];
        if (my) p[1] = 2.f * c[1] - p[1];
        if (mz) p[2] = 2.f * c[2] - p[2];
        sel = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
        // the 2^3 sub-brick `sel` is empty when its 8 voxel bits are
        uint32_t any = 0;
        for (int v = 0; v < 8; ++v) {
          const int b = (2 * (sel & 1) + (v & 1)) + 4 * (2 * ((sel >> 1) & 1) + ((v >> 1) & 1)) +
                        16 * (2 * ((sel >> 2) & 1) + ((v >> 2) & 1));
          any |= (leaves[leaf + b / 8] >> (b % 8)) & 1u;
        }
        if (!any) break;
        ++lev;
        hs = root_side / float(1u << (lev + 1));
        for (int k = 0; k < 3; ++k) c[k] += (p[k] > c[k]) ? hs : -1.f * hs;
        const int vox = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
        // the brick's bits in the encoder's default voxel-matrix order
        // (encoded_ssvdag.cpp:32, 317-345, xyz_to_byte_voxel :119-135):
        // local (x, y, z) in [0, 4)^3 at bit z + 4y + 16x
        const int bi = 2 * ((sel >> 2) & 1) + ((vox >> 2) & 1), bj = 2 * ((sel >> 1) & 1) + ((vox >> 1) & 1),
                  bk = 2 * (sel & 1) + (vox & 1);
        const int bit = bk + 4 * bj + 16 * bi;
        if ((leaves[leaf + bit / 8] >> (bit % 8)) & 1u) ++lev;
        break;
      }
    }
    if (broken) status = -2;
    out[q] = broken ? -2 : int32_t(lev);
  }
  return status;
}

int ora_to_dag(ora_octree* o) { return o ? to_dag(o) : -1; }
int ora_to_sdag(ora_octree* o) { return o ? to_sdag(o) : -1; }
int ora_to_sdag_ex(ora_octree* o, int skip_symmetry) { return o ? to_sdag(o, skip_symmetry != 0) : -1; }
int ora_init_child_levels(ora_octree* o) {
  if (!o) return -1;
  init_child_levels(o);
  return 0;
}
int ora_merge_across_levels(ora_octree* o) {
  if (!o || o->state != 2) return -1;
  uint64_t miss = 0;
  int r = merge_across_levels(o, &miss);
  o->st.n_missing_correspondences = miss;
  return r;
}

uint64_t ora_level_count(const ora_octree* o, uint32_t level) {
  return (o && level < o->d.size()) ? o->d[level].size() : 0;
}

int ora_get_level(const ora_octree* o, uint32_t level, uint8_t* rec) {
  if (!o || level >= o->d.size()) return -1;
  for (size_t i = 0; i < o->d[level].size(); ++i) {
    const Node& n = o->d[level][i];
    uint8_t* r = rec + 48 * i;
    uint32_t hdr = uint32_t(n.mask) | (uint32_t(n.mir[0]) << 8) | (uint32_t(n.mir[1]) << 16) | (uint32_t(n.mir[2]) << 24);
    std::memcpy(r, &hdr, 4);
    std::memcpy(r + 4, n.ch, 32);
    for (int c = 0; c < 8; ++c) r[36 + c] = uint8_t(n.clev[c] & 0xFFu);
    r[44] = n.inv;
    r[45] = r[46] = r[47] = 0;
  }
  return 0;
}

int ora_get_stats(const ora_octree* o, ora_stats* s) {
  if (!o || !s) return -1;
  *s = o->st;
  s->n_nodes = o->n_nodes;
  s->levels = o->levels;
  s->state = uint32_t(o->state);
  return 0;
}

int ora_tri_box(const double center[3], double half_side, const float tri[9]) {
  return tri_box(center, half_side, tri) ? 1 : 0;
}

}  // extern "C"
