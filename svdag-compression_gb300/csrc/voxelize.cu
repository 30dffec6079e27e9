// GeomOctree::buildSVO on the GPU (src/symvox/geom_octree.cpp:171-280).
//
// The reference voxelizes triangle by triangle with a DFS stack: popping a
// node tests its 8 children (7..0) against the triangle with an fp64 SAT,
// sets the hit bits, creates missing child nodes in that order and pushes
// them, so children are visited 0 first.  Node ids per level are creation
// order.
//
// Here the same set of (triangle, node) visits is produced level by level:
// the frontier F_l holds every pair (t, n) such that triangle t's DFS visits
// node n at level l, sorted by (t, path order of n).  A node at level l+1 is
// created by the first pair (lowest frontier index q) that hits it, and
// among children created by the same pair the order is child 7..0; its id is
// therefore the rank of the key  q*8 + (7 - child)  among all created
// children, computed with a bitmap + popcount scan instead of a sort.  The
// next frontier is written in (q, child ascending) order, which keeps it
// sorted by (t, path order).  cleanEmptyNodes (geom_octree.cpp:437-456) then
// runs bottom-up.
//
// The SAT (src/symvox/test_triangle_box.cpp:38-184) is evaluated with
// explicitly rounded fp64 intrinsics in the reference's operation order so
// no contraction into FMA can change a decision.
#include "ctx.cuh"

namespace svdag {
namespace {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// AXISTEST_* (test_triangle_box.cpp:59-102): reject when the projected
// interval misses [-rad, rad]; b_first selects the Z12 ordering (p2 < p1).
__device__ __forceinline__ bool axis_reject(double pa, double pb, double fa, double fb, double h, bool b_first) {
  double mn, mx;
  if (b_first) {
    if (pb < pa) { mn = pb; mx = pa; } else { mn = pa; mx = pb; }
  } else {
    if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; }
  }
  double rad = dmul(dadd(fa, fb), h);
  return (mn > rad || mx < -rad);
}

// p = a*u - b*w  (X and Z macros)
__device__ __forceinline__ double amb(double a, double u, double b, double w) { return dsub(dmul(a, u), dmul(b, w)); }
// p = -a*u + b*w (Y macros)
__device__ __forceinline__ double nab(double a, double u, double b, double w) { return dadd(dmul(-a, u), dmul(b, w)); }

// testTriBox (test_triangle_box.cpp:105-184)
__device__ bool tri_box(double cx, double cy, double cz, double h, const float t[9]) {
  const double v0x = dsub(double(t[0]), cx), v0y = dsub(double(t[1]), cy), v0z = dsub(double(t[2]), cz);
  const double v1x = dsub(double(t[3]), cx), v1y = dsub(double(t[4]), cy), v1z = dsub(double(t[5]), cz);
  const double v2x = dsub(double(t[6]), cx), v2y = dsub(double(t[7]), cy), v2z = dsub(double(t[8]), cz);
  const double e0x = dsub(v1x, v0x), e0y = dsub(v1y, v0y), e0z = dsub(v1z, v0z);
  const double e1x = dsub(v2x, v1x), e1y = dsub(v2y, v1y), e1z = dsub(v2z, v1z);
  const double e2x = dsub(v0x, v2x), e2y = dsub(v0y, v2y), e2z = dsub(v0z, v2z);
  double fex, fey, fez;
  // edge 0: AXISTEST_X01, _Y02, _Z12
  fex = fabs(e0x); fey = fabs(e0y); fez = fabs(e0z);
  if (axis_reject(amb(e0z, v0y, e0y, v0z), amb(e0z, v2y, e0y, v2z), fez, fey, h, false)) return false;
  if (axis_reject(nab(e0z, v0x, e0x, v0z), nab(e0z, v2x, e0x, v2z), fez, fex, h, false)) return false;
  if (axis_reject(amb(e0y, v1x, e0x, v1y), amb(e0y, v2x, e0x, v2y), fey, fex, h, true)) return false;
  // edge 1: AXISTEST_X01, _Y02, _Z0
  fex = fabs(e1x); fey = fabs(e1y); fez = fabs(e1z);
  if (axis_reject(amb(e1z, v0y, e1y, v0z), amb(e1z, v2y, e1y, v2z), fez, fey, h, false)) return false;
  if (axis_reject(nab(e1z, v0x, e1x, v0z), nab(e1z, v2x, e1x, v2z), fez, fex, h, false)) return false;
  if (axis_reject(amb(e1y, v0x, e1x, v0y), amb(e1y, v1x, e1x, v1y), fey, fex, h, false)) return false;
  // edge 2: AXISTEST_X2, _Y1, _Z12
  fex = fabs(e2x); fey = fabs(e2y); fez = fabs(e2z);
  if (axis_reject(amb(e2z, v0y, e2y, v0z), amb(e2z, v1y, e2y, v1z), fez, fey, h, false)) return false;
  if (axis_reject(nab(e2z, v0x, e2x, v0z), nab(e2z, v1x, e2x, v1z), fez, fex, h, false)) return false;
  if (axis_reject(amb(e2y, v1x, e2x, v1y), amb(e2y, v2x, e2x, v2y), fey, fex, h, true)) return false;
  // FINDMINMAX per axis (test_triangle_box.cpp:165-174)
  {
    double mn = v0x, mx = v0x;
    if (v1x < mn) mn = v1x;
    if (v1x > mx) mx = v1x;
    if (v2x < mn) mn = v2x;
    if (v2x > mx) mx = v2x;
    if (mn > h || mx < -h) return false;
  }
  {
    double mn = v0y, mx = v0y;
    if (v1y < mn) mn = v1y;
    if (v1y > mx) mx = v1y;
    if (v2y < mn) mn = v2y;
    if (v2y > mx) mx = v2y;
    if (mn > h || mx < -h) return false;
  }
  {
    double mn = v0z, mx = v0z;
    if (v1z < mn) mn = v1z;
    if (v1z > mx) mx = v1z;
    if (v2z < mn) mn = v2z;
    if (v2z > mx) mx = v2z;
    if (mn > h || mx < -h) return false;
  }
  // normal = e0 x e1, planeBoxOverlap (test_triangle_box.cpp:38-56, 179-180)
  const double nx = dsub(dmul(e0y, e1z), dmul(e0z, e1y));
  const double ny = dsub(dmul(e0z, e1x), dmul(e0x, e1z));
  const double nz = dsub(dmul(e0x, e1y), dmul(e0y, e1x));
  double minx, maxx, miny, maxy, minz, maxz;
  if (nx > 0.0) { minx = dsub(-h, v0x); maxx = dsub(h, v0x); } else { minx = dsub(h, v0x); maxx = dsub(-h, v0x); }
  if (ny > 0.0) { miny = dsub(-h, v0y); maxy = dsub(h, v0y); } else { miny = dsub(h, v0y); maxy = dsub(-h, v0y); }
  if (nz > 0.0) { minz = dsub(-h, v0z); maxz = dsub(h, v0z); } else { minz = dsub(h, v0z); maxz = dsub(-h, v0z); }
  const double dmin = dadd(dadd(dmul(nx, minx), dmul(ny, miny)), dmul(nz, minz));
  if (dmin > 0.0) return false;
  const double dmax = dadd(dadd(dmul(nx, maxx), dmul(ny, maxy)), dmul(nz, maxz));
  return dmax >= 0.0;
}

struct VoxParams {
  double root_c[3];
  double root_side;
  uint32_t level;        // level of the frontier's nodes
  uint32_t leaf_level;   // levels - 1
};

// Node centre from its Morton path, accumulated level by level exactly as
// the DFS does (centre + (+-k) per level, geom_octree.cpp:222-230).
__device__ __forceinline__ void node_center(const VoxParams& P, uint64_t path, double c[3]) {
  c[0] = P.root_c[0]; c[1] = P.root_c[1]; c[2] = P.root_c[2];
  for (uint32_t d = 0; d < P.level; ++d) {
    const uint32_t dig = uint32_t(path >> (3 * (P.level - 1 - d))) & 7u;
    const double k = __ddiv_rn(P.root_side, double(1u << (d + 2)));
    c[0] = dadd(c[0], (dig & 4) ? k : -k);
    c[1] = dadd(c[1], (dig & 2) ? k : -k);
    c[2] = dadd(c[2], (dig & 1) ? k : -k);
  }
}

// One thread per frontier pair: SAT against the node's 8 children.
__global__ void __launch_bounds__(256) k_expand(VoxParams P, const float* __restrict__ tris,
                                                const uint32_t* __restrict__ f_tri, const uint32_t* __restrict__ f_node,
                                                uint64_t F, const uint64_t* __restrict__ path,
                                                uint32_t* __restrict__ hdr, uint32_t* __restrict__ firstq,
                                                uint8_t* __restrict__ hits_out) {
  const double k = __ddiv_rn(P.root_side, double(1u << (P.level + 2)));  // getHalfSideD(level+1)
  const bool leaf = (P.level == P.leaf_level);
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < F; q += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = f_tri ? f_tri[q] : uint32_t(q);
    const uint32_t node = f_node ? f_node[q] : 0u;
    float tri[9];
    const float* tp = tris + 9ull * t;
#pragma unroll
    for (int j = 0; j < 9; ++j) tri[j] = tp[j];
    double c[3];
    node_center(P, path[node], c);
    uint32_t h = 0;
#pragma unroll 1
    for (int i = 7; i >= 0; --i) {
      const double cx = dadd(c[0], (i & 4) ? k : -k);
      const double cy = dadd(c[1], (i & 2) ? k : -k);
      const double cz = dadd(c[2], (i & 1) ? k : -k);
      if (tri_box(cx, cy, cz, k, tri)) h |= 1u << i;
    }
    if (h) atomicOr(&hdr[node], h);
    if (!leaf) {
      hits_out[q] = uint8_t(h);
      for (uint32_t m = h; m; m &= m - 1) {
        const int i = __ffs(m) - 1;
        atomicMin(&firstq[8ull * node + i], uint32_t(q));
      }
    }
  }
}

// Creation key of each created child: firstq * 8 + (7 - child).
__global__ void k_mark_keys(const uint32_t* __restrict__ firstq, uint64_t slots, uint32_t* __restrict__ bitmap) {
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < slots; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t fq = firstq[s];
    if (fq == kNone) continue;
    const uint64_t key = uint64_t(fq) * 8 + (7 - (s & 7));
    atomicOr(&bitmap[key >> 5], 1u << (key & 31));
  }
}

struct PopcIn {
  const uint32_t* w;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return __popc(w[i]); }
};
struct PopcU8In {
  const uint8_t* w;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const { return __popc(uint32_t(w[i])); }
};
struct U32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};
struct U64to32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint64_t v) const { a[i] = uint32_t(v); }
};

// Child ids = rank of the creation key; also the children's Morton paths.
__global__ void k_assign_children(const uint32_t* __restrict__ firstq, uint64_t slots, const uint32_t* __restrict__ bitmap,
                                  const uint32_t* __restrict__ woff, const uint64_t* __restrict__ path,
                                  uint32_t* __restrict__ ch, uint64_t* __restrict__ child_path) {
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < slots; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t fq = firstq[s];
    if (fq == kNone) { ch[s] = kNull; continue; }
    const uint64_t key = uint64_t(fq) * 8 + (7 - (s & 7));
    const uint32_t w = bitmap[key >> 5];
    const uint32_t rank = woff[key >> 5] + __popc(w & ((1u << (key & 31)) - 1u));
    ch[s] = rank;
    child_path[rank] = (path[s >> 3] << 3) | (s & 7);
  }
}

// Next frontier in (pair, child ascending) order.
__global__ void k_emit_frontier(const uint32_t* __restrict__ f_tri, const uint32_t* __restrict__ f_node, uint64_t F,
                                const uint8_t* __restrict__ hits, const uint32_t* __restrict__ off,
                                const uint32_t* __restrict__ ch, uint32_t* __restrict__ nf_tri, uint32_t* __restrict__ nf_node) {
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < F; q += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t h = hits[q];
    if (!h) continue;
    const uint32_t t = f_tri ? f_tri[q] : uint32_t(q);
    const uint32_t node = f_node ? f_node[q] : 0u;
    uint32_t o = off[q];
    for (; h; h &= h - 1) {
      const int i = __ffs(h) - 1;
      nf_tri[o] = t;
      nf_node[o] = ch[8ull * node + i];
      ++o;
    }
  }
}

// cleanEmptyNodes step for one level: parents at level lev-1 drop children
// whose mask at level lev is zero.
__global__ void k_clean_empty(uint32_t* __restrict__ phdr, uint32_t* __restrict__ pch, uint64_t np,
                              const uint32_t* __restrict__ chdr) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t c[8];
    load_children(pch, p, c);
    uint32_t clear = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (c[j] != kNull && (chdr[c[j]] & 0xFFu) == 0) { clear |= 1u << j; c[j] = kNull; }
    }
    if (clear) {
      phdr[p] &= ~clear;
      store_children(pch, p, c);
    }
  }
}

__global__ void k_count_voxels(const uint32_t* __restrict__ hdr, uint64_t n, unsigned long long* out) {
  uint64_t s = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    s += __popc(hdr[i] & 0xFFu);
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, (unsigned long long)s);
}

}  // namespace

void phase_voxelize(Ctx& c, uint32_t levels, const double bb[6]) {
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  if (!c.tris && c.n_tris) throw Error(SVDAG_ERR_INVALID_STATE, "voxelize: no triangles set");
  if (levels < 1 || levels > 21) throw Error(SVDAG_ERR_INVALID_ARG, "voxelize: levels must be in [1, 21]");
  if (c.n_tris >= (1ull << 32) - 1) throw Error(SVDAG_ERR_OVERFLOW, "voxelize: more than 2^32-2 triangles");

  // Octree bbox / root side as resizeSceneBbox (octree.hpp:101-105): float box,
  // root side = largest float side; root centre = bbox.center() in double.
  for (int k = 0; k < 6; ++k) c.bbox[k] = float(bb[k]);
  float s3[3];
  for (int k = 0; k < 3; ++k) s3[k] = ((c.bbox[3 + k] - c.bbox[k]) * 0.5f) * 2.0f;
  float rs = s3[0] > s3[1] ? s3[0] : s3[1];
  rs = rs > s3[2] ? rs : s3[2];
  c.root_side = double(rs);

  VoxParams P;
  for (int k = 0; k < 3; ++k) P.root_c[k] = (bb[k] + bb[3 + k]) * 0.5;
  P.root_side = c.root_side;
  P.leaf_level = levels - 1;

  c.levels = levels;
  c.lev.clear();
  c.lev.resize(levels);
  c.child_levels_init = false;

  // level 0: the root
  c.lev[0].n = 1;
  c.lev[0].hdr.alloc(1, st);
  c.lev[0].path.alloc(1, st);
  SVDAG_CUDA(cudaMemsetAsync(c.lev[0].hdr.get(), 0, 4, st));
  SVDAG_CUDA(cudaMemsetAsync(c.lev[0].path.get(), 0, 8, st));

  DBuf<uint32_t> f_tri, f_node;  // frontier; empty at level 0 (implicit (t, root))
  uint64_t F = c.n_tris;
  DBuf<uint64_t> d_total(1, st);
  DBuf<unsigned long long> d_vox(1, st);

  for (uint32_t l = 0; l < levels; ++l) {
    Level& L = c.lev[l];
    P.level = l;
    const bool leaf = (l == levels - 1);
    DBuf<uint32_t> firstq;
    DBuf<uint8_t> hits;
    if (!leaf) {
      firstq.alloc(8 * L.n, st);
      fill<uint32_t>(ex, firstq.get(), 8 * L.n, kNone);
      hits.alloc(F, st);
    }
    if (F)
      SVDAG_LAUNCH(ex, k_expand, grid_for(ex, F, 256, 32), 256, 0, P, c.tris, f_tri.get(), f_node.get(), F,
                   L.path.get(), L.hdr.get(), firstq.get(), hits.get());
    if (leaf) break;

    // --- create level l+1 in reference creation order
    const uint64_t slots = 8 * L.n;
    const uint64_t words = (8 * F + 31) / 32;
    DBuf<uint32_t> bitmap(words ? words : 1, st), woff(words ? words : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(bitmap.get(), 0, 4 * (words ? words : 1), st));
    SVDAG_LAUNCH(ex, k_mark_keys, grid_for(ex, slots, 256), 256, 0, firstq.get(), slots, bitmap.get());
    DBuf<uint32_t> d_n32(1, st);
    device_exclusive_scan<uint32_t>(ex, PopcIn{bitmap.get()}, words, U32Out{woff.get()}, d_n32.get());
    const uint64_t n_next = read_scalar(ex, d_n32.get());
    Level& N = c.lev[l + 1];
    N.n = n_next;
    L.ch.alloc(slots, st);
    N.hdr.alloc(n_next ? n_next : 1, st);
    N.path.alloc(n_next ? n_next : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(N.hdr.get(), 0, 4 * (n_next ? n_next : 1), st));
    SVDAG_LAUNCH(ex, k_assign_children, grid_for(ex, slots, 256), 256, 0, firstq.get(), slots, bitmap.get(),
                 woff.get(), L.path.get(), L.ch.get(), N.path.get());
    firstq.release();
    bitmap.release();
    woff.release();

    // --- next frontier
    DBuf<uint32_t> off(F ? F : 1, st);
    device_exclusive_scan<uint64_t>(ex, PopcU8In{hits.get()}, F, U64to32Out{off.get()}, d_total.get());
    const uint64_t F_next = read_scalar(ex, d_total.get());
    if (F_next >= (1ull << 32)) throw Error(SVDAG_ERR_OVERFLOW, "voxelize: frontier exceeds 2^32 pairs");
    DBuf<uint32_t> nf_tri(F_next ? F_next : 1, st), nf_node(F_next ? F_next : 1, st);
    if (F)
      SVDAG_LAUNCH(ex, k_emit_frontier, grid_for(ex, F, 256), 256, 0, f_tri.get(), f_node.get(), F, hits.get(),
                   off.get(), L.ch.get(), nf_tri.get(), nf_node.get());
    f_tri = std::move(nf_tri);
    f_node = std::move(nf_node);
    F = F_next;
  }
  f_tri.release();
  f_node.release();

  // cleanEmptyNodes, bottom-up with cascade
  for (uint32_t lev = levels - 1; lev > 0; --lev) {
    Level& P_ = c.lev[lev - 1];
    if (P_.n)
      SVDAG_LAUNCH(ex, k_clean_empty, grid_for(ex, P_.n, 256), 256, 0, P_.hdr.get(), P_.ch.get(), P_.n,
                   c.lev[lev].hdr.get());
  }
  for (auto& L : c.lev) L.path.release();

  SVDAG_CUDA(cudaMemsetAsync(d_vox.get(), 0, 8, st));
  const Level& LL = c.lev[levels - 1];
  if (LL.n) SVDAG_LAUNCH(ex, k_count_voxels, grid_for(ex, LL.n, 256), 256, 0, LL.hdr.get(), LL.n, d_vox.get());
  const uint64_t nvox = read_scalar(ex, d_vox.get());

  uint64_t nsvo = 0;
  for (uint32_t l = 1; l < levels; ++l) nsvo += c.lev[l].n;
  c.st.n_total_voxels = nvox;
  c.st.n_nodes_svo = nsvo;
  c.st.n_nodes_last_lev_svo = c.lev[levels - 1].n;
  c.st.n_nodes = nsvo;
  c.st.levels = levels;
  c.state = SVDAG_S_SVO;
}

}  // namespace svdag
