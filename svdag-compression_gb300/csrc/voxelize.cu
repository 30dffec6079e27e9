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
// The SAT (src/symvox/test_triangle_box.cpp:38-184) goes through the
// certified fp32 filter of sat.cuh, which falls back to the reference's exact
// fp64 operation order for every predicate it cannot decide, so each box
// decision equals the reference's.  Node centres are stored per node in fp64,
// each child's as parent centre + (+-k) exactly as the DFS computes it.
#include "ctx.cuh"
#include "sat.cuh"

namespace svdag {
namespace {

struct VoxParams {
  double root_c[3];
  double root_side;
  uint32_t level;        // level of the frontier's nodes
  uint32_t leaf_level;   // levels - 1
};

// Half side of the children of a level-l node: getHalfSideD(l+1)
// (src/symvox/octree.hpp:115) = rootSide / 2^(l+2), exact.
__host__ __device__ __forceinline__ double child_half_side(double root_side, uint32_t l) {
  return root_side / double(1ull << (l + 2));
}

// Expansion of one frontier tile per block, in two phases so the expensive
// box tests run with full warps:
//   1. one thread per pair loads the triangle and the node's child boxes,
//      classifies the triangle's extent against the 6 child slabs and decides
//      every child the slabs settle (certain miss / certain overlap);
//   2. the (pair, child) items left undecided are queued in shared memory and
//      the whole block works through the queue, one item per thread, with the
//      full certified test.
// Then each pair publishes its hit mask: OR into the node mask, first-pair
// index per created child, and the mask for the next frontier.
// 224 threads and 4 resident blocks per SM (28 warps, 73 registers) measured
// fastest among 128-256 threads x 2-6 blocks on the depth-12 terrain: the
// kernel is latency bound, and more warps in more blocks keep the SM issuing
// across the tile barriers despite a few spilled registers.
#ifndef SVDAG_EXPAND_THREADS
#define SVDAG_EXPAND_THREADS 224
#endif
constexpr int kExpandThreads = SVDAG_EXPAND_THREADS;

// A queued pair's edge and plane constants, read from the tile's shared
// memory at their use in the full test.
struct SmemPairSrc {
  const float (*st)[kExpandThreads];
  const float (*snb)[kExpandThreads];
  const float (*svm)[kExpandThreads];
  const float (*se)[kExpandThreads];
  const float (*spl)[kExpandThreads];
  uint32_t slot;
  __device__ __forceinline__ float t(int i) const { return st[i][slot]; }
  __device__ __forceinline__ float chi(int i) const { return snb[i][slot]; }
  __device__ __forceinline__ float clo() const { return snb[6][slot]; }
  __device__ __forceinline__ float vmax(int i) const { return svm[i][slot]; }
  __device__ __forceinline__ float e(int j, int q) const { return se[3 * j + q][slot]; }
  __device__ __forceinline__ float n(int q) const { return spl[q][slot]; }
  __device__ __forceinline__ float sn(int q) const { return spl[3 + q][slot]; }
  __device__ __forceinline__ float nh() const { return spl[6][slot]; }
};
static_assert(kExpandThreads % 32 == 0 && kExpandThreads <= 256, "tile: whole warps, static shared memory <= 48 KB");

#ifndef SVDAG_EXPAND_MIN_BLOCKS
#define SVDAG_EXPAND_MIN_BLOCKS 4
#endif
// one resident wave of blocks taking tiles from a counter (3% faster than a
// static grid-stride walk: the undecided-child queues vary per tile)
#ifndef SVDAG_EXPAND_GRID_PER_SM
#define SVDAG_EXPAND_GRID_PER_SM 4
#endif
#ifndef SVDAG_EXPAND_DYNAMIC
#define SVDAG_EXPAND_DYNAMIC 1
#endif
constexpr bool kExpandDynamic = SVDAG_EXPAND_DYNAMIC != 0;
__global__ void __launch_bounds__(kExpandThreads, SVDAG_EXPAND_MIN_BLOCKS) k_expand(VoxParams P, const float* __restrict__ tris,
                                                           const uint32_t* __restrict__ f_tri,
                                                           const uint32_t* __restrict__ f_node, uint64_t F,
                                                           const double* __restrict__ ctr, const float* __restrict__ nbox,
                                                           uint32_t* __restrict__ hdr, uint32_t* __restrict__ firstq,
                                                           uint8_t* __restrict__ hits_out,
                                                           uint32_t* __restrict__ tile_hits,
                                                           unsigned long long* __restrict__ n_fallback,
                                                           unsigned long long* __restrict__ tile_ctr) {
  __shared__ float s_t[9][kExpandThreads];
  __shared__ float s_nb[8][kExpandThreads];
  __shared__ float s_vmax[6][kExpandThreads];
  __shared__ float s_e[9][kExpandThreads];
  __shared__ float s_pl[7][kExpandThreads];  // plane normal, |m1|+|m2| per component, |n|_1 h
  __shared__ uint32_t s_tri[kExpandThreads], s_node[kExpandThreads], s_slab[kExpandThreads];
  __shared__ uint32_t s_hits[kExpandThreads];
  __shared__ uint16_t s_queue[8 * kExpandThreads];
  __shared__ uint32_t s_qn;
  __shared__ uint32_t s_wsum[kExpandThreads / 32];
  __shared__ uint64_t s_base;
  const double k = child_half_side(P.root_side, P.level);
  const float hf = float(k);
  const bool leaf = (P.level == P.leaf_level);
  const int tid = threadIdx.x;
  unsigned fb = 0;
  // tiles: a grid-stride walk, or (tile_ctr) taken one at a time from a
  // counter so that blocks finishing early take more.  Three barriers per
  // tile: after the classification, after the queue, and at the end (which
  // also publishes the next tile and the cleared queue count).
  uint64_t base = uint64_t(blockIdx.x) * kExpandThreads;
  if (tid == 0) {
    s_qn = 0;
    if (tile_ctr) s_base = atomicAdd(tile_ctr, 1ull) * kExpandThreads;
  }
  __syncthreads();
  if (tile_ctr) base = s_base;
  for (; base < F;) {
    const uint64_t q = base + tid;
    uint32_t hits = 0;
    if (q < F) {
      const uint32_t t = f_tri ? f_tri[q] : uint32_t(q);
      const uint32_t node = f_node ? f_node[q] : 0u;
      const float* tp = tris + 9ull * t;
      float tri[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) tri[j] = tp[j];
      sat::NodeBoxes nb;
      const float4* np = reinterpret_cast<const float4*>(nbox + 8ull * node);
      const float4 a = np[0], b = np[1];
      nb.chi[0] = a.x; nb.chi[1] = a.y; nb.chi[2] = a.z; nb.chi[3] = a.w;
      nb.chi[4] = b.x; nb.chi[5] = b.y; nb.clo = b.z; nb.ok = b.w;
      sat::Pair32 PP;
      sat::pair_core(tri, tp, ctr + 3ull * node, nb, k, PP);
      sat::pair_slab_classes(PP);
      uint32_t full;
      sat::child_masks(PP, hits, full);
      s_node[tid] = node;
      if (full) {
        sat::pair_tangency(PP);
        // this pair's undecided children in consecutive queue slots, and the
        // pair data the full test reads (pairs the slabs decide skip both)
        uint32_t slot = atomicAdd(&s_qn, uint32_t(__popc(full)));
        for (uint32_t m = full; m; m &= m - 1) s_queue[slot++] = uint16_t((tid << 3) | (__ffs(m) - 1));
        sat::pair_edges(PP);
#pragma unroll
        for (int j = 0; j < 9; ++j) s_e[j][tid] = PP.e[j / 3][j % 3];
#pragma unroll
        for (int j = 0; j < 9; ++j) s_t[j][tid] = tri[j];
#pragma unroll
        for (int j = 0; j < 6; ++j) { s_nb[j][tid] = nb.chi[j]; s_vmax[j][tid] = PP.vmax[j]; }
        s_nb[6][tid] = nb.clo;
        s_nb[7][tid] = nb.ok;
#pragma unroll
        for (int j = 0; j < 3; ++j) { s_pl[j][tid] = PP.n[j]; s_pl[3 + j][tid] = PP.sn[j]; }
        s_pl[6][tid] = PP.nh;
        s_tri[tid] = t;
        // slab classes, tangency, axis-aligned triangle, fp32 path
        s_slab[tid] = PP.slab | (PP.tang << 16) | (PP.flat << 24) | (PP.fast ? 0x80000000u : 0u);
      }
    }
    s_hits[tid] = hits;
    __syncthreads();
    const uint32_t nq = s_qn;
    for (uint32_t i = tid; i < nq; i += kExpandThreads) {
      const uint32_t item = s_queue[i];
      const uint32_t slot = item >> 3;
      const int ci = int(item & 7u);
      const uint32_t node = s_node[slot];
      const uint32_t word = s_slab[slot];
      // the scalars of the pair; triangle, boxes, edges and plane are read
      // from shared memory where the full test uses them
      sat::Pair32 PP;
      PP.h = hf;
      PP.fast = (word >> 31) != 0u;
      PP.slab = word & 0xFFFFu;
      PP.tang = (word >> 16) & 0x3Fu;
      PP.flat = (word >> 24) & 0x7u;
      PP.tp = tris + 9ull * s_tri[slot];
      PP.c = ctr + 3ull * node;
      PP.k = k;
      const SmemPairSrc src{s_t, s_nb, s_vmax, s_e, s_pl, slot};
      if (sat::child_full_src(PP, src, ci, &fb)) atomicOr(&s_hits[slot], 1u << ci);
    }
    __syncthreads();
    {
      // Publish per warp: lanes of the same node combine their hit masks and
      // first pair indices (pair index = q - lane + lane', increasing with the
      // lane), and one lane per node issues the atomics -- and only when the
      // value does not already hold the result (both updates are monotone).
      // On the upper levels thousands of pairs share a node, and unaggregated
      // same-address atomics serialise.
      const bool valid = q < F;
      const uint32_t h = valid ? s_hits[tid] : 0u;
      const uint32_t node = valid ? s_node[tid] : 0xFFFFFFFFu;
      const int lane = tid & 31;
      const unsigned grp = __match_any_sync(0xFFFFFFFFu, node);
      const bool lead = valid && lane == __ffs(int(grp)) - 1;
      uint32_t hg = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const unsigned b = __ballot_sync(0xFFFFFFFFu, (h >> i) & 1u) & grp;
        if (b) {
          hg |= 1u << i;
          if (lead && !leaf) {
            uint32_t* fq = &firstq[8ull * node + i];
            const uint32_t cand = uint32_t(q) - uint32_t(lane) + uint32_t(__ffs(int(b)) - 1);
            if (__ldcg(fq) > cand) atomicMin(fq, cand);
          }
        }
      }
      if (lead && hg && (__ldcg(&hdr[node]) & hg) != hg) atomicOr(&hdr[node], hg);
      if (!leaf) {
        if (valid) hits_out[q] = uint8_t(h);
        // next-frontier entries of this tile (its offset comes from a scan of these)
        const uint32_t wsum = __reduce_add_sync(0xFFFFFFFFu, uint32_t(__popc(h)));
        if (lane == 0) s_wsum[tid >> 5] = wsum;
      }
    }
    // every thread is past the queue (s_qn) and has published (s_wsum)
    if (tid == 0) {
      s_qn = 0;
      if (tile_ctr) s_base = atomicAdd(tile_ctr, 1ull) * kExpandThreads;
    }
    __syncthreads();
    if (!leaf && tid == 0) {
      // s_wsum is rewritten only after two more barriers this thread joins
      uint32_t t = 0;
#pragma unroll
      for (int w = 0; w < kExpandThreads / 32; ++w) t += s_wsum[w];
      tile_hits[base / kExpandThreads] = t;
    }
    base = tile_ctr ? s_base : base + uint64_t(gridDim.x) * kExpandThreads;
  }
  unsigned long long sum = fb;
  for (int o = 16; o; o >>= 1) sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(n_fallback, sum);
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
struct U32toU64In {
  const uint32_t* w;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const { return w[i]; }
};
struct U32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};
struct U64to32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint64_t v) const { a[i] = uint32_t(v); }
};

// Child ids = rank of the creation key; also the children's centres,
// parent centre + (+-k) per axis (geom_octree.cpp:222-230), and their child
// boxes.  When the parent's child-box centres are exact fp32 values (tail 0),
// the child's centre is one of them, and an fp32 sum whose TwoSum error is
// zero is the fp64 sum too; then no fp64 arithmetic is needed.  Otherwise
// (or when a sum is inexact) the centres are computed in fp64.
__global__ void k_assign_children(const uint32_t* __restrict__ firstq, uint64_t slots, const uint32_t* __restrict__ bitmap,
                                  const uint32_t* __restrict__ woff, const double* __restrict__ ctr,
                                  const float* __restrict__ pnbox, double k, double k_next, bool k_next_f32,
                                  uint32_t* __restrict__ ch, double* __restrict__ child_ctr,
                                  float* __restrict__ child_nbox) {
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < slots; s += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t fq = firstq[s];
    if (fq == kNone) { ch[s] = kNull; continue; }
    const uint64_t key = uint64_t(fq) * 8 + (7 - (s & 7));
    const uint32_t w = bitmap[key >> 5];
    const uint32_t rank = woff[key >> 5] + __popc(w & ((1u << (key & 31)) - 1u));
    ch[s] = rank;
    const uint64_t p = s >> 3;
    const uint32_t i = uint32_t(s & 7);
    float4* q = reinterpret_cast<float4*>(child_nbox + 8ull * rank);
    if (k_next_f32) {
      const float4* pb = reinterpret_cast<const float4*>(pnbox + 8ull * p);
      const float4 a = pb[0], b = pb[1];
      if (b.z == 0.f && b.w != 0.f) {
        const float c3[3] = {(i & 4) ? a.y : a.x, (i & 2) ? a.w : a.z, (i & 1) ? b.y : b.x};
        const float kf = float(k_next);
        float chi[6];
        bool exact = true;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          exact = sat::xsub(c3[ax], kf, chi[2 * ax]) && exact;
          exact = sat::xsub(c3[ax], -kf, chi[2 * ax + 1]) && exact;
        }
#pragma unroll
        for (int j = 0; j < 6; ++j) exact = exact && (fabsf(chi[j]) < 1.0e18f);
        if (exact) {
          child_ctr[3ull * rank + 0] = double(c3[0]);
          child_ctr[3ull * rank + 1] = double(c3[1]);
          child_ctr[3ull * rank + 2] = double(c3[2]);
          q[0] = make_float4(chi[0], chi[1], chi[2], chi[3]);
          q[1] = make_float4(chi[4], chi[5], 0.f, 1.f);
          continue;
        }
      }
    }
    const double cc[3] = {__dadd_rn(ctr[3 * p + 0], (i & 4) ? k : -k), __dadd_rn(ctr[3 * p + 1], (i & 2) ? k : -k),
                          __dadd_rn(ctr[3 * p + 2], (i & 1) ? k : -k)};
    child_ctr[3ull * rank + 0] = cc[0];
    child_ctr[3ull * rank + 1] = cc[1];
    child_ctr[3ull * rank + 2] = cc[2];
    sat::NodeBoxes nb;
    sat::node_boxes(cc, k_next, nb);
    q[0] = make_float4(nb.chi[0], nb.chi[1], nb.chi[2], nb.chi[3]);
    q[1] = make_float4(nb.chi[4], nb.chi[5], nb.clo, nb.ok);
  }
}

// Next frontier in (pair, child ascending) order, one tile of the expansion
// per block: a block scan of the hit counts plus the tile's offset.
__global__ void __launch_bounds__(kExpandThreads) k_emit_frontier(const uint32_t* __restrict__ f_tri,
                                                                  const uint32_t* __restrict__ f_node, uint64_t F,
                                                                  const uint8_t* __restrict__ hits,
                                                                  const uint32_t* __restrict__ tile_off,
                                                                  const uint32_t* __restrict__ ch,
                                                                  uint32_t* __restrict__ nf_tri,
                                                                  uint32_t* __restrict__ nf_node) {
  for (uint64_t tile = blockIdx.x; tile * kExpandThreads < F; tile += gridDim.x) {
    const uint64_t q = tile * kExpandThreads + threadIdx.x;
    uint32_t h = (q < F) ? hits[q] : 0u;
    uint32_t tot;
    uint32_t o = tile_off[tile] + block_excl_scan<uint32_t>(uint32_t(__popc(h)), &tot);
    if (!h) continue;
    const uint32_t t = f_tri ? f_tri[q] : uint32_t(q);
    const uint32_t node = f_node ? f_node[q] : 0u;
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

// testTriBox for the 8 children of arbitrary (triangle, node) pairs, with the
// decision sequence k_expand applies to a frontier pair: the slab
// classification first, the certified full test for the children it leaves
// open.  One pair per thread; bit ci of masks[i] = child ci overlaps.
__global__ void k_tri_box_children(const float* __restrict__ tris, const double* __restrict__ centers,
                                   const double* __restrict__ half_sides, uint64_t n, uint8_t* __restrict__ masks,
                                   unsigned long long* __restrict__ n_fallback) {
  unsigned fb = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const float* tp = tris + 9 * i;
    float t[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) t[j] = tp[j];
    const double* c = centers + 3 * i;
    const double k = half_sides[i];
    const double cc[3] = {c[0], c[1], c[2]};
    sat::NodeBoxes nb;
    sat::node_boxes(cc, k, nb);
    sat::Pair32 P;
    sat::pair_core(t, tp, c, nb, k, P);
    sat::pair_slabs(P);
    uint32_t m = 0, full = 0;
    for (int ci = 7; ci >= 0; --ci) {
      const int f = sat::child_fast(P, ci);
      if (f == 1) m |= 1u << ci;
      else if (f == 2) full |= 1u << ci;
    }
    if (full) {
      sat::pair_edges(P);
      for (uint32_t r = full; r; r &= r - 1) {
        const int ci = __ffs(int(r)) - 1;
        if (sat::child_full(P, ci, &fb)) m |= 1u << ci;
      }
    }
    masks[i] = uint8_t(m);
  }
  unsigned long long sum = fb;
  for (int o = 16; o; o >>= 1) sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(n_fallback, sum);
}

}  // namespace

void tri_box_children(Ctx& c, const float* h_tris, const double* h_centers, const double* h_half, uint64_t n,
                      uint8_t* h_masks, uint64_t* fallbacks) {
  const cudaStream_t st = c.stream;
  const uint64_t m = n ? n : 1;
  DBuf<float> d_t(9 * m, st);
  DBuf<double> d_c(3 * m, st), d_k(m, st);
  DBuf<uint8_t> d_m(m, st);
  DBuf<unsigned long long> d_fb(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_fb.get(), 0, 8, st));
  if (n) {
    SVDAG_CUDA(cudaMemcpyAsync(d_t.get(), h_tris, 36 * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_c.get(), h_centers, 24 * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_k.get(), h_half, 8 * n, cudaMemcpyHostToDevice, st));
    SVDAG_LAUNCH(c.ex, k_tri_box_children, grid_for(c.ex, n, 256), 256, 0, d_t.get(), d_c.get(), d_k.get(), n,
                 d_m.get(), d_fb.get());
    SVDAG_CUDA(cudaMemcpyAsync(h_masks, d_m.get(), n, cudaMemcpyDeviceToHost, st));
  }
  unsigned long long fbh = 0;
  SVDAG_CUDA(cudaMemcpyAsync(&fbh, d_fb.get(), 8, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  if (fallbacks) *fallbacks = fbh;
}

void phase_voxelize(Ctx& c, uint32_t levels, const double bb[6], const uint32_t* tri_list, uint64_t n_list) {
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
  c.leaf_ctr.release();
  c.leaf_ctr_n = 0;

  // level 0: the root
  c.lev[0].n = 1;
  c.lev[0].hdr.alloc(1, st);
  c.lev[0].ctr.alloc(3, st);
  c.lev[0].nbox.alloc(8, st);
  SVDAG_CUDA(cudaMemsetAsync(c.lev[0].hdr.get(), 0, 4, st));
  SVDAG_CUDA(cudaMemcpyAsync(c.lev[0].ctr.get(), P.root_c, 24, cudaMemcpyHostToDevice, st));
  {
    sat::NodeBoxes nb;
    sat::node_boxes(P.root_c, child_half_side(c.root_side, 0), nb);
    static thread_local float root_nb[8];
    for (int k = 0; k < 6; ++k) root_nb[k] = nb.chi[k];
    root_nb[6] = nb.clo;
    root_nb[7] = nb.ok;
    SVDAG_CUDA(cudaMemcpyAsync(c.lev[0].nbox.get(), root_nb, 32, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
  }

  // frontier; at level 0 the pairs (t, root) for every triangle, or for the
  // triangles of tri_list (ascending ids) when one is given
  DBuf<uint32_t> f_tri, f_node;
  const uint32_t* ft = tri_list;
  uint64_t F = tri_list ? n_list : c.n_tris;
  DBuf<uint64_t> d_total(1, st);
  DBuf<unsigned long long> d_vox(1, st), d_fb(1, st), d_tile(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_fb.get(), 0, 8, st));

  uint64_t pairs = 0;
  for (uint32_t l = 0; l < levels; ++l) {
    Level& L = c.lev[l];
    P.level = l;
    pairs += F;
    const bool leaf = (l == levels - 1);
    DBuf<uint32_t> firstq;
    DBuf<uint8_t> hits;
    DBuf<uint32_t> tile_hits;
    const uint64_t tiles = (F + kExpandThreads - 1) / kExpandThreads;
    if (!leaf) {
      firstq.alloc(8 * L.n, st);
      fill<uint32_t>(ex, firstq.get(), 8 * L.n, kNone);
      hits.alloc(F, st);
      tile_hits.alloc(tiles ? tiles : 1, st);
    }
    if (F) {
      if (kExpandDynamic) SVDAG_CUDA(cudaMemsetAsync(d_tile.get(), 0, sizeof(unsigned long long), st));
      SVDAG_LAUNCH(ex, k_expand, grid_for(ex, F, kExpandThreads, SVDAG_EXPAND_GRID_PER_SM), kExpandThreads, 0, P,
                   c.tris, ft, f_node.get(), F, L.ctr.get(), L.nbox.get(), L.hdr.get(), firstq.get(), hits.get(),
                   tile_hits.get(), d_fb.get(), kExpandDynamic ? d_tile.get() : nullptr);
    }
    if (leaf) break;

    // --- counts of level l+1 and of the next frontier (one host sync)
    const uint64_t slots = 8 * L.n;
    const uint64_t words = (8 * F + 31) / 32;
    DBuf<uint32_t> bitmap(words ? words : 1, st), woff(words ? words : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(bitmap.get(), 0, 4 * (words ? words : 1), st));
    SVDAG_LAUNCH(ex, k_mark_keys, grid_for(ex, slots, 256), 256, 0, firstq.get(), slots, bitmap.get());
    DBuf<uint32_t> d_n32(1, st);
    device_exclusive_scan<uint32_t>(ex, PopcIn{bitmap.get()}, words, U32Out{woff.get()}, d_n32.get());
    DBuf<uint32_t> tile_off(tiles ? tiles : 1, st);
    device_exclusive_scan<uint64_t>(ex, U32toU64In{tile_hits.get()}, tiles, U64to32Out{tile_off.get()}, d_total.get());
    uint64_t F_next = 0;
    uint32_t n32 = 0;
    SVDAG_CUDA(cudaMemcpyAsync(&n32, d_n32.get(), 4, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaMemcpyAsync(&F_next, d_total.get(), 8, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
    if (F_next >= (1ull << 32)) throw Error(SVDAG_ERR_OVERFLOW, "voxelize: frontier exceeds 2^32 pairs");

    // --- create level l+1 in reference creation order
    const uint64_t n_next = n32;
    Level& N = c.lev[l + 1];
    N.n = n_next;
    L.ch.alloc(slots, st);
    N.hdr.alloc(n_next ? n_next : 1, st);
    N.ctr.alloc(3 * (n_next ? n_next : 1), st);
    N.nbox.alloc(8 * (n_next ? n_next : 1), st);
    SVDAG_CUDA(cudaMemsetAsync(N.hdr.get(), 0, 4 * (n_next ? n_next : 1), st));
    // the fp32 path of node_boxes needs an fp32-exact half side in range
    const double k_next = child_half_side(c.root_side, l + 1);
    const bool k_next_f32 = k_next > 1.0e-30 && k_next < 1.0e18 && double(float(k_next)) == k_next;
    SVDAG_LAUNCH(ex, k_assign_children, grid_for(ex, slots, 256), 256, 0, firstq.get(), slots, bitmap.get(),
                 woff.get(), L.ctr.get(), L.nbox.get(), child_half_side(c.root_side, l), k_next, k_next_f32,
                 L.ch.get(), N.ctr.get(), N.nbox.get());
    firstq.release();
    bitmap.release();
    woff.release();

    // --- next frontier
    DBuf<uint32_t> nf_tri(F_next ? F_next : 1, st), nf_node(F_next ? F_next : 1, st);
    if (F)
      SVDAG_LAUNCH(ex, k_emit_frontier, unsigned(tiles < uint64_t(ex.sm_count) * 8 ? tiles : uint64_t(ex.sm_count) * 8),
                   kExpandThreads, 0, ft, f_node.get(), F, hits.get(), tile_off.get(), L.ch.get(),
                   nf_tri.get(), nf_node.get());
    f_tri = std::move(nf_tri);
    f_node = std::move(nf_node);
    ft = f_tri.get();
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
  // leavesCenters: the centres the leaf level's nodes were created with
  // (none for a single level, whose root is the leaf)
  if (c.keep_leaf_centers && levels >= 2) {
    c.leaf_ctr = std::move(c.lev[levels - 1].ctr);
    c.leaf_ctr_n = c.lev[levels - 1].n;
  }
  for (auto& L : c.lev) {
    L.ctr.release();
    L.nbox.release();
  }

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
  c.st.frontier_pairs = pairs;
  c.st.sat_fallbacks = read_scalar(ex, d_fb.get());
  c.state = SVDAG_S_SVO;
}

}  // namespace svdag
