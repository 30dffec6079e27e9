// GeomOctree::toDAG and GeomOctree::toSDAG on the GPU.
//
// toDAG (src/symvox/geom_octree.cpp:462-548) keeps, per level and bottom-up,
// the first occurrence of every distinct node key (mask, children[8],
// mirror masks) in index order and remaps the parents.  Here:
//   * leaf level: the key is the 8-bit mask, so a 256-entry first-occurrence
//     table (block-local atomicMin, then global) and a rank table replace the
//     map;
//   * inner levels: an open-addressing hash table of packed (tag32 | index)
//     slots; equal keys converge on the minimum index with atomicMin, so the
//     representative of every key is its first occurrence; a scan over
//     "is representative" flags gives the first-occurrence order ids.
//
// toSDAG (src/symvox/geom_octree.cpp:551-697) is greedy and sequential in the
// reference: node i takes the first of its 8 mirror variants (identity, X, Y,
// Z, XY, XZ, YZ, XYZ; variants normalised by invertInvs) found among the
// unique nodes before it, else becomes unique.  Only the first occurrence of
// a raw key can be unique, so the candidate for variant k of node i is the
// first occurrence of the raw key equal to that variant.  Node i is then
// decided once every earlier-ordered candidate is decided: one pass in index
// order per thread, waiting on undecided candidates (the lowest undecided
// index never waits, so the pass advances), gives exactly the sequential
// result.
//
// Each phase runs as one persistent cooperative kernel over all levels
// (k_dag_persistent, k_sdag_persistent; barrier and launch in persist.cuh)
// with a single read of the reduced counts at the end.  The per-level
// toDAG kernels serve the entry point that works in caller-provided scratch.
#include <algorithm>
#include <cstdlib>

#include "ctx.cuh"
#include "dedup.cuh"
#include "persist.cuh"

namespace svdag {
namespace {

constexpr uint32_t kUndecided = 0xFFFFFFFFu;
constexpr uint32_t kUnique = 0xFFFFFFFEu;

struct RepFlagIn {
  const uint32_t* rep;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return rep[i] == uint32_t(i) ? 1u : 0u; }
};
struct U32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};

// Unique nodes to the new level; corr[i] = id of i's representative.
__global__ void k_compact_dag(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                              const uint32_t* __restrict__ rep, const uint32_t* __restrict__ newid,
                              uint32_t* __restrict__ out_hdr, uint32_t* __restrict__ out_ch, uint32_t* __restrict__ corr) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t r = rep[i];
    if (r == kNone) { corr[i] = 0; continue; }
    corr[i] = newid[r];
    if (r == uint32_t(i)) {
      const uint32_t id = newid[i];
      out_hdr[id] = hdr[i];
      if (ch) {
        uint32_t c[8];
        load_children(ch, i, c);
        store_children(out_ch, id, c);
      }
    }
  }
}

// Parents at level lev-1: existing children (mask bits) -> corr.
__global__ void k_remap_parents(const uint32_t* __restrict__ phdr, uint32_t* __restrict__ pch, uint64_t np,
                                const uint32_t* __restrict__ corr) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = phdr[p] & 0xFFu;
    if (!m) continue;
    uint32_t c[8];
    load_children(pch, p, c);
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) c[j] = corr[c[j]];
    store_children(pch, p, c);
  }
}

// --- leaf level of toDAG: the key is the 8-bit mask.
__global__ void k_leaf_first(const uint32_t* __restrict__ hdr, uint64_t n, uint32_t* __restrict__ first) {
  __shared__ uint32_t sf[256];
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = kNone;
  __syncthreads();
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = hdr[i] & 0xFFu;
    if (m && sf[m] > uint32_t(i)) atomicMin(&sf[m], uint32_t(i));  // read first: common masks repeat
  }
  __syncthreads();
  for (int m = threadIdx.x; m < 256; m += blockDim.x)
    if (sf[m] != kNone) atomicMin(&first[m], sf[m]);
}

// rank[m] = first-occurrence order of mask m; writes the reduced leaf level.
__global__ void k_leaf_rank(const uint32_t* __restrict__ first, uint32_t* __restrict__ rank,
                            uint32_t* __restrict__ out_hdr, uint32_t* __restrict__ count) {
  __shared__ uint32_t sf[256];
  const int m = threadIdx.x;
  sf[m] = first[m];
  __syncthreads();
  uint32_t r = 0;
  if (sf[m] != kNone) {
    for (int k = 0; k < 256; ++k) r += (sf[k] < sf[m]) ? 1u : 0u;
    rank[m] = r;
    out_hdr[r] = uint32_t(m);
  } else {
    // a pointer to an empty node (only a joined chunk root can be one) maps to
    // 0, the reference's default correspondence (geom_octree.cpp:493-496)
    rank[m] = (m == 0) ? 0u : kNone;
  }
  __syncthreads();
  if (m == 0) {
    uint32_t c = 0;
    for (int k = 0; k < 256; ++k) c += (sf[k] != kNone) ? 1u : 0u;
    *count = c;
  }
}

__global__ void k_remap_parents_leafrank(const uint32_t* __restrict__ phdr, uint32_t* __restrict__ pch, uint64_t np,
                                         const uint32_t* __restrict__ leaf_hdr, const uint32_t* __restrict__ rank) {
  __shared__ uint32_t sr[256];
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sr[m] = rank[m];
  __syncthreads();
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = phdr[p] & 0xFFu;
    if (!m) continue;
    uint32_t c[8];
    load_children(pch, p, c);
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) {
        const uint32_t lm = leaf_hdr[c[j]] & 0xFFu;
        // an empty leaf never has a set parent bit after cleanEmptyNodes; the
        // reference's zero-initialised correspondence is kept for it
        c[j] = lm ? sr[lm] : 0u;
      }
    store_children(pch, p, c);
  }
}

// --- toSDAG helpers ---------------------------------------------------------

__device__ __forceinline__ uint32_t perm_bits(uint32_t m, int flip) {
  if (flip & 4) m = ((m & 0x0Fu) << 4) | ((m & 0xF0u) >> 4);
  if (flip & 2) m = ((m & 0x33u) << 2) | ((m & 0xCCu) >> 2);
  if (flip & 1) m = ((m & 0x55u) << 1) | ((m & 0xAAu) >> 1);
  return m;
}

// Node::mirror (src/symvox/octree_node.cpp:88-195): flip bit 4 = X, 2 = Y, 1 = Z.
__device__ __forceinline__ void mirror_node(uint32_t h, const uint32_t c[8], int flip, uint32_t& oh, uint32_t oc[8]) {
  uint32_t mask = perm_bits(h & 0xFFu, flip);
  uint32_t mx = perm_bits((h >> 8) & 0xFFu, flip);
  uint32_t my = perm_bits((h >> 16) & 0xFFu, flip);
  uint32_t mz = perm_bits((h >> 24) & 0xFFu, flip);
  uint32_t ptr = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    oc[k] = c[k ^ flip];
    if (oc[k] != kNull) ptr |= 1u << k;
  }
  if (flip & 4) mx ^= ptr;
  if (flip & 2) my ^= ptr;
  if (flip & 1) mz ^= ptr;
  oh = mask | (mx << 8) | (my << 16) | (mz << 24);
}

__device__ __forceinline__ bool same_key(uint32_t h1, const uint32_t c1[8], uint32_t h2, const uint32_t c2[8]) {
  bool eq = (h1 == h2);
#pragma unroll
  for (int k = 0; k < 8; ++k) eq &= (c1[k] == c2[k]);
  return eq;
}

// lookup order identity, X, Y, Z, XY, XZ, YZ, XYZ (geom_octree.cpp:630-658)
__constant__ int kVarFlip[8] = {0, 4, 2, 1, 6, 5, 3, 7};
// correspondence mirror flags for each variant: bit0 X, bit1 Y, bit2 Z
__constant__ uint8_t kVarAxes[8] = {0, 1, 2, 4, 3, 5, 6, 7};

// --- persistent forms of toDAG and toSDAG ------------------------------------
// One cooperative launch per phase runs every level (bottom-up), the
// sub-steps of a level separated by grid barriers; per-level scratch is
// sized from the largest level, outputs from each level's input count
// (a level only shrinks), and the reduced counts are read once at the end.

constexpr unsigned kResolveSpinLimit = 1u << 16;  // polls of one wait in the resolution pass

struct RedLevel {
  uint32_t* hdr;   // input level (children remapped in place by the level below)
  uint32_t* ch;    // null on the leaf level of toSDAG
  uint32_t* ohdr;  // reduced level, capacity n (toDAG leaf: 256)
  uint32_t* och;
  uint8_t* oinv;   // toSDAG: invariance bits of the reduced level
  uint64_t n;
  uint64_t slots;  // hash table size for this level (power of two)
};

struct RedArgs {
  RedLevel lev[kMaxRedLevels];
  uint32_t levels;
  unsigned long long* slots;  // hash table, sized for the largest level
  uint32_t* slot_of;          // per node of the current level
  uint32_t* rep;              // toDAG: first occurrence of the node's key
  uint32_t* newid;
  uint32_t* bsum;             // per block
  uint32_t* first;            // toDAG leaf: first occurrence per mask [256]
  uint32_t* cand;             // toSDAG: 8 candidates per node
  uint32_t* state;            // toSDAG: kUndecided, kUnique or the matched node
  uint8_t* inv;               // toSDAG: invariance bits per node
  uint8_t* var;               // toSDAG: variant of the match
  unsigned long long* left;   // toSDAG: nodes whose resolution wait ran out
  uint32_t* cnt;              // [levels] reduced counts
  int* err;
  GridBar* bar;
  unsigned long long* trace;  // step trace or null
  uint32_t top;               // toDAG: deepest level still to reduce (levels below: done by bulk launches)
};

// Level-ordered ids of the flagged nodes of this block's share:
// newid[i] = number of flagged nodes before i.  bsum holds every block's
// count (written before the last barrier); the total goes to *cnt.
template <class Flag>
__device__ __forceinline__ void emit_ids(const RedArgs& a, uint64_t b0, uint64_t b1, Flag flag, uint32_t* cnt) {
  uint32_t total;
  uint32_t base = block_offset(a.bsum, &total);
  if (blockIdx.x == 0 && threadIdx.x == 0) *cnt = total;
  for (uint64_t t0 = b0; t0 < b1; t0 += blockDim.x) {
    const uint64_t i = t0 + threadIdx.x;
    const uint32_t f = (i < b1 && flag(i)) ? 1u : 0u;
    uint32_t tile;
    const uint32_t pre = block_excl_scan<uint32_t>(f, &tile);
    if (f) a.newid[i] = base + pre;
    base += tile;
  }
}

template <class Flag>
__device__ __forceinline__ void count_share(const RedArgs& a, uint64_t b0, uint64_t b1, Flag flag) {
  uint32_t c = 0;
  SVDAG_BLOCK_STRIDE(i, b0, b1) c += flag(i) ? 1u : 0u;
  c = block_sum(c);
  if (threadIdx.x == 0) a.bsum[blockIdx.x] = c;
}

// toDAG (geom_octree.cpp:462-548): the leaf level by its 256 masks, inner
// levels through the hash table; each level's parents are remapped before
// the parent level is deduplicated.
__global__ void __launch_bounds__(kDagThreads, 1) k_dag_persistent(const RedArgs a) {
  __shared__ uint32_t sf[256], sr[256];
  unsigned trace_pos = 0;
  trace_mark(a.trace, trace_pos, kStEntry);
  const uint32_t L = a.levels;  // >= 2
  const RedLevel& leaf = a.lev[L - 1];
  const uint32_t inner0 = a.top == L - 1 ? L - 2 : a.top;  // first inner level reduced here
  if (blockIdx.x == 0)
    for (int m = threadIdx.x; m < 256; m += blockDim.x) a.first[m] = kNone;
  if (inner0 >= 1) clear_slots(a.slots, a.lev[inner0].slots);
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = kNone;
  SVDAG_STEP(a, L - 1, kStPrologue);
  if (a.top == L - 1) {
    // leaf level: first occurrence of every mask (four headers per 16-byte load)
    {
      const uint64_t n4 = leaf.n / 4;
      const uint4* h4 = reinterpret_cast<const uint4*>(leaf.hdr);
      SVDAG_GRID_STRIDE(q, n4) {
        const uint4 w = h4[q];
        const uint32_t hv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t m = hv[j] & 0xFFu, i = uint32_t(4 * q + j);
          if (m && sf[m] > i) atomicMin(&sf[m], i);  // read first: common masks repeat
        }
      }
      SVDAG_GRID_STRIDE(i, leaf.n - 4 * n4) {
        const uint32_t k = uint32_t(4 * n4 + i), m = leaf.hdr[k] & 0xFFu;
        if (m && sf[m] > k) atomicMin(&sf[m], k);
      }
    }
    __syncthreads();
    for (int m = threadIdx.x; m < 256; m += blockDim.x)
      if (sf[m] != kNone) atomicMin(&a.first[m], sf[m]);
    SVDAG_STEP(a, L - 1, kStLeafFirst);

    // rank of each mask by first occurrence (every block), the reduced leaf
    // level (block 0) and the leaves' parents
    for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = a.first[m];
    __syncthreads();
    uint32_t present = 0;
    for (int m = threadIdx.x; m < 256; m += blockDim.x) {
      uint32_t r;
      if (sf[m] != kNone) {
        r = 0;
        for (int k = 0; k < 256; ++k) r += (sf[k] < sf[m]) ? 1u : 0u;
        if (blockIdx.x == 0) leaf.ohdr[r] = uint32_t(m);
        ++present;
      } else {
        // a pointer to an empty node (only a joined chunk root can be one) maps
        // to 0, the reference's default correspondence (geom_octree.cpp:493-496)
        r = (m == 0) ? 0u : kNone;
      }
      sr[m] = r;
    }
    present = block_sum(present);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.cnt[L - 1] = present;
    {
      const RedLevel& P = a.lev[L - 2];
      SVDAG_GRID_STRIDE(p, P.n) {
        const uint32_t m = P.hdr[p] & 0xFFu;
        if (!m) continue;
        uint32_t c[8];
        load_children(P.ch, p, c);
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if ((m >> j) & 1u) {
            // an empty leaf never has a set parent bit after cleanEmptyNodes;
            // the reference's zero-initialised correspondence is kept for it
            const uint32_t lm = leaf.hdr[c[j]] & 0xFFu;
            c[j] = lm ? sr[lm] : 0u;
          }
        store_children(P.ch, p, c);
      }
    }
    SVDAG_STEP(a, L - 1, kStLeafRank);
  }

  for (uint32_t lev = inner0; lev >= 1; --lev) {
    const RedLevel& V = a.lev[lev];
    const Table T{a.slots, V.slots - 1};
    SVDAG_GRID_STRIDE(i, V.n) {
      uint32_t h, c[8];
      load_key(V.hdr, V.ch, i, h, c);
      if ((h & 0xFFu) == 0) { a.slot_of[i] = kNone; continue; }  // empty nodes are skipped (geom_octree.cpp:495)
      a.slot_of[i] = uint32_t(table_insert(T, V.hdr, V.ch, uint32_t(i), h, c, a.err));
    }
    SVDAG_STEP(a, lev, kStInsert);

    uint64_t b0, b1;
    block_share(V.n, b0, b1);
    SVDAG_BLOCK_STRIDE(i, b0, b1) {
      const uint32_t s = a.slot_of[i];
      a.rep[i] = (s == kNone) ? kNone : uint32_t(a.slots[s]);
    }
    __syncthreads();
    auto is_rep = [&](uint64_t i) { return a.rep[i] == uint32_t(i); };
    count_share(a, b0, b1, is_rep);
    SVDAG_STEP(a, lev, kStCount);

    emit_ids(a, b0, b1, is_rep, &a.cnt[lev]);
    if (lev >= 2) clear_slots(a.slots, a.lev[lev - 1].slots);
    SVDAG_STEP(a, lev, kStEmit);

    SVDAG_GRID_STRIDE(i, V.n) {
      if (a.rep[i] != uint32_t(i)) continue;
      const uint32_t id = a.newid[i];
      V.ohdr[id] = V.hdr[i];
      uint32_t c[8];
      load_children(V.ch, i, c);
      store_children(V.och, id, c);
    }
    const RedLevel& P = a.lev[lev - 1];
    SVDAG_GRID_STRIDE(p, P.n) {
      const uint32_t m = P.hdr[p] & 0xFFu;
      if (!m) continue;
      uint32_t c[8];
      load_children(P.ch, p, c);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if ((m >> j) & 1u) {
          const uint32_t r = a.rep[c[j]];
          c[j] = (r == kNone) ? 0u : a.newid[r];
        }
      store_children(P.ch, p, c);
    }
    SVDAG_STEP(a, lev, kStCompact);
  }
}

// toSDAG (geom_octree.cpp:551-697): per level, candidates of the 8 mirror
// variants, the resolution pass (see the file comment), then the unique nodes
// in order and the parents' pointers with their mirror bits.
__global__ void __launch_bounds__(kRedThreads, 1) k_sdag_persistent(const RedArgs a) {
  const uint32_t L = a.levels;  // >= 2
  unsigned trace_pos = 0;
  trace_mark(a.trace, trace_pos, kStEntry);
  clear_slots(a.slots, a.lev[L - 1].slots);
  if (blockIdx.x == 0 && threadIdx.x == 0) a.left[0] = 0;
  SVDAG_STEP(a, L - 1, kStPrologue);
  const uint8_t* child_inv = nullptr;
  for (uint32_t lev = L - 1; lev >= 1; --lev) {
    const RedLevel& V = a.lev[lev];
    const uint64_t n = V.n;
    const Table T{a.slots, V.slots - 1};
    SVDAG_GRID_STRIDE(i, n) {
      uint32_t h, c[8];
      load_key(V.hdr, V.ch, i, h, c);
      if ((h & 0xFFu) == 0) { a.slot_of[i] = kNone; continue; }
      a.slot_of[i] = uint32_t(table_insert(T, V.hdr, V.ch, uint32_t(i), h, c, a.err));
    }
    SVDAG_STEP(a, lev, kStInsert);

    // invariance bits and the candidates of the variants: eight lanes per
    // node, all on the same path -- lane v looks variant v up (v = 0: the raw
    // key, whose first occurrence the table holds), lanes 1-3 also test the
    // node's invariance on X, Y, Z (n == n.mirror(axis), geom_octree.cpp:604-606),
    // and lane k loads child k's invariance bits, shared by shuffles
    {
      const int v = threadIdx.x & 7;
      const int g0 = int(threadIdx.x & 24);  // first lane of the group in the warp
      const unsigned gmask = 0xFFu << g0;
      const int flip = kVarFlip[v];
      const uint64_t stride = (uint64_t(gridDim.x) * blockDim.x) >> 3;
      for (uint64_t i = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 3; i < n; i += stride) {
        uint32_t h, c[8];
        load_key(V.hdr, V.ch, i, h, c);
        const uint32_t mine = (child_inv && c[v] != kNull) ? uint32_t(child_inv[c[v]]) : 0u;
        uint32_t cinv[8];  // invariance bits of the child at mirrored position k
#pragma unroll
        for (int k = 0; k < 8; ++k) cinv[k] = __shfl_sync(gmask, mine, g0 | (k ^ flip));
        uint32_t vh, vc[8];
        mirror_node(h, c, flip, vh, vc);
        // lanes 1, 2, 3 hold the X, Y, Z mirrors (flips 4, 2, 1)
        const bool inv_bit = (v >= 1 && v <= 3) && same_key(h, c, vh, vc);
        const unsigned ib = __ballot_sync(gmask, inv_bit) >> g0;
        if (child_inv) {
          // invertInvs (geom_octree.cpp:822-831): drop the mirror bit of an
          // axis of this variant when the child is invariant on it
          uint32_t clrx = 0, clry = 0, clrz = 0;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            if (vc[k] == kNull) continue;
            const uint32_t ci = cinv[k];
            if ((flip & 4) && (ci & 1u)) clrx |= 1u << k;
            if ((flip & 2) && (ci & 2u)) clry |= 1u << k;
            if ((flip & 1) && (ci & 4u)) clrz |= 1u << k;
          }
          vh &= ~((clrx << 8) | (clry << 16) | (clrz << 24));
        }
        // lane 0: an empty node (never in a DAG) has no slot and no candidate
        a.cand[uint64_t(v) * n + i] = (v == 0 && (h & 0xFFu) == 0) ? kNone : table_find(T, V.hdr, V.ch, vh, vc);
        if (v == 0) {
          a.inv[i] = uint8_t((ib >> 1) & 7u);  // bit 0 X (lane 1), 1 Y (lane 2), 2 Z (lane 3)
          a.state[i] = kUndecided;
        }
      }
    }
    SVDAG_STEP(a, lev, kStCandidates);

    // resolution in one pass: each thread takes its nodes in index order; a
    // candidate before the node that is still undecided is waited for.  The
    // lowest undecided node waits for nothing, so the pass always advances
    // (all blocks are resident).  A wait that exceeds its limit leaves the
    // node undecided and flags the level for the serial finish.
    {
      unsigned long long gave_up = 0;
      SVDAG_GRID_STRIDE(i, n) {
        bool done = false, stalled = false;
        for (int k = 0; k < 8; ++k) {
          const uint32_t cnd = a.cand[uint64_t(k) * n + i];
          if (cnd == kNone || cnd >= uint32_t(i)) continue;
          uint32_t s = ld_cg32(&a.state[cnd]);
          for (unsigned spins = 0; s == kUndecided && spins < kResolveSpinLimit; ++spins) {
            __nanosleep(64);
            s = ld_cg32(&a.state[cnd]);
          }
          if (s == kUndecided) { stalled = true; break; }
          if (s == kUnique) {
            a.var[i] = uint8_t(k);
            __stcg(&a.state[i], cnd);
            done = true;
            break;
          }
        }
        if (stalled) { ++gave_up; continue; }
        if (!done) __stcg(&a.state[i], kUnique);
      }
      gave_up = block_sum(gave_up);
      if (threadIdx.x == 0 && gave_up) atomicAdd(&a.left[0], gave_up);
    }
    SVDAG_STEP(a, lev, kStRound);
    if (a.left[0] != 0) {
      // long dependency chains: one thread finishes in index order
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (uint64_t i = 0; i < n; ++i) {
          if (a.state[i] != kUndecided) continue;
          bool done = false;
          for (int k = 0; k < 8 && !done; ++k) {
            const uint32_t cnd = a.cand[uint64_t(k) * n + i];
            if (cnd == kNone || cnd >= uint32_t(i)) continue;
            if (ld_cg32(&a.state[cnd]) == kUnique) { a.var[i] = uint8_t(k); __stcg(&a.state[i], cnd); done = true; }
          }
          if (!done) __stcg(&a.state[i], kUnique);
        }
      }
      SVDAG_STEP(a, lev, kStSerial);
    }

    uint64_t b0, b1;
    block_share(n, b0, b1);
    auto is_unique = [&](uint64_t i) { return a.state[i] == kUnique; };
    count_share(a, b0, b1, is_unique);
    SVDAG_STEP(a, lev, kStCount);

    // every block has read the stall counter: reset it for the next level
    emit_ids(a, b0, b1, is_unique, &a.cnt[lev]);
    if (lev >= 2) clear_slots(a.slots, a.lev[lev - 1].slots);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.left[0] = 0;
    SVDAG_STEP(a, lev, kStEmit);

    SVDAG_GRID_STRIDE(i, n) {
      if (a.state[i] != kUnique) continue;
      const uint32_t id = a.newid[i];
      V.ohdr[id] = V.hdr[i];
      V.oinv[id] = a.inv[i];
      if (V.ch) {
        uint32_t c[8];
        load_children(V.ch, i, c);
        store_children(V.och, id, c);
      }
    }
    // parents: children with a pointer -> (id, mirror bits)
    const RedLevel& P = a.lev[lev - 1];
    SVDAG_GRID_STRIDE(p, P.n) {
      uint32_t c[8];
      load_children(P.ch, p, c);
      uint32_t mx = 0, my = 0, mz = 0;
      bool any = false;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (c[j] == kNull) continue;
        any = true;
        const uint32_t old = c[j];
        const uint32_t s = a.state[old];
        uint32_t m = 0;
        if (s == kUnique) {
          c[j] = a.newid[old];
        } else {
          c[j] = a.newid[s];
          m = kVarAxes[a.var[old]];
        }
        if (m & 1u) mx |= 1u << j;
        if (m & 2u) my |= 1u << j;
        if (m & 4u) mz |= 1u << j;
      }
      if (!any) continue;
      store_children(P.ch, p, c);
      if (mx | my | mz) P.hdr[p] = P.hdr[p] | (mx << 8) | (my << 16) | (mz << 24);
    }
    child_inv = V.oinv;
    SVDAG_STEP(a, lev, kStCompact);
  }
}

}  // namespace

// Bottom levels above this many nodes are reduced by ordinary launches at
// full occupancy before the persistent kernel takes the rest: on levels of
// hundreds of millions of nodes (the chunks of a depth-15 scene) the hash
// inserts and gathers want every warp slot of an SM, and the launches cost
// nothing next to their work.  SVDAG_BULK_LEVEL_NODES in the environment
// overrides the threshold.
constexpr uint64_t kBulkLevelNodes = 32ull << 20;
uint64_t bulk_level_nodes() {
  const char* e = std::getenv("SVDAG_BULK_LEVEL_NODES");
  if (!e || !*e) return kBulkLevelNodes;
  return std::strtoull(e, nullptr, 10);
}

void phase_reduce_dag(Ctx& c) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toDAG: the octree is not an SVO or DAG");
  const uint32_t L = c.levels;
  if (L > kMaxRedLevels) throw Error(SVDAG_ERR_INVALID_ARG, "toDAG: too many levels");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  uint64_t nnodes = 1;
  if (L >= 2) {
    RedArgs a{};
    a.levels = L;
    uint64_t max_n = 1, max_slots = 32;
    std::vector<DBuf<uint32_t>> ohdr(L), och(L);
    // levels reduced by bulk launches: the bottom ones above kBulkLevelNodes
    const uint64_t bulk = bulk_level_nodes();
    uint32_t top = L - 1;
    while (top >= 1 && c.lev[top].n > bulk) --top;
    a.top = top;
    for (uint32_t l = 0; l < L; ++l) {
      Level& V = c.lev[l];
      RedLevel& R = a.lev[l];
      R.hdr = V.hdr.get();
      R.ch = V.ch.get();
      R.n = V.n;
      if (l == 0) continue;
      if (l == L - 1) {
        ohdr[l].alloc(256, st);
      } else {
        if (V.n >= 0xFFFFFFF0ull) throw Error(SVDAG_ERR_OVERFLOW, "toDAG: more than 2^32 nodes in a level");
        R.slots = table_slots(V.n);
        if (l <= top) {
          max_n = std::max<uint64_t>(max_n, V.n);
          max_slots = std::max<uint64_t>(max_slots, R.slots);
        }
        ohdr[l].alloc(V.n ? V.n : 1, st);
        och[l].alloc(8 * (V.n ? V.n : 1), st);
        R.och = och[l].get();
      }
      R.ohdr = ohdr[l].get();
    }
    DBuf<RedCtl> ctl(1, st);
    SVDAG_CUDA(cudaMemsetAsync(ctl.get(), 0, sizeof(RedCtl), st));
    RedCtl* d_ctl = ctl.get();
    // bulk levels, bottom-up (no host synchronisation: counts go to the control block)
    for (uint32_t lev = L - 1; lev > top; --lev) {
      const Level& V = c.lev[lev];
      Level& P = c.lev[lev - 1];
      const uint64_t n = V.n;
      if (lev == L - 1) {
        DBuf<uint32_t> first(256, st), rank(256, st);
        fill<uint32_t>(ex, first.get(), 256, kNone);
        SVDAG_LAUNCH(ex, k_leaf_first, grid_for(ex, n, 256, 4), 256, 0, V.hdr.get(), n, first.get());
        SVDAG_LAUNCH(ex, k_leaf_rank, 1, 256, 0, first.get(), rank.get(), ohdr[lev].get(), &d_ctl->cnt[lev]);
        if (P.n)
          SVDAG_LAUNCH(ex, k_remap_parents_leafrank, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n,
                       V.hdr.get(), rank.get());
      } else {
        DBuf<unsigned long long> tb;
        const Table T = make_table(ex, n, tb);
        DBuf<uint32_t> slot_of(n, st), rep(n, st), newid(n, st), corr(n, st);
        SVDAG_LAUNCH(ex, k_insert, grid_for(ex, n, 256), 256, 0, T, V.hdr.get(), V.ch.get(), n, slot_of.get(),
                     &d_ctl->err);
        SVDAG_LAUNCH(ex, k_rep, grid_for(ex, n, 256), 256, 0, T, slot_of.get(), n, rep.get());
        tb.release();
        device_exclusive_scan<uint32_t>(ex, RepFlagIn{rep.get()}, n, U32Out{newid.get()}, &d_ctl->cnt[lev]);
        SVDAG_LAUNCH(ex, k_compact_dag, grid_for(ex, n, 256), 256, 0, V.hdr.get(), V.ch.get(), n, rep.get(),
                     newid.get(), ohdr[lev].get(), och[lev].get(), corr.get());
        if (P.n)
          SVDAG_LAUNCH(ex, k_remap_parents, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n, corr.get());
      }
    }
    PhaseTrace trace(st);
    if (top >= 1) {
      const uint64_t work = top == L - 1 ? std::max<uint64_t>(max_n, c.lev[L - 1].n) : max_n;
      const unsigned grid = persistent_grid(ex, k_dag_persistent, kDagThreads, work);
      DBuf<unsigned long long> slots(max_slots, st);
      DBuf<uint32_t> slot_of(max_n, st), rep(max_n, st), newid(max_n, st), bsum(grid, st), first(256, st);
      a.slots = slots.get();
      a.slot_of = slot_of.get();
      a.rep = rep.get();
      a.newid = newid.get();
      a.bsum = bsum.get();
      a.first = first.get();
      a.cnt = d_ctl->cnt;
      a.err = &d_ctl->err;
      a.bar = &d_ctl->bar;
      a.trace = trace.ptr();
      launch_persistent(ex, "k_dag_persistent", k_dag_persistent, grid, kDagThreads, 0, a);
    }
    RedCtl h;
    try {
      h = finish_persistent(ex, d_ctl, "toDAG");
    } catch (const Error&) {
      // the parents were remapped in place: the octree must be rebuilt
      c.state = SVDAG_S_EMPTY;
      throw;
    }
    trace.report(ex, "toDAG");
    for (uint32_t l = 1; l < L; ++l) {
      Level& V = c.lev[l];
      V.n = h.cnt[l];
      V.hdr = std::move(ohdr[l]);
      fit_buffer(V.hdr, V.n, st);
      if (l + 1 < L) {
        V.ch = std::move(och[l]);
        fit_buffer(V.ch, 8 * V.n, st);
      }
      nnodes += V.n;
    }
  }
  c.st.n_nodes_dag = nnodes;
  c.st.n_nodes = nnodes;
  c.state = SVDAG_S_DAG;
}

void phase_reduce_sdag(Ctx& c) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toSDAG: the octree is not a DAG");
  if (c.state == SVDAG_S_SVO && c.levels >= 2) {
    // The reference also reduces an SVO straight to an SDAG ("not best way",
    // geom_octree.cpp:554-556); its symmetry classes appear in the same
    // first-occurrence order whether or not toDAG ran first, so the result
    // is the DAG's toSDAG.  Its toSDAG leaves nNodesDAG as it was; the
    // SVO's outside masks go, as toDAG drops them.
    const uint64_t dag_nodes = c.st.n_nodes_dag;
    phase_reduce_dag(c);
    for (auto& V : c.lev) V.outm.release();
    c.st.n_nodes_dag = dag_nodes;
  }
  const uint32_t L = c.levels;
  if (L > kMaxRedLevels) throw Error(SVDAG_ERR_INVALID_ARG, "toSDAG: too many levels");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  uint64_t nnodes = 0;
  if (L >= 2) {
    RedArgs a{};
    a.levels = L;
    uint64_t max_n = 1, max_slots = 32;
    std::vector<DBuf<uint32_t>> ohdr(L), och(L);
    std::vector<DBuf<uint8_t>> oinv(L);
    for (uint32_t l = 0; l < L; ++l) {
      Level& V = c.lev[l];
      RedLevel& R = a.lev[l];
      R.hdr = V.hdr.get();
      R.ch = (l + 1 < L) ? V.ch.get() : nullptr;
      R.n = V.n;
      if (l == 0) continue;
      if (V.n >= 0xFFFFFFF0ull) throw Error(SVDAG_ERR_OVERFLOW, "toSDAG: more than 2^32 nodes in a level");
      R.slots = table_slots(V.n);
      max_n = std::max<uint64_t>(max_n, V.n);
      max_slots = std::max<uint64_t>(max_slots, R.slots);
      const uint64_t cap = V.n ? V.n : 1;
      ohdr[l].alloc(cap, st);
      oinv[l].alloc(cap, st);
      if (R.ch) och[l].alloc(8 * cap, st);
      R.ohdr = ohdr[l].get();
      R.och = och[l].get();
      R.oinv = oinv[l].get();
    }
    const unsigned grid = persistent_grid(ex, k_sdag_persistent, kRedThreads, max_n);
    DBuf<unsigned long long> slots(max_slots, st), left(1, st);
    DBuf<uint32_t> slot_of(max_n, st), cand(8 * max_n, st), state(max_n, st), newid(max_n, st), bsum(grid, st);
    DBuf<uint8_t> inv(max_n, st), var(max_n, st);
    DBuf<RedCtl> ctl(1, st);
    SVDAG_CUDA(cudaMemsetAsync(ctl.get(), 0, sizeof(RedCtl), st));
    a.slots = slots.get();
    a.slot_of = slot_of.get();
    a.cand = cand.get();
    a.state = state.get();
    a.newid = newid.get();
    a.bsum = bsum.get();
    a.inv = inv.get();
    a.var = var.get();
    a.left = left.get();
    a.cnt = ctl.get()->cnt;
    a.err = &ctl.get()->err;
    a.bar = &ctl.get()->bar;
    PhaseTrace trace(st);
    a.trace = trace.ptr();
    launch_persistent(ex, "k_sdag_persistent", k_sdag_persistent, grid, kRedThreads, 0, a);
    RedCtl h;
    try {
      h = finish_persistent(ex, ctl.get(), "toSDAG");
    } catch (const Error&) {
      // the parents were remapped in place: the octree must be rebuilt
      c.state = SVDAG_S_EMPTY;
      throw;
    }
    trace.report(ex, "toSDAG");
    for (uint32_t l = 1; l < L; ++l) {
      Level& V = c.lev[l];
      V.n = h.cnt[l];
      V.hdr = std::move(ohdr[l]);
      fit_buffer(V.hdr, V.n, st);
      V.inv = std::move(oinv[l]);
      fit_buffer(V.inv, V.n, st);
      if (l + 1 < L) {
        V.ch = std::move(och[l]);
        fit_buffer(V.ch, 8 * V.n, st);
      }
      nnodes += V.n;
    }
  }
  c.st.n_nodes_sdag = nnodes;
  c.st.n_nodes = nnodes;
  c.state = SVDAG_S_SDAG;
}

// ---------------------------------------------------------------------------
// toSDAG(internalCall, skipSymmetry = true) (src/symvox/geom_octree.cpp:
// 596-601, "pointer compression" only): per level, bottom-up, every
// non-empty node is kept in order with no invariance bits and no mirror
// lookups; the parents' pointers follow the kept nodes, and a pointer to a
// dropped empty node takes the reference's default correspondence (id 0, no
// mirror bits).  A DAG made by toDAG has no empty nodes, so there the pools
// stay as they are (one count per level, invariance bytes zeroed); imported
// pools and SVOs may have some, and are compacted (an SVO keeps its
// duplicates: the reference's skipSymmetry pass merges nothing).
namespace {

struct NonEmptyIn {
  const uint32_t* hdr;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return (hdr[i] & 0xFFu) ? 1u : 0u; }
};

__global__ void k_skip_compact(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                               const uint32_t* __restrict__ newidx, uint32_t* __restrict__ ohdr,
                               uint32_t* __restrict__ och) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    if (!(hdr[i] & 0xFFu)) continue;
    const uint32_t id = newidx[i];
    ohdr[id] = hdr[i];
    if (ch) {
      uint32_t c[8];
      load_children(ch, i, c);
      store_children(och, id, c);
    }
  }
}

// Parent pointers into a compacted level (child_hdr: its headers before).
__global__ void k_skip_remap(uint32_t* __restrict__ pch, uint64_t pn, const uint32_t* __restrict__ child_hdr,
                             const uint32_t* __restrict__ newidx) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < pn; p += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t c[8];
    load_children(pch, p, c);
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (c[j] != kNull) c[j] = (child_hdr[c[j]] & 0xFFu) ? newidx[c[j]] : 0u;
    store_children(pch, p, c);
  }
}

}  // namespace

void phase_reduce_sdag_skip_symmetry(Ctx& c) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toSDAG: the octree is not a DAG");
  // on an SVO (empty nodes and duplicates) the same rule: only the empty
  // nodes go; outside masks are numbered by the nodes before, and go too
  for (auto& V : c.lev) V.outm.release();
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;
  uint64_t nnodes = 0;
  for (uint32_t l = L > 0 ? L - 1 : 0; l >= 1; --l) {
    Level& V = c.lev[l];
    const uint64_t n = V.n;
    uint64_t kept = 0;
    if (n) {
      DBuf<uint32_t> newidx(n, st), d_cnt(1, st);
      device_exclusive_scan<uint32_t>(ex, NonEmptyIn{V.hdr.get()}, n, U32Out{newidx.get()}, d_cnt.get());
      kept = read_scalar(ex, d_cnt.get());
      if (kept != n) {
        const bool inner = l + 1 < L && V.ch.get();
        DBuf<uint32_t> ohdr(kept ? kept : 1, st), och;
        if (inner) och.alloc(8 * (kept ? kept : 1), st);
        SVDAG_LAUNCH(ex, k_skip_compact, grid_for(ex, n, 256), 256, 0, V.hdr.get(), inner ? V.ch.get() : nullptr, n,
                     newidx.get(), ohdr.get(), inner ? och.get() : nullptr);
        const Level& P = c.lev[l - 1];
        if (P.n && P.ch.get())
          SVDAG_LAUNCH(ex, k_skip_remap, grid_for(ex, P.n, 256), 256, 0, P.ch.get(), P.n, V.hdr.get(), newidx.get());
        V.hdr = std::move(ohdr);
        if (inner) V.ch = std::move(och);
        V.n = kept;
      }
    }
    V.inv.alloc(kept ? kept : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(V.inv.get(), 0, kept ? kept : 1, st));
    nnodes += kept;
  }
  c.st.n_nodes_sdag = nnodes;
  c.st.n_nodes = nnodes;
  c.state = SVDAG_S_SDAG;
}

// ---------------------------------------------------------------------------
// toDAG on caller-provided device scratch: the same kernels and the same
// result as phase_reduce_dag, with every temporary placed in `scratch` and
// each reduced level copied back to the front of its own buffers (a level
// only shrinks), so nothing is allocated.
//
// Scratch layout (offsets 256-byte aligned):
//   head [0, 4096):  error flag, level count, leaf first/rank/output tables
//   inner level of n nodes, from 4096:
//     A  max(8 * table slots, 32 n): hash table, then the compacted children
//     B  4 n: slot per node, then the compacted headers
//     rep, newid, corr: 4 n each;  tile sums and offsets of the scan
// Nothing has to be zero beforehand: the error flag, the hash table and the
// leaf first-occurrence table are cleared on the stream before their first
// read, on every call.
namespace {

constexpr uint64_t kHeadErr = 0, kHeadCnt = 64, kHeadFirst = 256, kHeadRank = 1280, kHeadLeafOut = 2304;
constexpr uint64_t kHeadBytes = 4096;

inline uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

struct InnerLayout {
  uint64_t slots, table, slot_of, rep, newid, corr, sums, offs, end;
};

InnerLayout inner_layout(uint64_t n) {
  InnerLayout L;
  const uint64_t m = n ? n : 1;
  const uint64_t nb = (m + kScanTile - 1) / kScanTile;
  L.slots = next_pow2(n < 16 ? 32 : 2 * n);
  L.table = kHeadBytes;
  L.slot_of = L.table + align256(std::max<uint64_t>(8 * L.slots, 32 * m));
  L.rep = L.slot_of + align256(4 * m);
  L.newid = L.rep + align256(4 * m);
  L.corr = L.newid + align256(4 * m);
  L.sums = L.corr + align256(4 * m);
  L.offs = L.sums + align256(4 * nb);
  L.end = L.offs + align256(4 * nb);
  return L;
}

// Exclusive scan with the tile sums and offsets in scratch (n <= kScanTile^2).
template <class T, class In, class Out>
void scan_in_scratch(const Exec& ex, In in, uint64_t n, Out out, T* d_total, T* sums, T* offs) {
  if (n == 0) {
    SVDAG_CUDA(cudaMemsetAsync(d_total, 0, sizeof(T), ex.stream));
    return;
  }
  const uint64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    SVDAG_LAUNCH(ex, (k_scan_tile_emit<T, In, Out>), 1, kScanThreads, 0, in, n, (const T*)nullptr, out, d_total);
    return;
  }
  SVDAG_LAUNCH(ex, (k_scan_tile_sums<T, In>), unsigned(nb), kScanThreads, 0, in, n, sums);
  SVDAG_LAUNCH(ex, (k_scan_tile_emit<T, ArrayIn<T>, ArrayOut<T>>), 1, kScanThreads, 0, ArrayIn<T>{sums}, nb,
               (const T*)nullptr, ArrayOut<T>{offs}, (T*)nullptr);
  SVDAG_LAUNCH(ex, (k_scan_tile_emit<T, In, Out>), unsigned(nb), kScanThreads, 0, in, n, (const T*)offs, out, d_total);
}

}  // namespace

void phase_reduce_dag_scratch(Ctx& c, uint8_t* scratch, uint64_t capacity) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toDAG: the octree is not an SVO or DAG");
  // every level is checked against the scratch before any work is queued,
  // so a rejected call leaves the octree untouched
  for (uint32_t lev = 1; lev + 1 < c.levels; ++lev) {
    const uint64_t n = c.lev[lev].n;
    const uint64_t need = inner_layout(n).end;
    if (need > capacity || (n + kScanTile - 1) / kScanTile > kScanTile)
      throw Error(SVDAG_ERR_OVERFLOW, "toDAG with static scratch: level " + std::to_string(lev) + " has " +
                                          std::to_string(n) + " nodes and needs " + std::to_string(need) +
                                          " bytes of scratch, above the " + std::to_string(capacity) +
                                          " bytes available (svdag_reduce_dag has no such limit)");
  }
  if (capacity < kHeadBytes) throw Error(SVDAG_ERR_OVERFLOW, "toDAG with static scratch: scratch too small");
  Exec ex = c.ex;
  ex.prof = nullptr;  // per-launch events would be created on demand
  const cudaStream_t st = c.stream;
  int* d_err = reinterpret_cast<int*>(scratch + kHeadErr);
  uint32_t* d_cnt = reinterpret_cast<uint32_t*>(scratch + kHeadCnt);
  SVDAG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  uint64_t nnodes = 1;
  for (uint32_t lev = c.levels - 1; lev > 0; --lev) {
    Level& L = c.lev[lev];
    Level& P = c.lev[lev - 1];
    const uint64_t n = L.n;
    if (lev == c.levels - 1) {
      uint32_t* first = reinterpret_cast<uint32_t*>(scratch + kHeadFirst);
      uint32_t* rank = reinterpret_cast<uint32_t*>(scratch + kHeadRank);
      uint32_t* out_hdr = reinterpret_cast<uint32_t*>(scratch + kHeadLeafOut);
      fill<uint32_t>(ex, first, 256, kNone);
      if (n) SVDAG_LAUNCH(ex, k_leaf_first, grid_for(ex, n, 256, 4), 256, 0, L.hdr.get(), n, first);
      SVDAG_LAUNCH(ex, k_leaf_rank, 1, 256, 0, first, rank, out_hdr, d_cnt);
      if (P.n)
        SVDAG_LAUNCH(ex, k_remap_parents_leafrank, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n,
                     L.hdr.get(), rank);
      const uint64_t d = read_scalar(ex, d_cnt);
      if (d) SVDAG_CUDA(cudaMemcpyAsync(L.hdr.get(), out_hdr, 4 * d, cudaMemcpyDeviceToDevice, st));
      L.n = d;
    } else {
      const InnerLayout Y = inner_layout(n);
      unsigned long long* slots = reinterpret_cast<unsigned long long*>(scratch + Y.table);
      uint32_t* slot_of = reinterpret_cast<uint32_t*>(scratch + Y.slot_of);
      uint32_t* rep = reinterpret_cast<uint32_t*>(scratch + Y.rep);
      uint32_t* newid = reinterpret_cast<uint32_t*>(scratch + Y.newid);
      uint32_t* corr = reinterpret_cast<uint32_t*>(scratch + Y.corr);
      SVDAG_CUDA(cudaMemsetAsync(slots, 0xFF, Y.slots * 8, st));
      const Table T{slots, Y.slots - 1};
      if (n) {
        SVDAG_LAUNCH(ex, k_insert, grid_for(ex, n, 256), 256, 0, T, L.hdr.get(), L.ch.get(), n, slot_of, d_err);
        SVDAG_LAUNCH(ex, k_rep, grid_for(ex, n, 256), 256, 0, T, slot_of, n, rep);
      }
      scan_in_scratch<uint32_t>(ex, RepFlagIn{rep}, n, U32Out{newid}, d_cnt, reinterpret_cast<uint32_t*>(scratch + Y.sums),
                                reinterpret_cast<uint32_t*>(scratch + Y.offs));
      const uint64_t d = read_scalar(ex, d_cnt);
      // the table and the slots are dead after k_rep: their space takes the compacted level
      uint32_t* out_ch = reinterpret_cast<uint32_t*>(scratch + Y.table);
      uint32_t* out_hdr = slot_of;
      if (n)
        SVDAG_LAUNCH(ex, k_compact_dag, grid_for(ex, n, 256), 256, 0, L.hdr.get(), L.ch.get(), n, rep, newid, out_hdr,
                     out_ch, corr);
      if (P.n)
        SVDAG_LAUNCH(ex, k_remap_parents, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n, corr);
      if (d) {
        SVDAG_CUDA(cudaMemcpyAsync(L.hdr.get(), out_hdr, 4 * d, cudaMemcpyDeviceToDevice, st));
        SVDAG_CUDA(cudaMemcpyAsync(L.ch.get(), out_ch, 32 * d, cudaMemcpyDeviceToDevice, st));
      }
      L.n = d;
    }
    nnodes += L.n;
  }
  try {
    check_err(ex, d_err, "toDAG");
  } catch (const Error&) {
    // the levels were compacted in place before the error was read: the
    // octree is no longer the SVO it was, and must be rebuilt
    c.state = SVDAG_S_EMPTY;
    throw;
  }
  c.st.n_nodes_dag = nnodes;
  c.st.n_nodes = nnodes;
  c.state = SVDAG_S_DAG;
}

}  // namespace svdag
