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
// decided once every earlier-ordered candidate is decided; rounds over the
// undecided nodes resolve the dependency chains (the lowest undecided index
// always resolves, so rounds terminate) and give exactly the sequential
// result.
#include <algorithm>

#include "ctx.cuh"
#include "dedup.cuh"

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

// Invariance bits, the 7 normalised variants and their candidates.
__global__ void k_sdag_candidates(Table T, const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                                  const uint32_t* __restrict__ slot_of, const uint8_t* __restrict__ child_inv,
                                  uint8_t* __restrict__ inv, uint32_t* __restrict__ cand) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t h, c[8];
    load_key(hdr, ch, i, h, c);
    const uint32_t s = slot_of[i];
    cand[i] = (s == kNone) ? kNone : uint32_t(T.slots[s]);
    // invariance on X, Y, Z (geom_octree.cpp:604-606): n == n.mirror(axis)
    uint32_t iv = 0;
    {
      uint32_t mh, mc[8];
      mirror_node(h, c, 4, mh, mc); if (same_key(h, c, mh, mc)) iv |= 1u;
      mirror_node(h, c, 2, mh, mc); if (same_key(h, c, mh, mc)) iv |= 2u;
      mirror_node(h, c, 1, mh, mc); if (same_key(h, c, mh, mc)) iv |= 4u;
    }
    inv[i] = uint8_t(iv);
    uint32_t cinv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) cinv[k] = (child_inv && c[k] != kNull) ? child_inv[c[k]] : 0u;
    for (int v = 1; v < 8; ++v) {
      const int flip = kVarFlip[v];
      uint32_t vh, vc[8];
      mirror_node(h, c, flip, vh, vc);
      if (child_inv) {
        // invertInvs (geom_octree.cpp:822-831): drop the mirror bit of an axis
        // of this variant when the child is invariant on it
        uint32_t clrx = 0, clry = 0, clrz = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (vc[k] == kNull) continue;
          const uint32_t ci = cinv[k ^ flip];
          if ((flip & 4) && (ci & 1u)) clrx |= 1u << k;
          if ((flip & 2) && (ci & 2u)) clry |= 1u << k;
          if ((flip & 1) && (ci & 4u)) clrz |= 1u << k;
        }
        vh &= ~((clrx << 8) | (clry << 16) | (clrz << 24));
      }
      cand[uint64_t(v) * n + i] = table_find(T, hdr, ch, vh, vc);
    }
  }
}

// One resolution round over undecided nodes (see file comment).
__global__ void k_sdag_round(const uint32_t* __restrict__ cand, uint64_t n, uint32_t* state, uint8_t* __restrict__ var,
                             unsigned long long* undecided) {
  unsigned long long left = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    if (ld_cg32(&state[i]) != kUndecided) continue;
    bool stuck = false, done = false;
    for (int k = 0; k < 8; ++k) {
      const uint32_t cnd = cand[uint64_t(k) * n + i];
      if (cnd == kNone || cnd >= uint32_t(i)) continue;
      const uint32_t s = ld_cg32(&state[cnd]);
      if (s == kUndecided) { stuck = true; break; }
      if (s == kUnique) {
        var[i] = uint8_t(k);
        __stcg(&state[i], cnd);
        done = true;
        break;
      }
    }
    if (!stuck && !done) __stcg(&state[i], kUnique);
    if (stuck) ++left;
  }
  for (int o = 16; o; o >>= 1) left += __shfl_down_sync(0xFFFFFFFFu, left, o);
  if ((threadIdx.x & 31) == 0 && left) atomicAdd(undecided, left);
}

// Sequential fallback for long dependency chains: one thread, index order.
__global__ void k_sdag_serial(const uint32_t* __restrict__ cand, uint64_t n, uint32_t* state, uint8_t* var) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (uint64_t i = 0; i < n; ++i) {
    if (state[i] != kUndecided) continue;
    bool done = false;
    for (int k = 0; k < 8 && !done; ++k) {
      const uint32_t cnd = cand[uint64_t(k) * n + i];
      if (cnd == kNone || cnd >= uint32_t(i)) continue;
      if (state[cnd] == kUnique) { var[i] = uint8_t(k); state[i] = cnd; done = true; }
    }
    if (!done) state[i] = kUnique;
  }
}

struct UniqueFlagIn {
  const uint32_t* state;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return state[i] == kUnique ? 1u : 0u; }
};

__global__ void k_compact_sdag(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, const uint8_t* __restrict__ inv,
                               uint64_t n, const uint32_t* __restrict__ state, const uint8_t* __restrict__ var,
                               const uint32_t* __restrict__ newid, uint32_t* __restrict__ out_hdr, uint32_t* __restrict__ out_ch,
                               uint8_t* __restrict__ out_inv, uint32_t* __restrict__ corr_id, uint8_t* __restrict__ corr_m) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t s = state[i];
    if (s == kUnique) {
      const uint32_t id = newid[i];
      corr_id[i] = id;
      corr_m[i] = 0;
      out_hdr[id] = hdr[i];
      out_inv[id] = inv[i];
      if (ch) {
        uint32_t c[8];
        load_children(ch, i, c);
        store_children(out_ch, id, c);
      }
    } else {
      corr_id[i] = newid[s];
      corr_m[i] = kVarAxes[var[i]];
    }
  }
}

// Parents at level lev-1: children with a pointer -> (id, mirror bits).
__global__ void k_remap_parents_sdag(uint32_t* __restrict__ phdr, uint32_t* __restrict__ pch, uint64_t np,
                                     const uint32_t* __restrict__ corr_id, const uint8_t* __restrict__ corr_m) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t c[8];
    load_children(pch, p, c);
    uint32_t mx = 0, my = 0, mz = 0;
    bool any = false;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (c[j] == kNull) continue;
      any = true;
      const uint32_t old = c[j];
      const uint32_t m = corr_m[old];
      c[j] = corr_id[old];
      if (m & 1u) mx |= 1u << j;
      if (m & 2u) my |= 1u << j;
      if (m & 4u) mz |= 1u << j;
    }
    if (!any) continue;
    store_children(pch, p, c);
    if (mx | my | mz) phdr[p] |= (mx << 8) | (my << 16) | (mz << 24);
  }
}

}  // namespace

void phase_reduce_dag(Ctx& c) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toDAG: the octree is not an SVO or DAG");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  DBuf<int> d_err(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, st));
  DBuf<uint32_t> d_cnt(1, st);
  uint64_t nnodes = 1;
  for (uint32_t lev = c.levels - 1; lev > 0; --lev) {
    Level& L = c.lev[lev];
    Level& P = c.lev[lev - 1];
    const uint64_t n = L.n;
    if (lev == c.levels - 1) {
      DBuf<uint32_t> first(256, st), rank(256, st);
      fill<uint32_t>(ex, first.get(), 256, kNone);
      DBuf<uint32_t> out_hdr(256, st);
      if (n) SVDAG_LAUNCH(ex, k_leaf_first, grid_for(ex, n, 256, 4), 256, 0, L.hdr.get(), n, first.get());
      SVDAG_LAUNCH(ex, k_leaf_rank, 1, 256, 0, first.get(), rank.get(), out_hdr.get(), d_cnt.get());
      if (P.n)
        SVDAG_LAUNCH(ex, k_remap_parents_leafrank, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n,
                     L.hdr.get(), rank.get());
      const uint64_t d = read_scalar(ex, d_cnt.get());
      L.hdr = std::move(out_hdr);
      L.n = d;
    } else {
      DBuf<unsigned long long> tb;
      Table T = make_table(ex, n, tb);
      DBuf<uint32_t> slot_of(n ? n : 1, st), rep(n ? n : 1, st), newid(n ? n : 1, st), corr(n ? n : 1, st);
      if (n) {
        SVDAG_LAUNCH(ex, k_insert, grid_for(ex, n, 256), 256, 0, T, L.hdr.get(), L.ch.get(), n, slot_of.get(), d_err.get());
        SVDAG_LAUNCH(ex, k_rep, grid_for(ex, n, 256), 256, 0, T, slot_of.get(), n, rep.get());
      }
      tb.release();
      slot_of.release();
      device_exclusive_scan<uint32_t>(ex, RepFlagIn{rep.get()}, n, U32Out{newid.get()}, d_cnt.get());
      const uint64_t d = read_scalar(ex, d_cnt.get());
      DBuf<uint32_t> out_hdr(d ? d : 1, st), out_ch(8 * (d ? d : 1), st);
      if (n)
        SVDAG_LAUNCH(ex, k_compact_dag, grid_for(ex, n, 256), 256, 0, L.hdr.get(), L.ch.get(), n, rep.get(),
                     newid.get(), out_hdr.get(), out_ch.get(), corr.get());
      if (P.n)
        SVDAG_LAUNCH(ex, k_remap_parents, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n, corr.get());
      L.hdr = std::move(out_hdr);
      L.ch = std::move(out_ch);
      L.n = d;
    }
    nnodes += L.n;
  }
  check_err(ex, d_err.get(), "toDAG");
  c.st.n_nodes_dag = nnodes;
  c.st.n_nodes = nnodes;
  c.state = SVDAG_S_DAG;
}

void phase_reduce_sdag(Ctx& c) {
  if (c.state != SVDAG_S_SVO && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "toSDAG: the octree is not a DAG");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  DBuf<int> d_err(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, st));
  DBuf<uint32_t> d_cnt(1, st);
  DBuf<unsigned long long> d_left(1, st);
  uint64_t nnodes = 0;
  const uint8_t* child_inv = nullptr;
  for (uint32_t lev = c.levels - 1; lev > 0; --lev) {
    Level& L = c.lev[lev];
    Level& P = c.lev[lev - 1];
    const uint64_t n = L.n;
    if (c.state == SVDAG_S_SVO) {
      // an SVO level may hold empty nodes; toSDAG skips them like toDAG
      throw Error(SVDAG_ERR_INVALID_STATE, "toSDAG on an SVO: run toDAG first");
    }
    DBuf<unsigned long long> tb;
    Table T = make_table(ex, n, tb);
    DBuf<uint32_t> slot_of(n ? n : 1, st), cand(8 * (n ? n : 1), st), state(n ? n : 1, st), newid(n ? n : 1, st);
    DBuf<uint8_t> inv(n ? n : 1, st), var(n ? n : 1, st);
    const uint32_t* ch = (lev == c.levels - 1) ? nullptr : L.ch.get();
    if (n) {
      SVDAG_LAUNCH(ex, k_insert, grid_for(ex, n, 256), 256, 0, T, L.hdr.get(), ch, n, slot_of.get(), d_err.get());
      SVDAG_LAUNCH(ex, k_sdag_candidates, grid_for(ex, n, 256), 256, 0, T, L.hdr.get(), ch, n, slot_of.get(),
                   child_inv, inv.get(), cand.get());
      fill<uint32_t>(ex, state.get(), n, kUndecided);
      // rounds in groups of 4 between host reads (a round with nothing left
      // is a no-op), at most 64 before the serial finish
      int rounds = 0;
      for (;;) {
        for (int r = 0; r < 4; ++r) {
          SVDAG_CUDA(cudaMemsetAsync(d_left.get(), 0, 8, st));
          SVDAG_LAUNCH(ex, k_sdag_round, grid_for(ex, n, 256), 256, 0, cand.get(), n, state.get(), var.get(),
                       d_left.get());
        }
        rounds += 4;
        if (read_scalar(ex, d_left.get()) == 0) break;
        if (rounds >= 64) {
          SVDAG_LAUNCH(ex, k_sdag_serial, 1, 32, 0, cand.get(), n, state.get(), var.get());
          break;
        }
      }
    }
    tb.release();
    slot_of.release();
    device_exclusive_scan<uint32_t>(ex, UniqueFlagIn{state.get()}, n, U32Out{newid.get()}, d_cnt.get());
    const uint64_t s = read_scalar(ex, d_cnt.get());
    DBuf<uint32_t> out_hdr(s ? s : 1, st), out_ch(ch ? 8 * (s ? s : 1) : 0, st), corr_id(n ? n : 1, st);
    DBuf<uint8_t> out_inv(s ? s : 1, st), corr_m(n ? n : 1, st);
    if (n)
      SVDAG_LAUNCH(ex, k_compact_sdag, grid_for(ex, n, 256), 256, 0, L.hdr.get(), ch, inv.get(), n, state.get(),
                   var.get(), newid.get(), out_hdr.get(), out_ch.get(), out_inv.get(), corr_id.get(), corr_m.get());
    if (P.n)
      SVDAG_LAUNCH(ex, k_remap_parents_sdag, grid_for(ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n,
                   corr_id.get(), corr_m.get());
    L.hdr = std::move(out_hdr);
    if (ch) L.ch = std::move(out_ch);
    L.inv = std::move(out_inv);
    L.n = s;
    child_inv = L.inv.get();
    nnodes += s;
  }
  check_err(ex, d_err.get(), "toSDAG");
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
