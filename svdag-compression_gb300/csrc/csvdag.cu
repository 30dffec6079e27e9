// GeomOctree::mergeAcrossAllLevels on the GPU
// (src/symvox/geom_octree_extension.cpp:1192-1544).
//
// The reference walks a "to check" set top-down (level 1 first).  A node A
// at level a is matched to the first node B (levels ascending, indices
// ascending, levels 1..a-1) whose top L-1-a levels equal A's subtree, as
// decided by compareSubtrees (geom_octree_extension.cpp:238-290); the hash
// multimap in front of it is only a shortlist that never drops an equal
// node.  A is then removed (corr = B, map assignment so it overwrites), and
// every node X below A gets corr = the node of B's subtree reached by the same
// child path, inserted with first-wins semantics across matches (processed
// in (level, index) order); within one comparison a node reached by several
// paths keeps its last visit, i.e. its lexicographically largest path.
// Unmatched checked nodes put their children into the next level's set.
// Finally levels are compacted bottom-up and every child pointer either
// follows the normal renumbering or is redirected to its corr node (level
// in childLevels); a redirect to a node that was itself removed stays
// 0xFFFFFFFF ("Missing correspondence", geom_octree_extension.cpp:1486-1491).
//
// GPU formulation.  Nodes get global indices g = off[level] + index, which
// order them exactly as the reference's (level, index) search.  For each
// height h = 0..L-2 every node at levels 1..L-1-h gets the class id TID_h =
// the smallest global index with the same truncated subtree of height h:
//   TID_0 = first node with the same mask,
//   TID_h = first node with the same (mask, TID_{h-1} of each child),
// computed with the shared hash table (min-index convergence).  The match of
// A at level a = L-1-h is TID_h(A) when it lies above level a.  The check set,
// the first-wins owner of every node (min over parents of the parent's owner
// or, for a matched root, the root itself) and the last-visit path (max over
// the owner's parents of path<<3|child) are then propagated level by level.
#include "ctx.cuh"
#include "dedup.cuh"

namespace svdag {
namespace {

struct TreeView {
  const uint32_t* const* hdr;  // [L] per-level hdr arrays
  const uint32_t* const* ch;   // [L] per-level child arrays (leaf entry unused)
  const uint32_t* off;         // [L+1] global offsets
  uint32_t L;
};

__device__ __forceinline__ uint32_t level_of(const TreeView& T, uint32_t g) {
  uint32_t lo = 0, hi = T.L;  // off[lo] <= g < off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&T.off[mid]) <= g) lo = mid; else hi = mid;
  }
  return lo;
}

#define GRID_STRIDE(i, n) \
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < (n); i += uint64_t(gridDim.x) * blockDim.x)

// TID_0: first global index per mask over levels 1..L-1.
__global__ void k_tid0_first(TreeView T, uint32_t g0, uint32_t g1, uint32_t* __restrict__ first) {
  __shared__ uint32_t sf[256];
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = kNone;
  __syncthreads();
  GRID_STRIDE(k, uint64_t(g1 - g0)) {
    const uint32_t g = g0 + uint32_t(k);
    const uint32_t l = level_of(T, g);
    const uint32_t m = T.hdr[l][g - T.off[l]] & 0xFFu;
    if (sf[m] > g) atomicMin(&sf[m], g);  // read first: common masks repeat
  }
  __syncthreads();
  for (int m = threadIdx.x; m < 256; m += blockDim.x)
    if (sf[m] != kNone) atomicMin(&first[m], sf[m]);
}

__global__ void k_tid0_assign(TreeView T, uint32_t g0, uint32_t g1, const uint32_t* __restrict__ first,
                              uint32_t* __restrict__ tid) {
  GRID_STRIDE(k, uint64_t(g1 - g0)) {
    const uint32_t g = g0 + uint32_t(k);
    const uint32_t l = level_of(T, g);
    tid[g] = first[T.hdr[l][g - T.off[l]] & 0xFFu];
  }
}

// Keys (mask, TID_{h-1} of each child) for nodes g in [g0, g1).
__global__ void k_tid_keys(TreeView T, uint32_t g0, uint32_t g1, const uint32_t* __restrict__ tid_prev,
                           uint32_t* __restrict__ khdr, uint32_t* __restrict__ kch) {
  GRID_STRIDE(k, uint64_t(g1 - g0)) {
    const uint32_t g = g0 + uint32_t(k);
    const uint32_t l = level_of(T, g);
    const uint32_t i = g - T.off[l];
    const uint32_t m = T.hdr[l][i] & 0xFFu;
    uint32_t c[8], o[8];
    load_children(T.ch[l], i, c);
    const uint32_t base = T.off[l + 1];
#pragma unroll
    for (int j = 0; j < 8; ++j) o[j] = ((m >> j) & 1u) ? tid_prev[base + c[j]] : kNull;
    khdr[k] = m;
    store_children(kch, k, o);
  }
}

// tid[g0 + k] = g0 + first occurrence of k's key.
__global__ void k_tid_assign(Table Tb, const uint32_t* __restrict__ slot_of, uint32_t g0, uint64_t n,
                             uint32_t* __restrict__ tid) {
  GRID_STRIDE(k, n) tid[g0 + k] = g0 + uint32_t(Tb.slots[slot_of[k]]);
}

// Match candidates of level a: the class representative when it lies above.
__global__ void k_candidates(const uint32_t* __restrict__ tid, uint32_t ga, uint32_t gb, uint32_t* __restrict__ cand) {
  GRID_STRIDE(k, uint64_t(gb - ga)) {
    const uint32_t g = ga + uint32_t(k);
    const uint32_t r = tid[g];
    cand[g] = (r < ga) ? r : kNone;
  }
}

// Check set of one level: matched nodes record their match; unmatched ones
// put their children into the next level's set (geom_octree_extension.cpp:1331-1407).
__global__ void k_check_level(TreeView T, uint32_t l, const uint32_t* __restrict__ cand, uint8_t* __restrict__ in_check,
                              uint32_t* __restrict__ own) {
  const uint32_t g0 = T.off[l], n = T.off[l + 1] - g0;
  GRID_STRIDE(i, uint64_t(n)) {
    const uint32_t g = g0 + uint32_t(i);
    if (!in_check[g]) continue;
    const uint32_t cd = cand[g];
    if (cd != kNone) { own[g] = cd; continue; }
    if (l + 1 >= T.L) continue;
    const uint32_t m = T.hdr[l][i] & 0xFFu;
    uint32_t c[8];
    load_children(T.ch[l], i, c);
    const uint32_t base = T.off[l + 1];
    // shared children are reached from many parents: write only a byte that
    // does not hold the mark yet (same-address stores serialise in L2)
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (((m >> j) & 1u) && !in_check[base + c[j]]) in_check[base + c[j]] = 1;
  }
}

// eff(P): the first match whose subtree holds P's children through P.
__device__ __forceinline__ uint32_t eff_of(uint32_t g, const uint32_t* owner, const uint32_t* own) {
  const uint32_t o = owner[g];
  if (o != kNone) return o;
  return (own[g] != kNone) ? g : kNone;
}

__global__ void k_owner_min(TreeView T, uint32_t l, const uint32_t* __restrict__ own, uint32_t* owner) {
  const uint32_t g0 = T.off[l], n = T.off[l + 1] - g0;
  GRID_STRIDE(i, uint64_t(n)) {
    const uint32_t g = g0 + uint32_t(i);
    const uint32_t e = eff_of(g, owner, own);
    if (e == kNone) continue;
    const uint32_t m = T.hdr[l][i] & 0xFFu;
    uint32_t c[8];
    load_children(T.ch[l], i, c);
    const uint32_t base = T.off[l + 1];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (((m >> j) & 1u) && __ldcg(&owner[base + c[j]]) > e) atomicMin(&owner[base + c[j]], e);
  }
}

__global__ void k_owner_path(TreeView T, uint32_t l, const uint32_t* __restrict__ own, const uint32_t* owner,
                             const unsigned long long* path, unsigned long long* best) {
  const uint32_t g0 = T.off[l], n = T.off[l + 1] - g0;
  GRID_STRIDE(i, uint64_t(n)) {
    const uint32_t g = g0 + uint32_t(i);
    const uint32_t e = eff_of(g, owner, own);
    if (e == kNone) continue;
    const unsigned long long pp = (owner[g] != kNone) ? path[g] : 0ull;
    const uint32_t m = T.hdr[l][i] & 0xFFu;
    uint32_t c[8];
    load_children(T.ch[l], i, c);
    const uint32_t base = T.off[l + 1];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) {
        const uint32_t x = base + c[j];
        const unsigned long long v = (pp << 3) | uint32_t(j);
        if (owner[x] == e && __ldcg(&best[x]) < v) atomicMax(&best[x], v);
      }
  }
}

__global__ void k_owner_bdesc(TreeView T, uint32_t l, const uint32_t* __restrict__ own, const uint32_t* owner,
                              unsigned long long* path, const unsigned long long* __restrict__ best, uint32_t* bdesc) {
  const uint32_t g0 = T.off[l], n = T.off[l + 1] - g0;
  GRID_STRIDE(i, uint64_t(n)) {
    const uint32_t g = g0 + uint32_t(i);
    const uint32_t e = eff_of(g, owner, own);
    if (e == kNone) continue;
    const bool owned = owner[g] != kNone;
    const unsigned long long pp = owned ? path[g] : 0ull;
    const uint32_t bp = owned ? bdesc[g] : own[g];  // B-side node of P
    const uint32_t m = T.hdr[l][i] & 0xFFu;
    uint32_t c[8];
    load_children(T.ch[l], i, c);
    const uint32_t base = T.off[l + 1];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) {
        const uint32_t x = base + c[j];
        const unsigned long long pk = (pp << 3) | uint32_t(j);
        if (owner[x] == e && best[x] == pk) {
          const uint32_t lb = level_of(T, bp);
          const uint32_t bc = T.ch[lb][8ull * (bp - T.off[lb]) + j];
          bdesc[x] = T.off[lb + 1] + bc;
          path[x] = pk;
        }
      }
  }
}

// corr = own match (overwrites) else the owner's B-side node.
__global__ void k_corr(uint32_t n, const uint32_t* __restrict__ own, const uint32_t* __restrict__ owner,
                       const uint32_t* __restrict__ bdesc, uint32_t* __restrict__ corr) {
  GRID_STRIDE(g, uint64_t(n)) {
    const uint32_t o = own[g];
    corr[g] = (o != kNone) ? o : ((owner[g] != kNone) ? bdesc[g] : kNone);
  }
}

struct KeepIn {
  const uint32_t* corr;
  __device__ __forceinline__ uint32_t operator()(uint64_t g) const { return corr[g] == kNone ? 1u : 0u; }
};
struct U32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};

// newidx[g] = rank of g among the kept nodes of its level, kNone if removed.
__global__ void k_newidx(TreeView T, uint32_t n, const uint32_t* __restrict__ corr, const uint32_t* __restrict__ prefix,
                         uint32_t* __restrict__ newidx) {
  GRID_STRIDE(g, uint64_t(n)) {
    const uint32_t l = level_of(T, uint32_t(g));
    newidx[g] = (corr[g] == kNone) ? prefix[g] - prefix[T.off[l]] : kNone;
  }
}

// Compacted level l with rewritten children and child levels.
__global__ void k_emit_level(TreeView T, uint32_t l, const uint32_t* __restrict__ corr, const uint32_t* __restrict__ newidx,
                             uint32_t* __restrict__ ohdr, uint32_t* __restrict__ och, uint8_t* __restrict__ oclev,
                             unsigned long long* missing) {
  const uint32_t g0 = T.off[l], n = T.off[l + 1] - g0;
  const bool inner = (l + 1 < T.L);
  GRID_STRIDE(i, uint64_t(n)) {
    const uint32_t g = g0 + uint32_t(i);
    if (corr[g] != kNone) continue;
    const uint32_t id = newidx[g];
    const uint32_t h = T.hdr[l][i];
    ohdr[id] = h;
    uint8_t cl[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) cl[j] = uint8_t(l + 1);
    if (inner) {
      const uint32_t m = h & 0xFFu;
      uint32_t c[8];
      load_children(T.ch[l], i, c);
      const uint32_t base = T.off[l + 1];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (!((m >> j) & 1u)) continue;
        const uint32_t x = base + c[j];
        const uint32_t t = corr[x];
        if (t != kNone) {
          cl[j] = uint8_t(level_of(T, t));
          c[j] = newidx[t];
          if (c[j] == kNone) atomicAdd(missing, 1ull);
        } else {
          c[j] = newidx[x];
        }
      }
      store_children(och, id, c);
    }
    uint2 packed;
    packed.x = uint32_t(cl[0]) | (uint32_t(cl[1]) << 8) | (uint32_t(cl[2]) << 16) | (uint32_t(cl[3]) << 24);
    packed.y = uint32_t(cl[4]) | (uint32_t(cl[5]) << 8) | (uint32_t(cl[6]) << 16) | (uint32_t(cl[7]) << 24);
    reinterpret_cast<uint2*>(oclev)[id] = packed;
  }
}

}  // namespace

void phase_cross_level_merge(Ctx& c) {
  if (c.state != SVDAG_S_DAG) throw Error(SVDAG_ERR_INVALID_STATE, "mergeAcrossAllLevels: the octree is not a DAG");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;

  // global offsets and per-level pointer tables
  std::vector<uint32_t> off(L + 1, 0);
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t o = uint64_t(off[l]) + c.lev[l].n;
    if (o >= 0xFFFFFFF0ull) throw Error(SVDAG_ERR_OVERFLOW, "mergeAcrossAllLevels: more than 2^32 nodes");
    off[l + 1] = uint32_t(o);
  }
  const uint32_t N = off[L];
  std::vector<const uint32_t*> hp(L), cp(L);
  for (uint32_t l = 0; l < L; ++l) { hp[l] = c.lev[l].hdr.get(); cp[l] = c.lev[l].ch.get(); }
  DBuf<uint32_t> d_off(L + 1, st);
  DBuf<const uint32_t*> d_hp(L, st), d_cp(L, st);
  SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), off.data(), 4 * (L + 1), cudaMemcpyHostToDevice, st));
  SVDAG_CUDA(cudaMemcpyAsync(d_hp.get(), hp.data(), sizeof(void*) * L, cudaMemcpyHostToDevice, st));
  SVDAG_CUDA(cudaMemcpyAsync(d_cp.get(), cp.data(), sizeof(void*) * L, cudaMemcpyHostToDevice, st));
  TreeView T{d_hp.get(), d_cp.get(), d_off.get(), L};

  DBuf<uint32_t> cand(N ? N : 1, st), own(N ? N : 1, st), owner(N ? N : 1, st), bdesc(N ? N : 1, st);
  fill<uint32_t>(ex, cand.get(), N, kNone);
  fill<uint32_t>(ex, own.get(), N, kNone);
  fill<uint32_t>(ex, owner.get(), N, kNone);

  if (L >= 3) {
    // ---- truncated-subtree class ids, h = 0 .. L-2
    DBuf<uint32_t> tid_a(N, st), tid_b(N, st);
    uint32_t* tid_prev = tid_a.get();
    uint32_t* tid_cur = tid_b.get();
    DBuf<int> d_err(1, st);
    SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, st));
    {
      DBuf<uint32_t> first(256, st);
      fill<uint32_t>(ex, first.get(), 256, kNone);
      const uint32_t g0 = off[1], g1 = off[L];
      SVDAG_LAUNCH(ex, k_tid0_first, grid_for(ex, g1 - g0, 256, 4), 256, 0, T, g0, g1, first.get());
      SVDAG_LAUNCH(ex, k_tid0_assign, grid_for(ex, g1 - g0, 256), 256, 0, T, g0, g1, first.get(), tid_prev);
      const uint32_t a = L - 1;
      SVDAG_LAUNCH(ex, k_candidates, grid_for(ex, off[a + 1] - off[a], 256), 256, 0, tid_prev, off[a], off[a + 1],
                   cand.get());
    }
    for (uint32_t h = 1; h + 1 < L; ++h) {
      const uint32_t a = L - 1 - h;  // deepest level of the domain; A-level of this height
      const uint32_t g0 = off[1], g1 = off[a + 1];
      const uint64_t n = g1 - g0;
      if (n == 0) continue;
      DBuf<uint32_t> khdr(n, st), kch(8 * n, st), slot_of(n, st);
      SVDAG_LAUNCH(ex, k_tid_keys, grid_for(ex, n, 256), 256, 0, T, g0, g1, tid_prev, khdr.get(), kch.get());
      DBuf<unsigned long long> tb;
      Table Tb = make_table(ex, n, tb);
      SVDAG_LAUNCH(ex, k_insert, grid_for(ex, n, 256), 256, 0, Tb, khdr.get(), kch.get(), n, slot_of.get(), d_err.get());
      SVDAG_LAUNCH(ex, k_tid_assign, grid_for(ex, n, 256), 256, 0, Tb, slot_of.get(), g0, n, tid_cur);
      SVDAG_LAUNCH(ex, k_candidates, grid_for(ex, off[a + 1] - off[a], 256), 256, 0, tid_cur, off[a], off[a + 1],
                   cand.get());
      std::swap(tid_prev, tid_cur);
    }
    check_err(ex, d_err.get(), "mergeAcrossAllLevels");
  }

  // ---- check set, top-down from level 1
  DBuf<uint8_t> in_check(N ? N : 1, st);
  SVDAG_CUDA(cudaMemsetAsync(in_check.get(), 0, N ? N : 1, st));
  if (L >= 2) {
    SVDAG_CUDA(cudaMemsetAsync(in_check.get() + off[1], 1, off[2] - off[1], st));
    for (uint32_t l = 1; l < L; ++l) {
      const uint32_t n = off[l + 1] - off[l];
      if (n) SVDAG_LAUNCH(ex, k_check_level, grid_for(ex, n, 256), 256, 0, T, l, cand.get(), in_check.get(), own.get());
    }
  }

  // ---- owners, last-visit paths and B-side nodes, top-down
  DBuf<unsigned long long> path(N ? N : 1, st), best(N ? N : 1, st);
  SVDAG_CUDA(cudaMemsetAsync(best.get(), 0, 8 * (N ? N : 1), st));
  for (uint32_t l = 1; l + 1 < L; ++l) {  // parents at l, children at l+1
    const uint32_t n = off[l + 1] - off[l];
    if (!n) continue;
    const unsigned gr = grid_for(ex, n, 256);
    SVDAG_LAUNCH(ex, k_owner_min, gr, 256, 0, T, l, own.get(), owner.get());
    SVDAG_LAUNCH(ex, k_owner_path, gr, 256, 0, T, l, own.get(), owner.get(), path.get(), best.get());
    SVDAG_LAUNCH(ex, k_owner_bdesc, gr, 256, 0, T, l, own.get(), owner.get(), path.get(), best.get(), bdesc.get());
  }
  path.release();
  best.release();

  // ---- compaction
  DBuf<uint32_t> corr(N ? N : 1, st), prefix(N ? N : 1, st), newidx(N ? N : 1, st);
  SVDAG_LAUNCH(ex, k_corr, grid_for(ex, N, 256), 256, 0, N, own.get(), owner.get(), bdesc.get(), corr.get());
  std::vector<uint32_t> pre(L + 1);
  {
    // kept counts per level from the prefix at each level start (+ total)
    DBuf<uint32_t> d_tot(1, st);
    device_exclusive_scan<uint32_t>(ex, KeepIn{corr.get()}, N, U32Out{prefix.get()}, d_tot.get());
    SVDAG_LAUNCH(ex, k_newidx, grid_for(ex, N, 256), 256, 0, T, N, corr.get(), prefix.get(), newidx.get());
    for (uint32_t l = 0; l < L; ++l) {
      if (off[l] < N) SVDAG_CUDA(cudaMemcpyAsync(&pre[l], prefix.get() + off[l], 4, cudaMemcpyDeviceToHost, st));
      else pre[l] = 0;
    }
    SVDAG_CUDA(cudaMemcpyAsync(&pre[L], d_tot.get(), 4, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
    for (uint32_t l = 0; l < L; ++l)
      if (off[l] >= N) pre[l] = pre[L];
  }
  DBuf<unsigned long long> d_missing(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_missing.get(), 0, 8, st));
  std::vector<Level> out(L);
  uint64_t kept_total = 0;
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t kept = uint64_t(pre[l + 1]) - pre[l];
    out[l].n = kept;
    out[l].hdr.alloc(kept ? kept : 1, st);
    if (l + 1 < L) out[l].ch.alloc(8 * (kept ? kept : 1), st);
    out[l].clev.alloc(8 * (kept ? kept : 1), st);
    const uint32_t n = off[l + 1] - off[l];
    if (n)
      SVDAG_LAUNCH(ex, k_emit_level, grid_for(ex, n, 256), 256, 0, T, l, corr.get(), newidx.get(), out[l].hdr.get(),
                   out[l].ch.get(), out[l].clev.get(), d_missing.get());
    if (l > 0) kept_total += kept;
  }
  const uint64_t missing = read_scalar(ex, d_missing.get());
  for (uint32_t l = 0; l < L; ++l) c.lev[l] = std::move(out[l]);
  c.st.n_nodes = 1 + kept_total;
  c.st.n_nodes_dag = 1 + kept_total;
  c.st.n_cross_level_merged = uint64_t(N - 1) - kept_total;
  c.st.n_missing_correspondences = missing;
  c.child_levels_init = true;
}

}  // namespace svdag
