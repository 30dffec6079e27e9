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
// All of it runs as one persistent cooperative kernel (k_csv_persistent) with
// grid barriers between the steps and one read of the kept counts at the end.
#include "ctx.cuh"
#include "dedup.cuh"
#include "persist.cuh"

namespace svdag {
namespace {

// Arguments of the persistent merge: the DAG's levels (read only), scratch
// over the N nodes' global indices, and the compacted output levels
// (capacity = each level's input count).
struct CsvArgs {
  const uint32_t* hdr[kMaxRedLevels];
  const uint32_t* ch[kMaxRedLevels];
  uint32_t* ohdr[kMaxRedLevels];
  uint32_t* och[kMaxRedLevels];
  uint8_t* oclev[kMaxRedLevels];
  uint32_t off[kMaxRedLevels + 1];  // global offsets
  uint32_t L, N;
  unsigned long long* slots;  // hash table sized for the largest height's domain
  uint32_t* tid_a;            // class ids of two consecutive heights
  uint32_t* tid_b;
  uint32_t* khdr;             // keys (mask, child class ids) of one height
  uint32_t* kch;
  uint32_t* slot_of;
  uint32_t* first;            // [256]
  uint32_t* cand;             // match candidate per node
  uint32_t* own;              // match of a checked node
  uint32_t* owner;            // first-wins owner
  uint32_t* bdesc;            // B-side node reached by the owner's path
  uint32_t* corr;
  uint32_t* prefix;
  uint32_t* newidx;
  uint32_t* bsum;
  uint32_t* check_bits;       // check set over the global indices
  uint32_t smem_words;        // words of the shared-memory bitmap
  unsigned long long* path;
  unsigned long long* best;
  unsigned long long* missing;
  uint32_t* cnt;  // [L] kept nodes per level
  int* err;
  GridBar* bar;
  unsigned long long* trace;  // step trace or null
};

__device__ __forceinline__ uint32_t level_of(const CsvArgs& a, uint32_t g) {
  uint32_t lo = 0, hi = a.L;  // off[lo] <= g < off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a.off[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint64_t slots_for(uint64_t n) {
  const uint64_t want = n < 16 ? 32 : 2 * n;
  return uint64_t(1) << (64 - __clzll(want - 1));
}

// eff(P): the first match whose subtree holds P's children through P.
__device__ __forceinline__ uint32_t eff_of(const CsvArgs& a, uint32_t g) {
  const uint32_t o = a.owner[g];
  if (o != kNone) return o;
  return (a.own[g] != kNone) ? g : kNone;
}

__global__ void __launch_bounds__(kRedThreads, 1) k_csv_persistent(const CsvArgs a) {
  __shared__ uint32_t sf[256];
  extern __shared__ uint32_t s_bits[];  // a.smem_words words
  const uint32_t L = a.L, N = a.N;
  unsigned trace_pos = 0;
  trace_mark(a.trace, trace_pos, kStEntry);
  // prologue: tables cleared, level 1 in the check set
  SVDAG_GRID_STRIDE(g, uint64_t(N)) {
    a.cand[g] = kNone;
    a.own[g] = kNone;
    a.owner[g] = kNone;
    a.best[g] = 0ull;
  }
  {
    // check set: level 1
    const uint32_t lo = L >= 2 ? a.off[1] : 0, hi = L >= 2 ? a.off[2] : 0;
    SVDAG_GRID_STRIDE(w, uint64_t((N + 31) >> 5)) {
      const uint32_t b0 = uint32_t(w) << 5;
      uint32_t v = 0;
      for (uint32_t k = 0; k < 32; ++k) v |= uint32_t(b0 + k >= lo && b0 + k < hi) << k;
      a.check_bits[w] = v;
    }
  }
  if (blockIdx.x == 0) {
    for (int m = threadIdx.x; m < 256; m += blockDim.x) a.first[m] = kNone;
    if (threadIdx.x == 0) *a.missing = 0ull;
  }
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = kNone;
  SVDAG_STEP(a, 0, kStPrologue);

  // ---- truncated-subtree class ids, h = 0 .. L-2
  uint32_t* tid_prev = a.tid_a;
  uint32_t* tid_cur = a.tid_b;
  if (L >= 3) {
    const uint32_t g0 = a.off[1], g1 = a.off[L];
    // TID_0: first global index per mask over levels 1..L-1
    __syncthreads();
    SVDAG_GRID_STRIDE(k, uint64_t(g1 - g0)) {
      const uint32_t g = g0 + uint32_t(k);
      const uint32_t l = level_of(a, g);
      const uint32_t m = a.hdr[l][g - a.off[l]] & 0xFFu;
      if (sf[m] > g) atomicMin(&sf[m], g);  // read first: common masks repeat
    }
    __syncthreads();
    for (int m = threadIdx.x; m < 256; m += blockDim.x)
      if (sf[m] != kNone) atomicMin(&a.first[m], sf[m]);
    SVDAG_STEP(a, 0, kStTid0First);
    const uint32_t la = L - 1;
    SVDAG_GRID_STRIDE(k, uint64_t(g1 - g0)) {
      const uint32_t g = g0 + uint32_t(k);
      const uint32_t l = level_of(a, g);
      const uint32_t t = a.first[a.hdr[l][g - a.off[l]] & 0xFFu];
      tid_prev[g] = t;
      // match candidates of level L-1: the class representative when it lies above
      if (l == la) a.cand[g] = (t < a.off[la]) ? t : kNone;
    }
    SVDAG_STEP(a, 0, kStTid0Assign);
    for (uint32_t h = 1; h + 1 < L; ++h) {
      const uint32_t la = L - 1 - h;  // deepest level of the domain; A-level of this height
      const uint32_t d1 = a.off[la + 1];
      const uint64_t n = d1 - g0;
      if (n == 0) continue;
      const Table T{a.slots, slots_for(n) - 1};
      // keys (mask, TID_{h-1} of each child); the table cleared
      SVDAG_GRID_STRIDE(k, n) {
        const uint32_t g = g0 + uint32_t(k);
        const uint32_t l = level_of(a, g);
        const uint32_t i = g - a.off[l];
        const uint32_t m = a.hdr[l][i] & 0xFFu;
        uint32_t c[8], o[8];
        load_children(a.ch[l], i, c);
        const uint32_t base = a.off[l + 1];
#pragma unroll
        for (int j = 0; j < 8; ++j) o[j] = ((m >> j) & 1u) ? tid_prev[base + c[j]] : kNull;
        a.khdr[k] = m;
        store_children(a.kch, k, o);
      }
      clear_slots(a.slots, T.mask + 1);
      SVDAG_STEP(a, h, kStKeys);
      SVDAG_GRID_STRIDE(k, n) {
        uint32_t hh, c[8];
        load_key(a.khdr, a.kch, k, hh, c);
        if ((hh & 0xFFu) == 0) { a.slot_of[k] = kNone; continue; }
        a.slot_of[k] = uint32_t(table_insert(T, a.khdr, a.kch, uint32_t(k), hh, c, a.err));
      }
      SVDAG_STEP(a, h, kStInsert);
      // TID_h = g0 + first occurrence of the key; candidates of level la
      SVDAG_GRID_STRIDE(k, n) {
        const uint32_t s = a.slot_of[k];
        const uint32_t g = g0 + uint32_t(k);
        const uint32_t t = (s == kNone) ? g : g0 + uint32_t(a.slots[s]);
        tid_cur[g] = t;
        if (g >= a.off[la]) a.cand[g] = (t < a.off[la]) ? t : kNone;
      }
      SVDAG_STEP(a, h, kStTidAssign);
      uint32_t* t = tid_prev;
      tid_prev = tid_cur;
      tid_cur = t;
    }
  }

  // ---- check set, top-down from level 1 (geom_octree_extension.cpp:1331-1407):
  // matched nodes record their match; unmatched ones put their children into
  // the next level's set.  The set is a bitmap over the global indices.  A
  // block first marks the children in a shared-memory copy of the child
  // level's words (when it fits), then ORs its non-zero words into the
  // bitmap: children are shared by many parents, and per-child global
  // stores would pile onto the same few L2 sectors.
  for (uint32_t l = 1; l < L; ++l) {
    const uint32_t g0 = a.off[l], n = a.off[l + 1] - g0;
    if (n == 0) continue;
    const uint32_t c0 = (l + 1 < L) ? a.off[l + 1] : 0, cn = (l + 1 < L) ? a.off[l + 2] - c0 : 0;
    const uint32_t w0 = c0 >> 5, words = cn ? ((c0 + cn + 31) >> 5) - w0 : 0;
    const bool local = cn && words <= a.smem_words;
    if (local) {
      for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) s_bits[w] = 0;
      __syncthreads();
    }
    SVDAG_GRID_STRIDE(i, uint64_t(n)) {
      const uint32_t g = g0 + uint32_t(i);
      if (!((a.check_bits[g >> 5] >> (g & 31)) & 1u)) continue;
      const uint32_t cd = a.cand[g];
      if (cd != kNone) { a.own[g] = cd; continue; }
      if (!cn) continue;
      const uint32_t m = a.hdr[l][i] & 0xFFu;
      uint32_t c[8];
      load_children(a.ch[l], i, c);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (!((m >> j) & 1u)) continue;
        const uint32_t x = c0 + c[j];
        if (local) {
          atomicOr(&s_bits[(x >> 5) - w0], 1u << (x & 31));
        } else if (!((a.check_bits[x >> 5] >> (x & 31)) & 1u)) {
          // a stale 0 from L1 only repeats the atomic; marks never clear
          atomicOr(&a.check_bits[x >> 5], 1u << (x & 31));
        }
      }
    }
    if (local) {
      __syncthreads();
      for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) {
        const uint32_t v = s_bits[w];
        if (v && (a.check_bits[w0 + w] & v) != v) atomicOr(&a.check_bits[w0 + w], v);
      }
    }
    SVDAG_STEP(a, l, kStCheck);
  }

  // ---- owners (min over parents), last-visit paths (max over the owner's
  // parents of path<<3|child) and B-side nodes, top-down
  for (uint32_t l = 1; l + 1 < L; ++l) {
    const uint32_t g0 = a.off[l], n = a.off[l + 1] - g0;
    if (n == 0) continue;
    const uint32_t base = a.off[l + 1];
    SVDAG_GRID_STRIDE(i, uint64_t(n)) {
      const uint32_t g = g0 + uint32_t(i);
      const uint32_t e = eff_of(a, g);
      if (e == kNone) continue;
      const uint32_t m = a.hdr[l][i] & 0xFFu;
      uint32_t c[8];
      load_children(a.ch[l], i, c);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (((m >> j) & 1u) && a.owner[base + c[j]] > e) atomicMin(&a.owner[base + c[j]], e);
    }
    SVDAG_STEP(a, l, kStOwnerMin);
    SVDAG_GRID_STRIDE(i, uint64_t(n)) {
      const uint32_t g = g0 + uint32_t(i);
      const uint32_t e = eff_of(a, g);
      if (e == kNone) continue;
      const unsigned long long pp = (a.owner[g] != kNone) ? a.path[g] : 0ull;
      const uint32_t m = a.hdr[l][i] & 0xFFu;
      uint32_t c[8];
      load_children(a.ch[l], i, c);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if ((m >> j) & 1u) {
          const uint32_t x = base + c[j];
          const unsigned long long v = (pp << 3) | uint32_t(j);
          if (a.owner[x] == e && a.best[x] < v) atomicMax(&a.best[x], v);
        }
    }
    SVDAG_STEP(a, l, kStOwnerPath);
    SVDAG_GRID_STRIDE(i, uint64_t(n)) {
      const uint32_t g = g0 + uint32_t(i);
      const uint32_t e = eff_of(a, g);
      if (e == kNone) continue;
      const bool owned = a.owner[g] != kNone;
      const unsigned long long pp = owned ? a.path[g] : 0ull;
      const uint32_t bp = owned ? a.bdesc[g] : a.own[g];  // B-side node of P
      const uint32_t m = a.hdr[l][i] & 0xFFu;
      uint32_t c[8];
      load_children(a.ch[l], i, c);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if ((m >> j) & 1u) {
          const uint32_t x = base + c[j];
          const unsigned long long pk = (pp << 3) | uint32_t(j);
          if (a.owner[x] == e && a.best[x] == pk) {
            const uint32_t lb = level_of(a, bp);
            const uint32_t bc = a.ch[lb][8ull * (bp - a.off[lb]) + j];
            a.bdesc[x] = a.off[lb + 1] + bc;
            a.path[x] = pk;
          }
        }
    }
    SVDAG_STEP(a, l, kStOwnerBdesc);
  }

  // ---- compaction: corr = own match (overwrites) else the owner's B-side
  // node; kept nodes numbered per level in global order
  uint64_t b0, b1;
  block_share(N, b0, b1);
  SVDAG_BLOCK_STRIDE(g, b0, b1) {
    const uint32_t o = a.own[g];
    a.corr[g] = (o != kNone) ? o : ((a.owner[g] != kNone) ? a.bdesc[g] : kNone);
  }
  __syncthreads();
  auto kept = [&](uint64_t g) { return a.corr[g] == kNone; };
  {
    uint32_t c = 0;
    SVDAG_BLOCK_STRIDE(g, b0, b1) c += kept(g) ? 1u : 0u;
    c = block_sum(c);
    if (threadIdx.x == 0) a.bsum[blockIdx.x] = c;
  }
  SVDAG_STEP(a, 0, kStCount);
  uint32_t total;
  {
    uint32_t base = block_offset(a.bsum, &total);
    for (uint64_t t0 = b0; t0 < b1; t0 += blockDim.x) {
      const uint64_t g = t0 + threadIdx.x;
      const uint32_t f = (g < b1 && kept(g)) ? 1u : 0u;
      uint32_t tile;
      const uint32_t pre = block_excl_scan<uint32_t>(f, &tile);
      if (g < b1) a.prefix[g] = base + pre;
      base += tile;
    }
  }
  SVDAG_STEP(a, 0, kStPrefix);
  auto level_start = [&](uint32_t l) { return a.off[l] < N ? a.prefix[a.off[l]] : total; };
  SVDAG_GRID_STRIDE(g, uint64_t(N)) {
    const uint32_t l = level_of(a, uint32_t(g));
    a.newidx[g] = kept(g) ? a.prefix[g] - level_start(l) : kNone;
  }
  if (blockIdx.x == 0)
    for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) a.cnt[l] = level_start(l + 1 < L ? l + 1 : L) - level_start(l);
  SVDAG_STEP(a, 0, kStNewidx);
  // compacted levels with rewritten children and child levels; a redirect
  // to a removed node stays 0xFFFFFFFF (geom_octree_extension.cpp:1486-1491)
  unsigned long long missing = 0;
  SVDAG_GRID_STRIDE(g, uint64_t(N)) {
    if (!kept(g)) continue;
    const uint32_t l = level_of(a, uint32_t(g));
    const uint32_t i = uint32_t(g) - a.off[l];
    const uint32_t id = a.newidx[g];
    const uint32_t h = a.hdr[l][i];
    a.ohdr[l][id] = h;
    uint8_t cl[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) cl[j] = uint8_t(l + 1);
    if (l + 1 < L) {
      const uint32_t m = h & 0xFFu;
      uint32_t c[8];
      load_children(a.ch[l], i, c);
      const uint32_t base = a.off[l + 1];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (!((m >> j) & 1u)) continue;
        const uint32_t x = base + c[j];
        const uint32_t t = a.corr[x];
        if (t != kNone) {
          cl[j] = uint8_t(level_of(a, t));
          c[j] = a.newidx[t];
          if (c[j] == kNone) ++missing;
        } else {
          c[j] = a.newidx[x];
        }
      }
      store_children(a.och[l], id, c);
    }
    uint2 packed;
    packed.x = uint32_t(cl[0]) | (uint32_t(cl[1]) << 8) | (uint32_t(cl[2]) << 16) | (uint32_t(cl[3]) << 24);
    packed.y = uint32_t(cl[4]) | (uint32_t(cl[5]) << 8) | (uint32_t(cl[6]) << 16) | (uint32_t(cl[7]) << 24);
    reinterpret_cast<uint2*>(a.oclev[l])[id] = packed;
  }
  missing = block_sum(missing);
  if (threadIdx.x == 0 && missing) atomicAdd(a.missing, missing);
  trace_mark(a.trace, trace_pos, kStEmitLevels);  // block 0's own end
}

}  // namespace

void phase_cross_level_merge(Ctx& c) {
  if (c.state != SVDAG_S_DAG) throw Error(SVDAG_ERR_INVALID_STATE, "mergeAcrossAllLevels: the octree is not a DAG");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;
  if (L > kMaxRedLevels) throw Error(SVDAG_ERR_INVALID_ARG, "mergeAcrossAllLevels: too many levels");

  CsvArgs a{};
  a.L = L;
  a.off[0] = 0;
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t o = uint64_t(a.off[l]) + c.lev[l].n;
    if (o >= 0xFFFFFFF0ull) throw Error(SVDAG_ERR_OVERFLOW, "mergeAcrossAllLevels: more than 2^32 nodes");
    a.off[l + 1] = uint32_t(o);
  }
  const uint32_t N = a.off[L];
  a.N = N;
  std::vector<Level> out(L);
  for (uint32_t l = 0; l < L; ++l) {
    a.hdr[l] = c.lev[l].hdr.get();
    a.ch[l] = c.lev[l].ch.get();
    const uint64_t cap = c.lev[l].n ? c.lev[l].n : 1;
    out[l].hdr.alloc(cap, st);
    if (l + 1 < L) out[l].ch.alloc(8 * cap, st);
    out[l].clev.alloc(8 * cap, st);
    a.ohdr[l] = out[l].hdr.get();
    a.och[l] = out[l].ch.get();
    a.oclev[l] = out[l].clev.get();
  }
  // the largest class-id domain is levels 1..L-2 (height 1)
  const uint64_t dom = (L >= 3) ? uint64_t(a.off[L - 1]) - a.off[1] : 0;
  const uint64_t Nn = N ? N : 1, dn = dom ? dom : 1;
  // shared-memory bitmap: the largest child level's words, up to kMaxPersistentSmem
  uint32_t smem_words = 0;
  for (uint32_t l = 2; l < L; ++l)
    smem_words = std::max<uint32_t>(smem_words, ((a.off[l + 1] + 31) >> 5) - (a.off[l] >> 5));
  smem_words = std::min<uint32_t>(smem_words, uint32_t(kMaxPersistentSmem / 4));
  a.smem_words = smem_words;
  const unsigned grid = persistent_grid(ex, k_csv_persistent, kRedThreads, Nn, 4 * smem_words);
  DBuf<unsigned long long> slots(table_slots(dn), st), path(Nn, st), best(Nn, st), missing(1, st);
  DBuf<uint32_t> tid_a(Nn, st), tid_b(Nn, st), khdr(dn, st), kch(8 * dn, st), slot_of(dn, st), first(256, st),
      cand(Nn, st), own(Nn, st), owner(Nn, st), bdesc(Nn, st), corr(Nn, st), prefix(Nn, st), newidx(Nn, st),
      bsum(grid, st);
  DBuf<uint32_t> check_bits((Nn + 31) / 32, st);
  DBuf<RedCtl> ctl(1, st);
  SVDAG_CUDA(cudaMemsetAsync(ctl.get(), 0, sizeof(RedCtl), st));
  a.slots = slots.get();
  a.tid_a = tid_a.get();
  a.tid_b = tid_b.get();
  a.khdr = khdr.get();
  a.kch = kch.get();
  a.slot_of = slot_of.get();
  a.first = first.get();
  a.cand = cand.get();
  a.own = own.get();
  a.owner = owner.get();
  a.bdesc = bdesc.get();
  a.corr = corr.get();
  a.prefix = prefix.get();
  a.newidx = newidx.get();
  a.bsum = bsum.get();
  a.check_bits = check_bits.get();
  a.path = path.get();
  a.best = best.get();
  a.missing = missing.get();
  a.cnt = ctl.get()->cnt;
  a.err = &ctl.get()->err;
  a.bar = &ctl.get()->bar;
  PhaseTrace trace(st);
  a.trace = trace.ptr();
  launch_persistent(ex, "k_csv_persistent", k_csv_persistent, grid, kRedThreads, 4 * smem_words, a);
  uint64_t n_missing = 0;
  SVDAG_CUDA(cudaMemcpyAsync(&n_missing, missing.get(), 8, cudaMemcpyDeviceToHost, st));
  const RedCtl h = finish_persistent(ex, ctl.get(), "mergeAcrossAllLevels");
  trace.report(ex, "mergeAcrossAllLevels");
  uint64_t kept_total = 0;
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t kept = h.cnt[l];
    out[l].n = kept;
    fit_buffer(out[l].hdr, kept, st);
    if (l + 1 < L) fit_buffer(out[l].ch, 8 * kept, st);
    fit_buffer(out[l].clev, 8 * kept, st);
    if (l > 0) kept_total += kept;
  }
  for (uint32_t l = 0; l < L; ++l) c.lev[l] = std::move(out[l]);
  c.st.n_nodes = 1 + kept_total;
  c.st.n_nodes_dag = 1 + kept_total;
  c.st.n_cross_level_merged = uint64_t(N - 1) - kept_total;
  c.st.n_missing_correspondences = n_missing;
  c.child_levels_init = true;
}

}  // namespace svdag
