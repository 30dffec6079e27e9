// Lossy LSVDAG: merge similar subtrees of a DAG within a voxel error bound.
//
// The reference's toLossyDag (src/symvox/geom_octree_extension.cpp:797-1179)
// finds candidate pairs with a multimap of subtree hashes and diffSubtrees
// (:294-368), clusters them with the external MCL binary (cluster.hpp:156)
// and merges each cluster into its representative, bottom-up.  MCL is not
// available, and the candidate order in the reference depends on OpenMP
// scheduling, so this path is project-defined (its exact form is restated by
// the oracle and pinned there):
//   * candidates: the DAG nodes of levels L-1-max_above .. L-1-min_above that
//     are still referenced and not inside a subtree kept as a merge target;
//   * distance: the exact voxel Hamming distance of two subtrees (XOR
//     popcount of their leaf voxels, the quantity diffSubtrees bounds);
//   * a merge i -> j is allowed when dist <= floor(max_error * 8^(L-lev)),
//     i.e. at most max_error of the voxels of the replaced subtree's cube
//     (8^(L-lev) voxels at level lev) change;
//   * clustering: leader rule in node order -- node i joins the lowest-index
//     leader among its allowed partners below it, else leads (rounds resolve
//     the dependency chains exactly as the sequential rule);
//   * levels run top-down; a leader's subtree is frozen (no merges inside it),
//     a merged node's subtree drops out, so no subtree is altered twice; then
//     unreachable nodes are removed and toDAG merges new duplicates, as the
//     reference ends with toDAG (geom_octree_extension.cpp:1178).
// Pairs come from an exact enumeration (every pair whose voxel counts allow
// the bound: |v_i - v_j| <= dist) or from the learned proposer (mlp.cu); both
// are checked with the exact distance.
#include <algorithm>
#include <chrono>
#include <numeric>

#include "ctx.cuh"
#include "lossy.cuh"

namespace svdag {
namespace {

constexpr uint32_t kUnd = 0xFFFFFFFFu;   // undecided
constexpr uint32_t kLead = 0xFFFFFFFEu;  // leader

struct LevelPtrs {
  const uint32_t* hdr[32];
  const uint32_t* ch[32];
};

// Leaf bytes of each candidate's subtree in Morton order: slot s (k octal
// digits = the child path) holds the leaf node's mask, 0 where the path ends.
__global__ void k_subtree_bytes(LevelPtrs P, uint32_t lev, uint32_t k, const uint32_t* __restrict__ cand, uint32_t n,
                                uint8_t* __restrict__ out) {
  const uint64_t slots = 1ull << (3 * k);
  for (uint32_t c = blockIdx.x; c < n; c += gridDim.x) {
    const uint32_t root = cand[c];
    for (uint64_t s = threadIdx.x; s < slots; s += blockDim.x) {
      uint32_t node = root, l = lev;
      uint32_t b = 0;
      bool ok = true;
      for (uint32_t step = 0; step < k; ++step) {
        const uint32_t d = uint32_t(s >> (3 * (k - 1 - step))) & 7u;
        if (!((P.hdr[l][node] >> d) & 1u)) { ok = false; break; }
        node = P.ch[l][8ull * node + d];
        ++l;
      }
      if (ok) b = (k == 0) ? 0u : (P.hdr[l][node] & 0xFFu);
      out[uint64_t(c) * slots + s] = uint8_t(b);
    }
  }
}

__global__ void k_popcounts(const uint64_t* __restrict__ w, uint64_t words, uint32_t n, uint32_t* __restrict__ pop) {
  const int lane = threadIdx.x & 31;
  for (uint32_t c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); c < n; c += gridDim.x * (blockDim.x / 32)) {
    uint32_t s = 0;
    for (uint64_t i = lane; i < words; i += 32) s += __popcll(w[uint64_t(c) * words + i]);
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    if (lane == 0) pop[c] = s;
  }
}

// Exact distance of candidate pairs (a warp per pair); keeps the pairs within
// their bound as edges (lo, hi).
__global__ void k_pair_dist(const uint64_t* __restrict__ w, uint64_t words, const uint32_t* __restrict__ pop,
                            const uint2* __restrict__ pairs, uint64_t n_pairs, uint32_t lim,
                            uint2* __restrict__ edges, unsigned long long* __restrict__ n_edges, uint64_t cap) {
  const int lane = threadIdx.x & 31;
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x / 32) + (threadIdx.x >> 5); p < n_pairs;
       p += uint64_t(gridDim.x) * (blockDim.x / 32)) {
    const uint2 q = pairs[p];
    const uint32_t gap = pop[q.x] > pop[q.y] ? pop[q.x] - pop[q.y] : pop[q.y] - pop[q.x];
    if (gap > lim) continue;  // warp-uniform
    uint32_t s = 0;
    const uint64_t* a = w + uint64_t(q.x) * words;
    const uint64_t* b = w + uint64_t(q.y) * words;
    for (uint64_t i = lane; i < words; i += 32) s += __popcll(a[i] ^ b[i]);
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    if (lane == 0 && s <= lim) {
      const unsigned long long at = atomicAdd(n_edges, 1ull);
      if (at < cap) edges[at] = make_uint2(min(q.x, q.y), max(q.x, q.y));
    }
  }
}

// Exact enumeration: candidates sorted by voxel count; each position pairs
// with the following ones while their counts can still meet the bound.
__global__ void k_band_pairs(const uint32_t* __restrict__ order, uint32_t n, const uint64_t* __restrict__ band_off,
                             uint2* __restrict__ pairs) {
  for (uint32_t p = blockIdx.x; p < n; p += gridDim.x) {
    const uint32_t i = order[p];
    const uint64_t o = band_off[p];
    const uint64_t cnt = band_off[p + 1] - o;
    for (uint64_t t = threadIdx.x; t < cnt; t += blockDim.x) pairs[o + t] = make_uint2(i, order[p + 1 + t]);
  }
}

// Leader rule, one round (see file comment); nb = lower partners per node (CSR, ascending).
__global__ void k_leader_round(const uint64_t* __restrict__ off, const uint32_t* __restrict__ nb, uint32_t n,
                               uint32_t* state, unsigned long long* undecided) {
  unsigned long long left = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (__ldcg(&state[i]) != kUnd) continue;
    bool stuck = false, done = false;
    for (uint64_t e = off[i]; e < off[i + 1]; ++e) {
      const uint32_t j = nb[e];
      const uint32_t s = __ldcg(&state[j]);
      if (s == kUnd) { stuck = true; break; }
      if (s == kLead) { __stcg(&state[i], j); done = true; break; }
    }
    if (!stuck && !done) __stcg(&state[i], kLead);
    if (stuck) ++left;
  }
  for (int o = 16; o; o >>= 1) left += __shfl_down_sync(0xFFFFFFFFu, left, o);
  if ((threadIdx.x & 31) == 0 && left) atomicAdd(undecided, left);
}

__global__ void k_leader_serial(const uint64_t* __restrict__ off, const uint32_t* __restrict__ nb, uint32_t n,
                                uint32_t* state) {
  if (blockIdx.x || threadIdx.x) return;
  for (uint32_t i = 0; i < n; ++i) {
    if (state[i] != kUnd) continue;
    uint32_t r = kLead;
    for (uint64_t e = off[i]; e < off[i + 1]; ++e)
      if (state[nb[e]] == kLead) { r = nb[e]; break; }
    state[i] = r;
  }
}

// Parents' pointers to merged nodes -> their leaders.
__global__ void k_redirect(const uint32_t* __restrict__ phdr, uint32_t* __restrict__ pch, uint64_t np,
                           const uint32_t* __restrict__ node_state) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = phdr[p] & 0xFFu;
    for (int j = 0; j < 8; ++j) {
      if (!((m >> j) & 1u)) continue;
      const uint32_t c = pch[8 * p + j];
      const uint32_t s = node_state[c];
      if (s != kUnd && s != kLead) pch[8 * p + j] = s;
    }
  }
}

// Flags of the next level from the flagged nodes of this one (reachability,
// or the frozen subtrees below leaders).
__global__ void k_mark_children(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                                const uint8_t* __restrict__ flag, uint8_t* __restrict__ next) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < n; p += uint64_t(gridDim.x) * blockDim.x) {
    if (!flag[p]) continue;
    const uint32_t m = hdr[p] & 0xFFu;
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) next[ch[8 * p + j]] = 1;
  }
}

struct FlagIn {
  const uint8_t* f;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return f[i] ? 1u : 0u; }
};
struct CandOut {
  const uint8_t* reach;
  const uint8_t* frozen;
  uint32_t* list;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t pos) const {
    if (reach[i] && !frozen[i]) list[pos] = uint32_t(i);
  }
};
struct CandIn {
  const uint8_t* reach;
  const uint8_t* frozen;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return (reach[i] && !frozen[i]) ? 1u : 0u; }
};
struct IdxOut {
  const uint8_t* f;
  uint32_t* newidx;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t pos) const { newidx[i] = f[i] ? pos : kNone; }
};

__global__ void k_compact_level(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                                const uint32_t* __restrict__ newidx, const uint32_t* __restrict__ child_newidx,
                                uint32_t* __restrict__ ohdr, uint32_t* __restrict__ och) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t id = newidx[i];
    if (id == kNone) continue;
    const uint32_t h = hdr[i];
    ohdr[id] = h;
    if (!ch) continue;
    for (int j = 0; j < 8; ++j) {
      const uint32_t c = ch[8 * i + j];
      och[8ull * id + j] = ((h >> j) & 1u) ? child_newidx[c] : kNull;
    }
  }
}

// Candidate state -> node state (merged nodes carry their leader's node id).
__global__ void k_scatter_state(const uint32_t* __restrict__ cand, const uint32_t* __restrict__ cstate, uint32_t n,
                                uint32_t* __restrict__ node_state, uint8_t* __restrict__ leader_flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t s = cstate[i];
    if (s == kLead) {
      node_state[cand[i]] = kLead;
      leader_flag[cand[i]] = 1;
    } else if (s != kUnd) {
      node_state[cand[i]] = cand[s];
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
uint32_t lossy_limit(const LossyConfig& cfg, uint32_t levels, uint32_t lev) {
  return uint32_t(cfg.max_error * double(1ull << (3 * (levels - lev))));
}

LevelSubtrees lossy_subtrees(Ctx& c, uint32_t lev, const uint32_t* d_cand, uint32_t n) {
  const Exec& ex = c.ex;
  LevelSubtrees S;
  S.n = n;
  S.k = c.levels - 1 - lev;
  S.words = std::max<uint64_t>(1, (1ull << (3 * S.k)) / 8);
  S.bytes.alloc(S.words * 8 * (n ? n : 1), c.stream);
  S.pop.alloc(n ? n : 1, c.stream);
  LevelPtrs P{};
  for (uint32_t l = 0; l < c.levels && l < 32; ++l) { P.hdr[l] = c.lev[l].hdr.get(); P.ch[l] = c.lev[l].ch.get(); }
  if (n) {
    SVDAG_LAUNCH(ex, k_subtree_bytes, unsigned(std::min<uint32_t>(n, 152u * 16)), 256, 0, P, lev, S.k, d_cand, n,
                 reinterpret_cast<uint8_t*>(S.bytes.get()));
    SVDAG_LAUNCH(ex, k_popcounts, grid_for(ex, n, 8), 256, 0, S.bytes.get(), S.words, n, S.pop.get());
  }
  return S;
}

uint64_t lossy_check_pairs(Ctx& c, const LevelSubtrees& S, const uint2* d_pairs, uint64_t n_pairs, uint32_t lim,
                           DBuf<uint2>& edges) {
  const Exec& ex = c.ex;
  const uint64_t cap = std::max<uint64_t>(n_pairs, 1);
  edges.alloc(cap, c.stream);
  DBuf<unsigned long long> d_n(1, c.stream);
  SVDAG_CUDA(cudaMemsetAsync(d_n.get(), 0, 8, c.stream));
  if (n_pairs)
    SVDAG_LAUNCH(ex, k_pair_dist, grid_for(ex, n_pairs, 8, 16), 256, 0, S.bytes.get(), S.words, S.pop.get(), d_pairs,
                 n_pairs, lim, edges.get(), d_n.get(), cap);
  return read_scalar(ex, d_n.get());
}

void phase_lossy(Ctx& c, const LossyConfig& cfg, LossyProposer* proposer, LossyResult& res) {
  if (c.state != SVDAG_S_DAG) throw Error(SVDAG_ERR_INVALID_STATE, "lossy: the octree is not a DAG");
  if (c.levels > 32) throw Error(SVDAG_ERR_INVALID_ARG, "lossy: too many levels");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;
  if (cfg.min_above > cfg.max_above) throw Error(SVDAG_ERR_INVALID_ARG, "lossy: min_above > max_above");
  if (!(cfg.max_error >= 0.0 && cfg.max_error < 1.0)) throw Error(SVDAG_ERR_INVALID_ARG, "lossy: max_error in [0, 1)");
  res = LossyResult{};
  for (uint32_t l = 1; l < L; ++l) res.nodes_before += c.lev[l].n;
  res.nodes_before += 1;
  const auto t0 = std::chrono::steady_clock::now();

  // candidate levels, top-down
  std::vector<uint32_t> levs;
  for (uint32_t a = cfg.max_above + 1; a-- > cfg.min_above;) {
    if (a + 1 >= L) continue;  // level L-1-a must be >= 1
    levs.push_back(L - 1 - a);
  }
  // flags per level: reachable, frozen
  std::vector<DBuf<uint8_t>> reach(L), frozen(L);
  for (uint32_t l = 0; l < L; ++l) {
    reach[l].alloc(c.lev[l].n ? c.lev[l].n : 1, st);
    frozen[l].alloc(c.lev[l].n ? c.lev[l].n : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(frozen[l].get(), 0, c.lev[l].n ? c.lev[l].n : 1, st));
  }
  auto mark_reach = [&]() {
    for (uint32_t l = 0; l < L; ++l) SVDAG_CUDA(cudaMemsetAsync(reach[l].get(), 0, c.lev[l].n ? c.lev[l].n : 1, st));
    SVDAG_CUDA(cudaMemsetAsync(reach[0].get(), 1, 1, st));
    for (uint32_t l = 0; l + 1 < L; ++l)
      if (c.lev[l].n)
        SVDAG_LAUNCH(ex, k_mark_children, grid_for(ex, c.lev[l].n, 256), 256, 0, c.lev[l].hdr.get(), c.lev[l].ch.get(),
                     c.lev[l].n, reach[l].get(), reach[l + 1].get());
  };
  DBuf<uint32_t> d_cnt(1, st);
  DBuf<unsigned long long> d_left(1, st);
  for (uint32_t lev : levs) {
    mark_reach();
    const uint64_t nl = c.lev[lev].n;
    // candidates: reachable, not frozen
    DBuf<uint32_t> cand(nl ? nl : 1, st);
    device_exclusive_scan<uint32_t>(ex, CandIn{reach[lev].get(), frozen[lev].get()}, nl,
                                    CandOut{reach[lev].get(), frozen[lev].get(), cand.get()}, d_cnt.get());
    const uint32_t n = uint32_t(read_scalar(ex, d_cnt.get()));
    res.candidates += n;
    if (n < 2) continue;
    LevelSubtrees S = lossy_subtrees(c, lev, cand.get(), n);
    S.lim = lossy_limit(cfg, L, lev);

    // pairs
    DBuf<uint2> pairs;
    uint64_t n_pairs = 0;
    const auto tp = std::chrono::steady_clock::now();
    if (proposer) {
      n_pairs = proposer->propose(c, lev, S, cfg, pairs);
    } else {
      std::vector<uint32_t> hp(n);
      SVDAG_CUDA(cudaMemcpyAsync(hp.data(), S.pop.get(), 4ull * n, cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
      std::vector<uint32_t> order(n);
      std::iota(order.begin(), order.end(), 0u);
      std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return hp[a] < hp[b]; });
      std::vector<uint64_t> off(n + 1, 0);
      uint32_t e = 0;
      for (uint32_t p = 0; p < n; ++p) {
        // partners q > p whose voxel counts are within the bound
        if (e < p + 1) e = p + 1;
        while (e < n && hp[order[e]] - hp[order[p]] <= S.lim) ++e;
        off[p + 1] = off[p] + (e - p - 1);
      }
      n_pairs = off[n];
      DBuf<uint32_t> d_order(n, st);
      DBuf<uint64_t> d_off(n + 1, st);
      SVDAG_CUDA(cudaMemcpyAsync(d_order.get(), order.data(), 4ull * n, cudaMemcpyHostToDevice, st));
      SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), off.data(), 8ull * (n + 1), cudaMemcpyHostToDevice, st));
      pairs.alloc(n_pairs ? n_pairs : 1, st);
      if (n_pairs)
        SVDAG_LAUNCH(ex, k_band_pairs, std::min<uint32_t>(n, 152u * 16), 256, 0, d_order.get(), n, d_off.get(),
                     pairs.get());
    }
    res.propose_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp).count();
    res.pairs_evaluated += n_pairs;
    DBuf<uint2> edges;
    const uint64_t n_edges = std::min<uint64_t>(lossy_check_pairs(c, S, pairs.get(), n_pairs, S.lim, edges),
                                                std::max<uint64_t>(n_pairs, 1));
    pairs.release();
    res.edges += n_edges;

    // leader rule over the partners below each candidate (CSR built on the host)
    std::vector<uint2> he(n_edges);
    if (n_edges)
      SVDAG_CUDA(cudaMemcpyAsync(he.data(), edges.get(), 8ull * n_edges, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
    edges.release();
    std::sort(he.begin(), he.end(), [](const uint2& a, const uint2& b) { return a.y != b.y ? a.y < b.y : a.x < b.x; });
    std::vector<uint64_t> off(n + 1, 0);
    std::vector<uint32_t> nb(n_edges);
    for (uint64_t i = 0; i < n_edges; ++i) { off[he[i].y + 1]++; nb[i] = he[i].x; }
    for (uint32_t i = 0; i < n; ++i) off[i + 1] += off[i];
    DBuf<uint64_t> d_off(n + 1, st);
    DBuf<uint32_t> d_nb(n_edges ? n_edges : 1, st), cstate(n, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), off.data(), 8ull * (n + 1), cudaMemcpyHostToDevice, st));
    if (n_edges) SVDAG_CUDA(cudaMemcpyAsync(d_nb.get(), nb.data(), 4ull * n_edges, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemsetAsync(cstate.get(), 0xFF, 4ull * n, st));
    for (int round = 0;; ++round) {
      SVDAG_CUDA(cudaMemsetAsync(d_left.get(), 0, 8, st));
      SVDAG_LAUNCH(ex, k_leader_round, grid_for(ex, n, 256), 256, 0, d_off.get(), d_nb.get(), n, cstate.get(),
                   d_left.get());
      if (read_scalar(ex, d_left.get()) == 0) break;
      if (round >= 64) {
        SVDAG_LAUNCH(ex, k_leader_serial, 1, 32, 0, d_off.get(), d_nb.get(), n, cstate.get());
        break;
      }
    }
    // apply: merged -> leader in the parents; leaders' subtrees frozen
    DBuf<uint32_t> node_state(nl, st);
    DBuf<uint8_t> lead(nl, st);
    SVDAG_CUDA(cudaMemsetAsync(node_state.get(), 0xFF, 4 * nl, st));
    SVDAG_CUDA(cudaMemsetAsync(lead.get(), 0, nl, st));
    SVDAG_LAUNCH(ex, k_scatter_state, grid_for(ex, n, 256), 256, 0, cand.get(), cstate.get(), n, node_state.get(),
                 lead.get());
    {
      std::vector<uint32_t> hs(n);
      SVDAG_CUDA(cudaMemcpyAsync(hs.data(), cstate.get(), 4ull * n, cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
      for (uint32_t s : hs) res.merged += (s != kLead && s != kUnd) ? 1 : 0;
    }
    const Level& PL = c.lev[lev - 1];
    if (PL.n)
      SVDAG_LAUNCH(ex, k_redirect, grid_for(ex, PL.n, 256), 256, 0, PL.hdr.get(), PL.ch.get(), PL.n, node_state.get());
    // frozen below leaders (and below already frozen nodes)
    SVDAG_LAUNCH(ex, k_mark_children, grid_for(ex, nl, 256), 256, 0, c.lev[lev].hdr.get(), c.lev[lev].ch.get(), nl,
                 lead.get(), frozen[lev + 1].get());
    for (uint32_t l = lev + 1; l + 1 < L; ++l)
      if (c.lev[l].n)
        SVDAG_LAUNCH(ex, k_mark_children, grid_for(ex, c.lev[l].n, 256), 256, 0, c.lev[l].hdr.get(), c.lev[l].ch.get(),
                     c.lev[l].n, frozen[l].get(), frozen[l + 1].get());
  }

  // drop unreachable nodes, bottom-up renumbering
  mark_reach();
  std::vector<DBuf<uint32_t>> newidx(L);
  std::vector<uint64_t> cnt(L, 0);
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t nl = c.lev[l].n;
    newidx[l].alloc(nl ? nl : 1, st);
    device_exclusive_scan<uint32_t>(ex, FlagIn{reach[l].get()}, nl, IdxOut{reach[l].get(), newidx[l].get()},
                                    d_cnt.get());
    cnt[l] = read_scalar(ex, d_cnt.get());
  }
  for (uint32_t l = 0; l < L; ++l) {
    Level& LV = c.lev[l];
    const bool inner = l + 1 < L;
    DBuf<uint32_t> oh(cnt[l] ? cnt[l] : 1, st), oc;
    if (inner) oc.alloc(8 * (cnt[l] ? cnt[l] : 1), st);
    if (LV.n)
      SVDAG_LAUNCH(ex, k_compact_level, grid_for(ex, LV.n, 256), 256, 0, LV.hdr.get(), inner ? LV.ch.get() : nullptr,
                   LV.n, newidx[l].get(), inner ? newidx[l + 1].get() : nullptr, oh.get(), oc.get());
    LV.hdr = std::move(oh);
    if (inner) LV.ch = std::move(oc);
    LV.n = cnt[l];
    LV.inv.release();
    LV.clev.release();
  }
  c.child_levels_init = false;
  c.state = SVDAG_S_DAG;
  phase_reduce_dag(c);  // new duplicates after the merges
  res.nodes_after = c.st.n_nodes;
  res.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace svdag
