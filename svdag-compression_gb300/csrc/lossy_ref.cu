// The candidate-edge stage of the reference's lossy LSVDAG on the GPU:
// GeomOctree::sortByEffectiveRefCount (src/symvox/geom_octree_extension.cpp:
// 521-620) and, for one level, the edges toLossyDag hands to its clustering
// (:904-1049): node hashes (computeNodeHash, :34-74), candidates by equal
// hash or, two levels above the leaves, by a one-bit-different hash (:966-988),
// the deep subtree difference diffSubtrees (:294-368) with its abort rules,
// and the acceptance bound and edge weight (:901, :1033-1036).  The
// clustering itself is the external MCL program in the reference and is not
// part of this stage; which nodes of the level below are cluster
// representatives is an input (their parents take no part, :946-958).
//
// Node order: sortByEffectiveRefCount sorts every level by effective
// reference count (the number of root paths to the node, summed in 32-bit
// unsigned arithmetic as the reference does) with std::sort, descending --
// the same unstable sort, comparator and element layout as the SSVDAG
// encoder's, so the GPU restatement of that introsort (refsort.cu) gives the
// same order.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.cuh"
#include "dedup.cuh"

namespace svdag {
namespace {

// Effective reference counts of level lev from level lev-1 (32-bit, wrapping).
__global__ void k_eff_refcount(const uint32_t* __restrict__ pch, const uint32_t* __restrict__ prc, uint64_t np,
                               uint32_t* __restrict__ rc) {
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < np; p += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t c[8];
    load_children(pch, p, c);
    const uint32_t r = prc[p];
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (c[k] != kNull) atomicAdd(&rc[c[k]], r);
  }
}

// inv[order[i]] = i
__global__ void k_invert(const uint32_t* __restrict__ order, uint64_t n, uint32_t* __restrict__ inv) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    inv[order[i]] = uint32_t(i);
}

// Sorted level: node i = old node order[i], existing children (mask bits)
// renamed through the level below's indirection.
__global__ void k_permute_level(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                                const uint32_t* __restrict__ order, const uint32_t* __restrict__ child_ind,
                                uint32_t* __restrict__ out_hdr, uint32_t* __restrict__ out_ch) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t o = order ? order[i] : uint32_t(i);
    const uint32_t h = hdr[o];
    out_hdr[i] = h;
    if (ch) {
      uint32_t c[8];
      load_children(ch, o, c);
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if ((h >> k) & 1u) c[k] = child_ind[c[k]];
      store_children(out_ch, i, c);
    }
  }
}

// computeNodeHash: depth 1 concatenates the 8 child masks (child 0 in the top
// byte); depth d >= 2 folds the children's depth d-1 hashes (std::hash of a
// 64-bit integer is the identity in libstdc++).  `child_key` holds the depth
// d-1 hashes of the level below (NULL: masks, for depth 1).
__global__ void k_node_hash(const uint32_t* __restrict__ ch, uint64_t n, const uint32_t* __restrict__ child_hdr,
                            const uint64_t* __restrict__ child_key, uint64_t* __restrict__ key) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t c[8];
    load_children(ch, i, c);
    uint64_t k = 0;
    if (!child_key) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        k <<= 8;
        if (c[j] != kNull) k += child_hdr[c[j]] & 0xFFu;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint64_t o = k;
        uint64_t h = o << (j + 1);
        if (c[j] != kNull) h = child_key[c[j]];
        k = ((o << 1) ^ h) ^ o;
      }
    }
    key[i] = k;
  }
}

// Multimap of hashes: open addressing on hash + 1 (0 = empty; the hash
// 2^64 - 1 has its own list), each slot the head of a list of nodes through
// `next`.
struct KeyMap {
  unsigned long long* keys;  // hash + 1
  uint32_t* heads;
  uint32_t* next;
  uint32_t* max_head;  // list of the nodes whose hash is 2^64 - 1
  uint64_t mask;
};

__global__ void k_map_insert(KeyMap M, const uint64_t* __restrict__ key, uint64_t n, int* __restrict__ err) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const unsigned long long k1 = key[i] + 1ull;
    uint32_t* head = nullptr;
    if (k1 == 0) {
      head = M.max_head;
    } else {
      uint64_t s = (k1 * 0x9E3779B97F4A7C15ull) >> 17 & M.mask;
      for (uint64_t probe = 0; probe <= M.mask; ++probe, s = (s + 1) & M.mask) {
        const unsigned long long prev = atomicCAS(&M.keys[s], 0ull, k1);
        if (prev == 0ull || prev == k1) { head = &M.heads[s]; break; }
      }
    }
    if (!head) { atomicExch(err, 1); continue; }
    M.next[i] = atomicExch(head, uint32_t(i));
  }
}

__device__ __forceinline__ uint32_t map_head(const KeyMap& M, uint64_t key) {
  const unsigned long long k1 = key + 1ull;
  if (k1 == 0) return *M.max_head;
  uint64_t s = (k1 * 0x9E3779B97F4A7C15ull) >> 17 & M.mask;
  for (uint64_t probe = 0; probe <= M.mask; ++probe, s = (s + 1) & M.mask) {
    const unsigned long long v = M.keys[s];
    if (v == 0ull) return kNone;
    if (v == k1) return M.heads[s];
  }
  return kNone;
}

struct LevelView {
  const uint32_t* hdr;
  const uint32_t* ch;  // NULL on the leaf level
};
constexpr int kMaxLevels = 21;
struct Pools {
  LevelView lev[kMaxLevels];
  uint32_t levels;
};

// diffSubtrees(lev, lev, A, B, abort, acc, leaves) with the reference's
// traversal order and early exits, as an explicit stack.
__device__ void diff_subtrees(const Pools& P, uint32_t lev0, uint32_t a0, uint32_t b0, uint32_t abort_at,
                              uint32_t& acc, uint32_t& leaves) {
  const uint32_t L = P.levels;
  uint32_t sa[kMaxLevels], sb[kMaxLevels];
  uint8_t si[kMaxLevels];
  int top = 0;
  sa[0] = a0;
  sb[0] = b0;
  si[0] = 0;
  while (top >= 0) {
    const uint32_t lev = lev0 + uint32_t(top);
    const uint32_t a = sa[top], b = sb[top];
    const uint32_t ma = P.lev[lev].hdr[a] & 0xFFu, mb = P.lev[lev].hdr[b] & 0xFFu;
    if (lev == L - 1) {
      // leaf: compare the voxel bits
      const uint32_t d = __popc(ma ^ mb);
      ++leaves;
      acc += d;
      if (d > 4) acc += abort_at + 1;
      --top;  // back to the parent, which then checks the threshold
      if (top >= 0 && acc >= abort_at) return;
      continue;
    }
    bool descended = false;
    while (si[top] < 8) {
      const int i = si[top]++;
      const bool ea = (ma >> i) & 1u, eb = (mb >> i) & 1u;
      if (ea != eb) {
        if (lev == L - 2) {
          const uint32_t child = ea ? P.lev[lev].ch[8ull * a + i] : P.lev[lev].ch[8ull * b + i];
          const uint32_t d = __popc(P.lev[lev + 1].hdr[child] & 0xFFu);
          ++leaves;
          acc += d;
          if (d > 4) {
            acc += abort_at + 1;
            break;  // return from this call
          }
          continue;
        }
        acc += abort_at;
        si[top] = 8;
        break;
      }
      if (!ea) continue;
      // both children exist: compare their subtrees
      sa[top + 1] = P.lev[lev].ch[8ull * a + i];
      sb[top + 1] = P.lev[lev].ch[8ull * b + i];
      si[top + 1] = 0;
      ++top;
      descended = true;
      break;
    }
    if (descended) continue;
    // this call returns
    --top;
    if (top >= 0 && acc >= abort_at) return;
  }
}

struct EdgeParams {
  uint32_t level, levels;
  uint32_t max_diff;        // maxAllowedDiff
  uint32_t included;        // includedNodeRefCount
  int flip_probe;           // two levels above the leaves: hash +- one bit, weight 1
};

// Candidate edges of every node A of the level (see the file comment): the
// edge (A, B, weight) for each partner B before A in the sorted order.  With
// out == NULL only counts.
__global__ void k_edges(Pools P, EdgeParams E, KeyMap M, const uint64_t* __restrict__ key, uint64_t n,
                        const uint32_t* __restrict__ rc, const uint8_t* __restrict__ reps_below,
                        unsigned long long* __restrict__ count, uint2* __restrict__ out, float* __restrict__ w,
                        uint64_t cap) {
  const LevelView V = P.lev[E.level];
  for (uint64_t ia = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; ia < n; ia += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t A = uint32_t(ia);
    if (rc[A] > E.included) continue;
    if (reps_below) {
      const uint32_t m = V.hdr[A] & 0xFFu;
      bool parent_of_rep = false;
      for (int c = 0; c < 8 && !parent_of_rep; ++c)
        if ((m >> c) & 1u) parent_of_rep = reps_below[V.ch[8ull * A + c]] != 0;
      if (parent_of_rep) continue;
    }
    const uint64_t k = key[A];
    const int probes = E.flip_probe ? 64 : 1;
    for (int bit = 0; bit < probes; ++bit) {
      const uint64_t kk = E.flip_probe ? (k ^ (1ull << bit)) : k;
      for (uint32_t B = map_head(M, kk); B != kNone; B = M.next[B]) {
        if (B >= A) continue;
        if (rc[B] > E.included) continue;
        float weight = 1.f;
        if (!E.flip_probe) {
          uint32_t diff = 0, leaves = 0;
          diff_subtrees(P, E.level, A, B, E.max_diff + 1, diff, leaves);
          // :1033 -- maxAllowedSubtreeDiff = 4.0 * numLeaves, as a float
          const float sub = float(4.0 * double(leaves));
          if (!(diff <= E.max_diff && float(diff) < sub)) continue;
          weight = __fsub_rn(1.0f, __fdiv_rn(float(diff), __fadd_rn(float(E.max_diff), 1.0f)));
        }
        const unsigned long long slot = atomicAdd(count, 1ull);
        if (out && slot < cap) {
          out[slot] = make_uint2(A, B);
          w[slot] = weight;
        }
      }
    }
  }
}

void level_refcounts(Ctx& c, std::vector<DBuf<uint32_t>>& rc) {
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  rc.clear();
  rc.resize(c.levels);
  for (uint32_t l = 0; l < c.levels; ++l) {
    const uint64_t n = c.lev[l].n;
    rc[l].alloc(n ? n : 1, st);
    SVDAG_CUDA(cudaMemsetAsync(rc[l].get(), 0, 4 * (n ? n : 1), st));
  }
  const uint32_t one = 1;
  SVDAG_CUDA(cudaMemcpyAsync(rc[0].get(), &one, 4, cudaMemcpyHostToDevice, st));
  for (uint32_t l = 1; l < c.levels; ++l) {
    const Level& Pl = c.lev[l - 1];
    if (Pl.n && Pl.ch.get())
      SVDAG_LAUNCH(ex, k_eff_refcount, grid_for(ex, Pl.n, 256), 256, 0, Pl.ch.get(), rc[l - 1].get(), Pl.n,
                   rc[l].get());
  }
  SVDAG_CUDA(cudaStreamSynchronize(st));  // `one` is a host stack value
}

void check_lossy_state(const Ctx& c) {
  if (c.state != SVDAG_S_DAG) throw Error(SVDAG_ERR_INVALID_STATE, "lossy candidates: the octree is not a DAG");
  for (const auto& L : c.lev)
    if (L.clev.get()) throw Error(SVDAG_ERR_INVALID_STATE, "lossy candidates: cross-level merged octree");
  if (c.levels > kMaxLevels) throw Error(SVDAG_ERR_INVALID_ARG, "lossy candidates: too many levels");
}

}  // namespace

void phase_sort_by_effective_refcount(Ctx& c) {
  check_lossy_state(c);
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  std::vector<DBuf<uint32_t>> rc;
  level_refcounts(c, rc);
  DBuf<uint32_t> child_ind;  // indirection of the level below: old index -> new index
  for (int lev = int(c.levels) - 1; lev >= 0; --lev) {
    Level& L = c.lev[lev];
    const uint64_t n = L.n;
    DBuf<uint32_t> order, ind(n ? n : 1, st);
    if (lev > 0 && n) {
      order.alloc(n, st);
      refcount_order(ex, rc[lev].get(), n, order.get());
      SVDAG_LAUNCH(ex, k_invert, grid_for(ex, n, 256), 256, 0, order.get(), n, ind.get());
    } else if (n) {
      std::vector<uint32_t> id(n);
      for (uint64_t i = 0; i < n; ++i) id[i] = uint32_t(i);
      SVDAG_CUDA(cudaMemcpyAsync(ind.get(), id.data(), 4 * n, cudaMemcpyHostToDevice, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
    }
    const bool inner = uint32_t(lev) + 1 < c.levels;
    DBuf<uint32_t> out_hdr(n ? n : 1, st), out_ch(inner ? 8 * (n ? n : 1) : 0, st);
    if (n)
      SVDAG_LAUNCH(ex, k_permute_level, grid_for(ex, n, 256), 256, 0, L.hdr.get(), inner ? L.ch.get() : nullptr, n,
                   order.get(), child_ind.get(), out_hdr.get(), out_ch.get());
    L.hdr = std::move(out_hdr);
    if (inner) L.ch = std::move(out_ch);
    child_ind = std::move(ind);
  }
  SVDAG_CUDA(cudaStreamSynchronize(st));
}

void lossy_candidate_edges(Ctx& c, uint32_t level, float diff_factor, int included, const uint8_t* h_reps,
                           std::vector<uint32_t>& src, std::vector<uint32_t>& tgt, std::vector<float>& weight) {
  check_lossy_state(c);
  if (level == 0 || level + 2 > c.levels)
    throw Error(SVDAG_ERR_INVALID_ARG, "lossy candidates: level must be in [1, levels - 2]");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;
  const uint64_t n = c.lev[level].n;
  std::vector<DBuf<uint32_t>> rc;
  level_refcounts(c, rc);
  // computeNodeHash depth at this level (:904): max(levels - lev - 2, 1)
  const uint32_t depth = std::max<int>(int(L) - int(level) - 2, 1);
  DBuf<uint64_t> key, child_key;
  for (uint32_t d = 1; d <= depth; ++d) {
    const uint32_t lv = level + depth - d;  // the level whose depth-d hashes this pass makes
    const uint64_t m = c.lev[lv].n;
    key.alloc(m ? m : 1, st);
    if (m)
      SVDAG_LAUNCH(ex, k_node_hash, grid_for(ex, m, 256), 256, 0, c.lev[lv].ch.get(), m, c.lev[lv + 1].hdr.get(),
                   d == 1 ? nullptr : child_key.get(), key.get());
    child_key = std::move(key);
  }
  key = std::move(child_key);
  // multimap of this level's hashes
  uint64_t slots = 64;
  while (slots < 2 * (n ? n : 1)) slots <<= 1;
  DBuf<unsigned long long> mkeys(slots, st);
  DBuf<uint32_t> heads(slots, st), next(n ? n : 1, st), max_head(1, st);
  DBuf<int> err(1, st);
  SVDAG_CUDA(cudaMemsetAsync(mkeys.get(), 0, 8 * slots, st));
  SVDAG_CUDA(cudaMemsetAsync(heads.get(), 0xFF, 4 * slots, st));
  SVDAG_CUDA(cudaMemsetAsync(max_head.get(), 0xFF, 4, st));
  SVDAG_CUDA(cudaMemsetAsync(err.get(), 0, 4, st));
  const KeyMap M{mkeys.get(), heads.get(), next.get(), max_head.get(), slots - 1};
  if (n) SVDAG_LAUNCH(ex, k_map_insert, grid_for(ex, n, 256), 256, 0, M, key.get(), n, err.get());
  check_err(ex, err.get(), "lossy candidates");
  // representatives of the level below
  DBuf<uint8_t> reps;
  if (h_reps) {
    const uint64_t nb = c.lev[level + 1].n;
    reps.alloc(nb ? nb : 1, st);
    if (nb) SVDAG_CUDA(cudaMemcpyAsync(reps.get(), h_reps, nb, cudaMemcpyHostToDevice, st));
  }
  Pools P{};
  P.levels = L;
  for (uint32_t l = 0; l < L; ++l) P.lev[l] = LevelView{c.lev[l].hdr.get(), l + 1 < L ? c.lev[l].ch.get() : nullptr};
  EdgeParams E;
  E.level = level;
  E.levels = L;
  // :901 -- std::round(std::pow(levels - lev, 2) * allowedLossyDiffFactor), in double
  E.max_diff = unsigned(std::round(std::pow(double(L - level), 2) * double(diff_factor)));
  E.included = uint32_t(std::max(included, 0));
  E.flip_probe = (level == L - 2) ? 1 : 0;
  DBuf<unsigned long long> cnt(1, st);
  SVDAG_CUDA(cudaMemsetAsync(cnt.get(), 0, 8, st));
  if (n)
    SVDAG_LAUNCH(ex, k_edges, grid_for(ex, n, 128), 128, 0, P, E, M, key.get(), n, rc[level].get(),
                 h_reps ? reps.get() : nullptr, cnt.get(), nullptr, nullptr, 0);
  const uint64_t total = read_scalar(ex, cnt.get());
  DBuf<uint2> out(total ? total : 1, st);
  DBuf<float> w(total ? total : 1, st);
  if (total) {
    SVDAG_CUDA(cudaMemsetAsync(cnt.get(), 0, 8, st));
    SVDAG_LAUNCH(ex, k_edges, grid_for(ex, n, 128), 128, 0, P, E, M, key.get(), n, rc[level].get(),
                 h_reps ? reps.get() : nullptr, cnt.get(), out.get(), w.get(), total);
  }
  std::vector<uint2> ho(total);
  std::vector<float> hw(total);
  if (total) {
    SVDAG_CUDA(cudaMemcpyAsync(ho.data(), out.get(), 8 * total, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaMemcpyAsync(hw.data(), w.get(), 4 * total, cudaMemcpyDeviceToHost, st));
  }
  SVDAG_CUDA(cudaStreamSynchronize(st));
  // ascending (source, target): the atomic append leaves no particular order
  std::vector<uint64_t> idx(total);
  for (uint64_t i = 0; i < total; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
    return ho[a].x != ho[b].x ? ho[a].x < ho[b].x : ho[a].y < ho[b].y;
  });
  src.resize(total);
  tgt.resize(total);
  weight.resize(total);
  for (uint64_t i = 0; i < total; ++i) {
    src[i] = ho[idx[i]].x;
    tgt[i] = ho[idx[i]].y;
    weight[i] = hw[idx[i]];
  }
}

}  // namespace svdag
