// Voxel-brick chunks: the plain per-chunk ingest and the batched build.
//
// A chunk of depth d is a dense grid of 2^d voxels per side given as
// 8^(d-1) leaf bricks (2^3 voxels, bit 4x+2y+z) in Morton order (x the most
// significant bit of each coordinate triple).  The reference has no voxel
// input; a grid enters it as node pools through the NodeData constructor
// (src/symvox/geom_octree.cpp:49-60): level d-1 = the non-empty bricks in
// Morton order, each level above = the non-empty cells of 8 consecutive
// entries of the level below, the root always present.  toDAG, toSDAG and the
// cross-level merge then run on those pools as on any other.
//
// Plain form (svdag_import_bricks): those SVO pools are materialised in a
// context, which the ordinary per-chunk pipeline reduces.
//
// Batched form (svdag_batch_*): many chunks at once, height by height (height
// h = level d-1-h, so every chunk's leaves are height 0).  The SVO is never
// materialised: toDAG's first-occurrence order over a level is the Morton
// order of its non-empty cells, so each cell's DAG id is found directly from
// its key (mask, DAG ids of its 8 children) in one hash table shared by all
// chunks, with the chunk id in the key; equal keys converge on the smallest
// global cell index, i.e. the first occurrence within their chunk.  One
// launch per step covers every chunk of a height.  One height above the
// leaves the key is the equivalent (chunk, 8 brick bytes) (k_batch_insert_h1);
// each height's table is sized from the share of distinct keys earlier waves
// saw there, and rebuilt at full size when that proves too small; the
// representatives are numbered from one flag bit per cell.  The DAGs then go
// through toSDAG and the cross-level merge per chunk, on several streams at
// once.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <new>
#include <thread>

#include "ctx.cuh"
#include "dedup.cuh"

namespace svdag {
namespace {

// ---------------------------------------------------------------------------
// Seeded 3D value noise (lattice period 16 voxels, trilinear), used to make
// synthetic occupancy grids.
__host__ __device__ __forceinline__ uint32_t hash3(uint32_t x, uint32_t y, uint32_t z, uint32_t s) {
  uint32_t h = x * 0x8DA6B343u ^ y * 0xD8163841u ^ z * 0xCB1AB31Fu ^ s * 0x165667B1u;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}
__host__ __device__ __forceinline__ float lattice(uint32_t x, uint32_t y, uint32_t z, uint32_t s) {
  return float(hash3(x, y, z, s) >> 8) * (1.0f / 16777216.0f);
}
__host__ __device__ __forceinline__ float value_noise3(uint32_t x, uint32_t y, uint32_t z, uint32_t s) {
  const uint32_t X = x >> 4, Y = y >> 4, Z = z >> 4;
  const float fx = float(x & 15u) * (1.0f / 16.0f), fy = float(y & 15u) * (1.0f / 16.0f),
              fz = float(z & 15u) * (1.0f / 16.0f);
  float c[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      const float a = lattice(X + i, Y + j, Z, s), b = lattice(X + i, Y + j, Z + 1, s);
      c[i][j] = a + (b - a) * fz;
    }
  const float c0 = c[0][0] + (c[0][1] - c[0][0]) * fy, c1 = c[1][0] + (c[1][1] - c[1][0]) * fy;
  return c0 + (c1 - c0) * fx;
}

// Morton brick index -> brick coordinates (x most significant per triple).
__host__ __device__ __forceinline__ void morton_decode(uint64_t m, uint32_t& x, uint32_t& y, uint32_t& z) {
  x = y = z = 0;
  for (int i = 0; i < 21; ++i) {
    z |= uint32_t((m >> (3 * i)) & 1u) << i;
    y |= uint32_t((m >> (3 * i + 1)) & 1u) << i;
    x |= uint32_t((m >> (3 * i + 2)) & 1u) << i;
  }
}

__global__ void k_noise_samples(uint32_t side, uint32_t seed, uint32_t n, float* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t h = hash3(i, 0x51ED27u, 0x2F0Bu, seed ^ 0xA5A5A5A5u);
    const uint32_t g = hash3(h, i, 7u, seed);
    const uint32_t k = hash3(g, h, 11u, seed);
    out[i] = value_noise3(h % side, g % side, k % side, seed);
  }
}

__global__ void k_noise_bricks(uint64_t n_bricks, uint32_t seed, float thr, uint8_t* __restrict__ out) {
  for (uint64_t b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; b < n_bricks; b += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t bx, by, bz;
    morton_decode(b, bx, by, bz);
    uint32_t m = 0;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const uint32_t x = 2 * bx + ((v >> 2) & 1), y = 2 * by + ((v >> 1) & 1), z = 2 * bz + (v & 1);
      m |= uint32_t(value_noise3(x, y, z, seed) < thr) << v;
    }
    out[b] = uint8_t(m);
  }
}

// ---------------------------------------------------------------------------
// Plain form: SVO pools of one chunk.

// Cells of one level: occupancy from the level below (bricks or child ids).
struct BrickNonEmpty {
  const uint8_t* b;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return b[i] ? 1u : 0u; }
};
struct CellNonEmpty {
  const uint32_t* below;  // node index per cell of the level below (kNone = empty)
  bool root;
  __device__ __forceinline__ uint32_t operator()(uint64_t j) const {
    if (root) return 1u;
    const uint4 a = reinterpret_cast<const uint4*>(below + 8 * j)[0], b = reinterpret_cast<const uint4*>(below + 8 * j)[1];
    return (a.x & a.y & a.z & a.w & b.x & b.y & b.z & b.w) == kNone ? 0u : 1u;
  }
};
struct IndexOut {
  uint32_t* idx;
  const uint8_t* b;
  const uint32_t* below;
  bool root;
  __device__ __forceinline__ void operator()(uint64_t j, uint32_t pos) const {
    bool ne;
    if (b) {
      ne = b[j] != 0;
    } else if (root) {
      ne = true;
    } else {
      const uint4 a = reinterpret_cast<const uint4*>(below + 8 * j)[0], c = reinterpret_cast<const uint4*>(below + 8 * j)[1];
      ne = (a.x & a.y & a.z & a.w & c.x & c.y & c.z & c.w) != kNone;
    }
    idx[j] = ne ? pos : kNone;
  }
};

__global__ void k_leaf_nodes(const uint8_t* __restrict__ b, uint64_t n, const uint32_t* __restrict__ idx,
                             uint32_t* __restrict__ hdr, unsigned long long* vox) {
  uint64_t s = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = b[i];
    if (m) {
      hdr[idx[i]] = m;
      s += __popc(m);
    }
  }
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(vox, (unsigned long long)s);
}

__global__ void k_inner_nodes(const uint32_t* __restrict__ below, uint64_t n, const uint32_t* __restrict__ idx,
                              uint32_t* __restrict__ hdr, uint32_t* __restrict__ ch) {
  for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < n; j += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t id = idx[j];
    if (id == kNone) continue;
    uint32_t c[8], m = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t v = below[8 * j + k];
      c[k] = (v == kNone) ? kNull : v;
      m |= uint32_t(v != kNone) << k;
    }
    hdr[id] = m;
    store_children(ch, id, c);
  }
}

// ---------------------------------------------------------------------------
// Batched form.

struct ChunkSet {
  const uint64_t* base;   // [n+1] global cell offset of each chunk at this height
  uint32_t n;
};
__device__ __forceinline__ uint32_t chunk_of(const ChunkSet& S, uint64_t g) {
  uint32_t lo = 0, hi = S.n;  // base[lo] <= g < base[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (S.base[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

struct HeightView {
  ChunkSet cells;                // cells of this height
  const uint32_t* part;          // [n] chunk id of each participating entry
  const uint8_t* const* bricks;  // [n] (height 1) bricks of each entry
  const uint32_t* leaf_rank;     // [chunks*256] (height 1) leaf DAG id per mask
  const uint64_t* below_base;    // [n] (height >= 2) global offset of each entry's cells one height down
  const uint32_t* below_ids;     // (height >= 2) DAG id per cell one height down (kNone = empty)
  const uint8_t* is_top;         // [n] 1 when this height is the entry's root level
  uint32_t h;
};

// Key of cell g: chunk, mask and the DAG ids of its 8 children.
__device__ __forceinline__ uint32_t cell_key(const HeightView& V, uint64_t g, uint32_t& e, uint32_t ids[8]) {
  e = chunk_of(V.cells, g);
  const uint64_t j = g - V.cells.base[e];
  uint32_t m = 0;
  if (V.h == 1) {
    const uint64_t w = reinterpret_cast<const uint64_t*>(V.bricks[e])[j];
    const uint32_t* rk = V.leaf_rank + 256u * V.part[e];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t b = uint32_t(w >> (8 * k)) & 0xFFu;
      ids[k] = b ? rk[b] : kNull;
      m |= uint32_t(b != 0) << k;
    }
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(V.below_ids + V.below_base[e] + 8 * j);
    const uint4 a = p[0], c = p[1];
    const uint32_t v[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      ids[k] = (v[k] == kNone) ? kNull : v[k];
      m |= uint32_t(v[k] != kNone) << k;
    }
  }
  return m;
}

__device__ __forceinline__ uint64_t key_hash(uint32_t chunk, uint32_t m, const uint32_t ids[8]) {
  uint64_t h = mix_word(0x243F6A8885A308D3ull, chunk);
  h = mix_word(h, m);
#pragma unroll
  for (int k = 0; k < 8; ++k) h = mix_word(h, ids[k]);
  return finish_hash(h);
}

constexpr int kGBits = 40;  // cell index bits in a slot (the rest: hash tag)
constexpr uint64_t kGMask = (1ull << kGBits) - 1;
// Probes after which an insert into a table sized from an estimate gives up
// (the table is then rebuilt at full size).
constexpr uint64_t kProbeLimit = 512;
// Largest table (slot positions and the kNone mark fit 32 bits; a height of
// 2^30 cells -- a wave's largest -- still loads it at most half).
constexpr uint64_t kMaxTableSlots = 1ull << 31;

// Probe for the key of cell g; returns its slot (inserted, or found holding
// an equal key, lowered to g when g is smaller), or ~0 when `limit` + 1 slots
// were probed without either (always the case for a full table when limit =
// mask).
__device__ __forceinline__ uint64_t batch_probe(const HeightView& V, uint64_t g, uint32_t chunk, uint32_t m,
                                                const uint32_t ids[8], uint64_t hk,
                                                unsigned long long* __restrict__ slots, uint64_t mask,
                                                uint64_t limit) {
  const uint64_t tag = hk >> kGBits;
  const unsigned long long mine = (tag << kGBits) | g;
  uint64_t pos = hk & mask;
  for (uint64_t probe = 0; probe <= limit; ++probe) {
    unsigned long long cur = __ldcg(&slots[pos]);
    if (cur == kEmpty64) {
      const unsigned long long prev = atomicCAS(&slots[pos], kEmpty64, mine);
      if (prev == kEmpty64) return pos;
      cur = prev;
    }
    if ((cur >> kGBits) == tag) {
      const uint64_t g2 = cur & kGMask;
      uint32_t e2, ids2[8];
      const uint32_t m2 = cell_key(V, g2, e2, ids2);
      bool eq = (V.part[e2] == chunk) && (m2 == m);
#pragma unroll
      for (int k = 0; k < 8; ++k) eq &= (ids2[k] == ids[k]);
      if (eq) {
        if (g < g2) atomicMin(&slots[pos], mine);
        return pos;
      }
    }
    pos = (pos + 1) & mask;
  }
  return ~0ull;
}

// Inserts every non-empty cell's key and records in slot_of[g] the slot that
// holds it (~0 for empty cells).  Lanes of a warp with the same key -- runs
// of identical cells are common in solid or empty regions -- probe once: the
// lowest such lane (also the smallest cell index) probes for all of them.
// A probe that gives up sets *err; with limit < mask (a table sized from an
// estimate) the other warps then stop early, as the insert will be redone.
__global__ void k_batch_insert(HeightView V, uint64_t total, unsigned long long* __restrict__ slots, uint64_t mask,
                               uint64_t limit, uint32_t* __restrict__ slot_of, int* err) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t w = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; (w << 5) < total; w += warps) {
    if (limit < mask) {
      // warp-uniform: every lane takes the flag lane 0 read
      int stop = 0;
      if (lane == 0) stop = *reinterpret_cast<volatile int*>(err);
      if (__shfl_sync(0xFFFFFFFFu, stop, 0)) return;
    }
    const uint64_t g = (w << 5) + lane;
    uint32_t e = 0, ids[8], m = 0;
    bool part = false;
    if (g < total) {
      m = cell_key(V, g, e, ids);
      part = m || V.is_top[e];
    }
    const unsigned act = __ballot_sync(0xFFFFFFFFu, part);
    if (!part) {
      if (g < total) slot_of[g] = kNone;
      continue;
    }
    const uint32_t chunk = V.part[e];
    const uint64_t hk = key_hash(chunk, m, ids);
    const unsigned grp = __match_any_sync(act, hk);
    const int lead = __ffs(int(grp)) - 1;
    // the leader's key, to confirm equal keys behind equal hashes
    bool same = true;
    same &= __shfl_sync(act, chunk, lead) == chunk;
    same &= __shfl_sync(act, m, lead) == m;
#pragma unroll
    for (int k = 0; k < 8; ++k) same &= __shfl_sync(act, ids[k], lead) == ids[k];
    uint64_t pos = 0;
    if (int(lane) == lead) pos = batch_probe(V, g, chunk, m, ids, hk, slots, mask, limit);
    const uint64_t lpos = __shfl_sync(act, pos, lead);
    if (int(lane) != lead) pos = same ? lpos : batch_probe(V, g, chunk, m, ids, hk, slots, mask, limit);
    if (pos == ~0ull) atomicExch(err, 1);
    slot_of[g] = pos == ~0ull ? kNone : uint32_t(pos);
  }
}

// Height 1 (cells of 8 bricks): within one entry (chunk), a brick's leaf DAG
// id is a one-to-one function of its mask (the rank of the mask's first
// occurrence), so two cells have equal keys exactly when they are cells of
// the same entry with the same 8 brick bytes.  The key is therefore (entry,
// 64-bit brick word): one load per cell, no rank lookups, and a probe that
// meets a candidate confirms it with one load of the candidate's word.  The
// representatives -- and so every id -- are the ones the general key gives.
// The entry of a warp's cells is searched once per warp (lanes past its end
// search for their own).
__device__ __forceinline__ uint64_t brick_word(const HeightView& V, uint32_t e, uint64_t g) {
  return reinterpret_cast<const uint64_t*>(V.bricks[e])[g - V.cells.base[e]];
}

__device__ __forceinline__ uint64_t h1_probe(const HeightView& V, uint64_t g, uint32_t e, uint64_t word, uint64_t hk,
                                             unsigned long long* __restrict__ slots, uint64_t mask, uint64_t limit) {
  const uint64_t tag = hk >> kGBits;
  const unsigned long long mine = (tag << kGBits) | g;
  const uint64_t lo = V.cells.base[e], hi = V.cells.base[e + 1];
  uint64_t pos = hk & mask;
  for (uint64_t probe = 0; probe <= limit; ++probe) {
    unsigned long long cur = __ldcg(&slots[pos]);
    if (cur == kEmpty64) {
      const unsigned long long prev = atomicCAS(&slots[pos], kEmpty64, mine);
      if (prev == kEmpty64) return pos;
      cur = prev;
    }
    if ((cur >> kGBits) == tag) {
      const uint64_t g2 = cur & kGMask;
      // equal keys only within the entry: a candidate outside it differs
      if (g2 >= lo && g2 < hi && brick_word(V, e, g2) == word) {
        if (g < g2) atomicMin(&slots[pos], mine);
        return pos;
      }
    }
    pos = (pos + 1) & mask;
  }
  return ~0ull;
}

__global__ void k_batch_insert_h1(HeightView V, uint64_t total, unsigned long long* __restrict__ slots, uint64_t mask,
                                  uint64_t limit, uint32_t* __restrict__ slot_of, int* err) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t w = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; (w << 5) < total; w += warps) {
    if (limit < mask) {
      // warp-uniform: every lane takes the flag lane 0 read
      int stop = 0;
      if (lane == 0) stop = *reinterpret_cast<volatile int*>(err);
      if (__shfl_sync(0xFFFFFFFFu, stop, 0)) return;
    }
    const uint64_t g0 = w << 5, g = g0 + lane;
    uint32_t e = 0;
    if (lane == 0) e = chunk_of(V.cells, g0);
    e = __shfl_sync(0xFFFFFFFFu, e, 0);
    uint64_t word = 0;
    bool part = false;
    if (g < total) {
      if (g >= V.cells.base[e + 1]) e = chunk_of(V.cells, g);
      word = brick_word(V, e, g);
      part = word != 0 || V.is_top[e];
    }
    const unsigned act = __ballot_sync(0xFFFFFFFFu, part);
    if (!part) {
      if (g < total) slot_of[g] = kNone;
      continue;
    }
    const uint64_t hk = finish_hash(mix_word(mix_word(mix_word(0x3C6EF372FE94F82Bull, e), uint32_t(word)),
                                             uint32_t(word >> 32)));
    // lanes with the same (entry, word) probe once, through the lowest
    const unsigned grp = __match_any_sync(act, hk);
    const int lead = __ffs(int(grp)) - 1;
    const uint32_t le = __shfl_sync(act, e, lead);  // both shuffles on every active lane
    const uint64_t lw = __shfl_sync(act, word, lead);
    const bool same = le == e && lw == word;
    uint64_t pos = 0;
    if (int(lane) == lead) pos = h1_probe(V, g, e, word, hk, slots, mask, limit);
    const uint64_t lpos = __shfl_sync(act, pos, lead);
    if (int(lane) != lead) pos = same ? lpos : h1_probe(V, g, e, word, hk, slots, mask, limit);
    if (pos == ~0ull) atomicExch(err, 1);
    slot_of[g] = pos == ~0ull ? kNone : uint32_t(pos);
  }
}

// The representative (smallest index with the same key) of every non-empty
// cell: the index its slot holds once every insert is done; and one bit per
// cell, set for the representatives (bit g & 31 of word g >> 5, one word per
// warp by ballot).  Nothing to do when an insert into an estimated table gave
// up (retry non-null and set: slot_of is incomplete and the height is
// redone).
__global__ void k_batch_rep(uint64_t total, const unsigned long long* __restrict__ slots, uint64_t mask,
                            const int* __restrict__ retry, uint32_t* __restrict__ rep, uint32_t* __restrict__ flags) {
  if (retry && *retry) return;
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t w = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; (w << 5) < total; w += warps) {
    const uint64_t g = (w << 5) + lane;
    bool own = false;
    if (g < total) {
      const uint32_t p = rep[g];
      const uint32_t r = p > mask ? kNone : uint32_t(slots[p] & kGMask);
      rep[g] = r;
      own = r == g;
    }
    const unsigned b = __ballot_sync(0xFFFFFFFFu, own);
    if (lane == 0) flags[w] = b;
  }
}

struct FlagPopc {
  const uint32_t* w;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return __popc(w[i]); }
};
struct U32Out {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};

// Number of representatives before cell g (woff: exclusive prefix of the
// flag words' popcounts): a representative's node number in the wave.
__device__ __forceinline__ uint32_t flag_rank(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ woff,
                                              uint64_t g) {
  const uint64_t w = g >> 5;
  return woff[w] + uint32_t(__popc(flags[w] & ((1u << (g & 31u)) - 1u)));
}

// Node number of each entry's first cell (the entry's DAG nodes are the
// numbers from there to the next entry's), and the wave's total.
__global__ void k_entry_bases(uint32_t n, const uint64_t* __restrict__ base, const uint32_t* __restrict__ flags,
                              const uint32_t* __restrict__ woff, const uint32_t* __restrict__ d_total,
                              uint32_t* __restrict__ out) {
  for (uint32_t e = threadIdx.x; e <= n; e += blockDim.x) out[e] = e < n ? flag_rank(flags, woff, base[e]) : *d_total;
}

// DAG id (within the chunk) of every cell, and the DAG nodes of this height,
// written straight into each entry's own level buffers (hdr_e[e], ch_e[e])
// (node numbers of a wave fit 32 bits: a wave has at most 2^30 cells).
__global__ void k_batch_emit(HeightView V, uint64_t total, const uint32_t* __restrict__ rep,
                             const uint32_t* __restrict__ flags, const uint32_t* __restrict__ woff,
                             const uint64_t* __restrict__ rep_base, uint32_t* __restrict__ ids_out,
                             uint32_t* const* __restrict__ hdr_e, uint32_t* const* __restrict__ ch_e) {
  for (uint64_t g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; g < total; g += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t r = rep[g];
    if (r == kNone) { ids_out[g] = kNone; continue; }
    const uint32_t e = chunk_of(V.cells, g);
    const uint32_t id = uint32_t(flag_rank(flags, woff, r) - rep_base[e]);
    ids_out[g] = id;
    if (r == g) {
      uint32_t e2, ids[8];
      const uint32_t m = cell_key(V, g, e2, ids);
      hdr_e[e][id] = m;
      store_children(ch_e[e], id, ids);
    }
  }
}

// Leaf height: first occurrence of every mask per chunk, ranks, voxel counts.
__global__ void k_batch_leaf_first(const uint8_t* const* __restrict__ bricks, const uint64_t* __restrict__ n_bricks,
                                   uint32_t* __restrict__ first, unsigned long long* __restrict__ vox) {
  const uint32_t c = blockIdx.y;
  const uint8_t* b = bricks[c];
  const uint64_t n = n_bricks[c];
  __shared__ uint32_t sf[256];
  for (int m = threadIdx.x; m < 256; m += blockDim.x) sf[m] = kNone;
  __syncthreads();
  // 8 bricks per load (the brick arrays are 8-byte aligned, n a multiple of 8)
  const uint64_t* w8 = reinterpret_cast<const uint64_t*>(b);
  unsigned long long s = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n / 8; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t w = w8[i];
    if (!w) continue;
    s += __popcll(w);
    const uint32_t m0 = uint32_t(w) & 0xFFu;
    if (w == uint64_t(m0) * 0x0101010101010101ull) {
      // 8 equal bricks (solid or repeated regions): only the first can be a
      // first occurrence
      const uint32_t at = uint32_t(8 * i);
      if (sf[m0] > at) atomicMin(&sf[m0], at);
      continue;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t m = uint32_t(w >> (8 * k)) & 0xFFu;
      const uint32_t at = uint32_t(8 * i + k);
      if (m && sf[m] > at) atomicMin(&sf[m], at);
    }
  }
  __syncthreads();
  for (int m = threadIdx.x; m < 256; m += blockDim.x)
    if (sf[m] != kNone) atomicMin(&first[256u * c + m], sf[m]);
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(&vox[c], s);
}

__global__ void k_batch_leaf_rank(const uint32_t* __restrict__ first, uint32_t* __restrict__ rank,
                                  uint32_t* __restrict__ leaf_hdr, uint32_t* __restrict__ leaf_count) {
  const uint32_t c = blockIdx.x;
  __shared__ uint32_t sf[256];
  const int m = threadIdx.x;
  sf[m] = first[256u * c + m];
  __syncthreads();
  if (sf[m] != kNone) {
    uint32_t r = 0;
    for (int k = 0; k < 256; ++k) r += (sf[k] < sf[m]) ? 1u : 0u;
    rank[256u * c + m] = r;
    leaf_hdr[256u * c + r] = uint32_t(m);
  } else {
    rank[256u * c + m] = kNone;
  }
  if (m == 0) {
    uint32_t n = 0;
    for (int k = 0; k < 256; ++k) n += (sf[k] != kNone) ? 1u : 0u;
    leaf_count[c] = n;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
float synth_noise_bricks(cudaStream_t st, uint32_t depth, uint64_t seed, double fill, uint8_t* out) {
  if (depth < 2 || depth > 11) throw Error(SVDAG_ERR_INVALID_ARG, "noise bricks: depth must be in [2, 11]");
  if (!(fill > 0.0 && fill < 1.0)) throw Error(SVDAG_ERR_INVALID_ARG, "noise bricks: fill must be in (0, 1)");
  const uint32_t s32 = uint32_t(seed ^ (seed >> 32));
  const uint32_t ns = 1u << 16;
  DBuf<float> smp(ns, st);
  k_noise_samples<<<64, 256, 0, st>>>(1u << depth, s32, ns, smp.get());
  SVDAG_CUDA(cudaPeekAtLastError());
  std::vector<float> h(ns);
  SVDAG_CUDA(cudaMemcpyAsync(h.data(), smp.get(), 4ull * ns, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  const size_t k = std::min<size_t>(ns - 1, size_t(fill * ns));
  std::nth_element(h.begin(), h.begin() + k, h.end());
  const float thr = h[k];
  const uint64_t nb = 1ull << (3 * (depth - 1));
  k_noise_bricks<<<unsigned(std::min<uint64_t>((nb + 255) / 256, 152ull * 16)), 256, 0, st>>>(nb, s32, thr, out);
  SVDAG_CUDA(cudaPeekAtLastError());
  return thr;
}

void phase_import_bricks(Ctx& c, uint32_t depth, const uint8_t* bricks) {
  if (depth < 2 || depth > 11) throw Error(SVDAG_ERR_INVALID_ARG, "import_bricks: depth must be in [2, 11]");
  if (!bricks || (reinterpret_cast<uintptr_t>(bricks) & 7u))
    throw Error(SVDAG_ERR_INVALID_ARG, "import_bricks: bricks must be a device pointer aligned to 8 bytes");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  c.levels = depth;
  c.lev.clear();
  c.lev.resize(depth);
  c.child_levels_init = false;
  DBuf<uint32_t> idx, up, d_n(1, st);
  DBuf<unsigned long long> d_vox(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_vox.get(), 0, 8, st));
  // leaves
  uint64_t cells = 1ull << (3 * (depth - 1));
  idx.alloc(cells, st);
  device_exclusive_scan<uint32_t>(ex, BrickNonEmpty{bricks}, cells, IndexOut{idx.get(), bricks, nullptr, false},
                                  d_n.get());
  uint64_t n = read_scalar(ex, d_n.get());
  {
    Level& L = c.lev[depth - 1];
    L.n = n;
    L.hdr.alloc(n ? n : 1, st);
    SVDAG_LAUNCH(ex, k_leaf_nodes, grid_for(ex, cells, 256), 256, 0, bricks, cells, idx.get(), L.hdr.get(), d_vox.get());
  }
  for (int l = int(depth) - 2; l >= 0; --l) {
    cells >>= 3;
    up.alloc(cells, st);
    device_exclusive_scan<uint32_t>(ex, CellNonEmpty{idx.get(), l == 0}, cells,
                                    IndexOut{up.get(), nullptr, idx.get(), l == 0}, d_n.get());
    n = read_scalar(ex, d_n.get());
    Level& L = c.lev[l];
    L.n = n;
    L.hdr.alloc(n ? n : 1, st);
    L.ch.alloc(8 * (n ? n : 1), st);
    SVDAG_LAUNCH(ex, k_inner_nodes, grid_for(ex, cells, 256), 256, 0, idx.get(), cells, up.get(), L.hdr.get(),
                 L.ch.get());
    std::swap(idx, up);
  }
  uint64_t nodes = 0;
  for (uint32_t l = 0; l < depth; ++l) nodes += c.lev[l].n;
  c.st = svdag_stats{};
  c.st.levels = depth;
  c.st.n_total_voxels = read_scalar(ex, d_vox.get());
  c.st.n_nodes = nodes;
  c.st.n_nodes_dag = nodes;
  c.state = SVDAG_S_DAG;  // the NodeData constructor's state
}

// ---------------------------------------------------------------------------
namespace {

// One wave of chunks (sel = their indices in B.chunks), all heights.
void build_wave(Batch& B, const std::vector<uint32_t>& sel) {
  const Exec& ex = B.ex;
  const cudaStream_t st = B.stream;
  const uint32_t N = uint32_t(sel.size());
  if (!N) return;
  auto CH = [&](uint32_t c) -> const BatchChunk& { return B.chunks[sel[c]]; };
  auto RES = [&](uint32_t c) -> BatchResult& { return B.results[sel[c]]; };
  uint32_t maxd = 0;
  for (uint32_t c = 0; c < N; ++c) maxd = std::max(maxd, CH(c).depth);

  // --- leaf height: per-chunk first occurrence of every mask
  std::vector<const uint8_t*> hb(N);
  std::vector<uint64_t> hn(N);
  for (uint32_t c = 0; c < N; ++c) { hb[c] = CH(c).bricks; hn[c] = 1ull << (3 * (CH(c).depth - 1)); }
  DBuf<const uint8_t*> d_bricks(N, st);
  DBuf<uint64_t> d_nb(N, st);
  DBuf<uint32_t> first(256ull * N, st), rank(256ull * N, st), leaf_hdr(256ull * N, st), leaf_cnt(N, st);
  DBuf<unsigned long long> vox(N, st);
  DBuf<int> d_err(1, st), d_retry(1, st);
  SVDAG_CUDA(cudaMemcpyAsync(d_bricks.get(), hb.data(), sizeof(void*) * N, cudaMemcpyHostToDevice, st));
  SVDAG_CUDA(cudaMemcpyAsync(d_nb.get(), hn.data(), 8ull * N, cudaMemcpyHostToDevice, st));
  SVDAG_CUDA(cudaMemsetAsync(first.get(), 0xFF, 4 * 256ull * N, st));
  SVDAG_CUDA(cudaMemsetAsync(vox.get(), 0, 8ull * N, st));
  SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, st));
  SVDAG_CUDA(cudaMemsetAsync(d_retry.get(), 0, 4, st));
  // SVDAG_BATCH_TABLE_SHARE replaces the learned distinct-key shares (every
  // height) with a fixed one: small values force the full-size rebuild
  double share_env = 0;
  if (const char* e = std::getenv("SVDAG_BATCH_TABLE_SHARE")) share_env = std::atof(e);
  {
    uint64_t mx = 0;
    for (auto v : hn) mx = std::max(mx, v);
    const unsigned gx = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((mx / 8 + 255) / 256, 2048)));
    SVDAG_LAUNCH(ex, k_batch_leaf_first, dim3(gx, N), 256, 0, d_bricks.get(), d_nb.get(), first.get(), vox.get());
  }
  SVDAG_LAUNCH(ex, k_batch_leaf_rank, N, 256, 0, first.get(), rank.get(), leaf_hdr.get(), leaf_cnt.get());
  std::vector<uint32_t> h_leaf_cnt(N);
  std::vector<unsigned long long> h_vox(N);
  SVDAG_CUDA(cudaMemcpyAsync(h_leaf_cnt.data(), leaf_cnt.get(), 4ull * N, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaMemcpyAsync(h_vox.data(), vox.get(), 8ull * N, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  for (uint32_t c = 0; c < N; ++c) {
    BatchResult& R = RES(c);
    const uint32_t d = CH(c).depth;
    R.dag.reset(new svdag_ctx());
    Ctx& X = R.dag->c;
    X.device = B.device;
    X.stream = st;
    X.ex = B.ex;
    X.levels = d;
    X.lev.resize(d);
    X.state = SVDAG_S_DAG;
    X.st = svdag_stats{};
    X.st.levels = d;
    X.st.n_total_voxels = h_vox[c];
    Level& L = X.lev[d - 1];
    L.n = h_leaf_cnt[c];
    L.hdr.alloc(L.n ? L.n : 1, st);
    if (L.n)
      SVDAG_CUDA(cudaMemcpyAsync(L.hdr.get(), leaf_hdr.get() + 256ull * c, 4ull * L.n, cudaMemcpyDeviceToDevice, st));
  }

  // --- heights 1 .. maxd-1
  DBuf<uint32_t> below_ids;  // DAG ids of the cells one height down
  std::vector<uint64_t> below_base_h;
  std::vector<uint32_t> below_part;
  for (uint32_t h = 1; h < maxd; ++h) {
    std::vector<uint32_t> part;
    std::vector<uint64_t> base{0};
    std::vector<uint8_t> top;
    std::vector<const uint8_t*> pb;
    std::vector<uint64_t> bb;  // below base per entry
    // entries deepest first, so every entry's cell range starts on a multiple
    // of 8 except the single root cells at the end (16-byte child-id loads)
    std::vector<uint32_t> order(N);
    for (uint32_t c = 0; c < N; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return CH(a).depth > CH(b).depth; });
    for (uint32_t c : order) {
      const uint32_t d = CH(c).depth;
      if (d <= h) continue;
      const uint32_t l = d - 1 - h;
      part.push_back(c);
      base.push_back(base.back() + (1ull << (3 * l)));
      top.push_back(l == 0 ? 1 : 0);
      pb.push_back(CH(c).bricks);
      if (h >= 2) {
        const size_t k = size_t(std::find(below_part.begin(), below_part.end(), c) - below_part.begin());
        bb.push_back(below_base_h[k]);
      } else {
        bb.push_back(0);
      }
    }
    const uint32_t n = uint32_t(part.size());
    const uint64_t total = base.back();
    if (total > kGMask) throw Error(SVDAG_ERR_OVERFLOW, "batch: more than 2^40 cells on one height");
    DBuf<uint64_t> d_base(n + 1, st), d_bb(n, st);
    DBuf<uint32_t> d_part(n, st);
    DBuf<uint8_t> d_top(n, st);
    DBuf<const uint8_t*> d_pb(n, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_base.get(), base.data(), 8ull * (n + 1), cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_bb.get(), bb.data(), 8ull * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_part.get(), part.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_top.get(), top.data(), n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_pb.get(), pb.data(), sizeof(void*) * n, cudaMemcpyHostToDevice, st));
    HeightView V;
    V.cells = ChunkSet{d_base.get(), n};
    V.part = d_part.get();
    V.bricks = d_pb.get();
    V.leaf_rank = rank.get();
    V.below_base = d_bb.get();
    V.below_ids = below_ids.get();
    V.is_top = d_top.get();
    V.h = h;

    // Hash table: load <= 1 / B.tuning.table_factor over every cell of the
    // height (full size), or over twice the largest share of distinct keys
    // that earlier waves and builds saw at this height -- the distinct keys
    // are a few per cent of the cells on the lowest heights, so the table is
    // much smaller to clear and to probe.  An insert into the smaller table
    // that probes kProbeLimit slots in vain sets d_retry, and the height is
    // redone with the full-size table.
    const unsigned tb = B.tuning.threads;
    if (total >= (1ull << 32)) throw Error(SVDAG_ERR_OVERFLOW, "batch: more than 2^32 cells on one height");
    const uint64_t full = std::min<uint64_t>(
        kMaxTableSlots, next_pow2(uint64_t(double(std::max<uint64_t>(total, 16)) * B.tuning.table_factor)));
    const double share = share_env > 0 ? share_env : (h < B.distinct_share.size() ? B.distinct_share[h] : 0.0);
    uint64_t size = full;
    if (share > 0) {
      const double keys = std::max(2.0 * share * double(total), 65536.0);
      size = std::min(full, next_pow2(uint64_t(keys * B.tuning.table_factor)));
    }
    // the slot of each cell's key, then its representative (kNone: empty
    // cell), in 32 bits: cell indices of a height are below 2^32 (checked
    // above) and tables are capped at 2^31 slots
    DBuf<uint32_t> rep(total, st);
    const uint64_t words = (total + 31) / 32;
    DBuf<uint32_t> flags(words, st), woff(words, st);
    DBuf<uint32_t> d_total(1, st), d_bases(n + 1, st);
    auto dedup = [&](uint64_t tsize) {
      const bool bounded = tsize < full;
      DBuf<unsigned long long> slots(tsize, st);
      SVDAG_CUDA(cudaMemsetAsync(slots.get(), 0xFF, 8 * tsize, st));
      const uint64_t lim = bounded ? std::min<uint64_t>(kProbeLimit, tsize - 1) : tsize - 1;
      int* flag = bounded ? d_retry.get() : d_err.get();
      if (h == 1)
        SVDAG_LAUNCH(ex, k_batch_insert_h1, grid_for(ex, total, tb, 8), tb, 0, V, total, slots.get(), tsize - 1, lim,
                     rep.get(), flag);
      else
        SVDAG_LAUNCH(ex, k_batch_insert, grid_for(ex, total, tb, 8), tb, 0, V, total, slots.get(), tsize - 1, lim,
                     rep.get(), flag);
      SVDAG_LAUNCH(ex, k_batch_rep, grid_for(ex, total, tb, 8), tb, 0, total, slots.get(), tsize - 1,
                   bounded ? d_retry.get() : nullptr, rep.get(), flags.get());
      slots.release();
      // node numbers: a scan over the flag words' popcounts (32 cells each)
      device_exclusive_scan<uint32_t>(ex, FlagPopc{flags.get()}, words, U32Out{woff.get()}, d_total.get());
      SVDAG_LAUNCH(ex, k_entry_bases, 1, 256, 0, n, d_base.get(), flags.get(), woff.get(), d_total.get(),
                   d_bases.get());
    };
    // DAG nodes of each entry: the node numbers from its first cell's to the
    // next entry's; read together with the retry flag (one synchronisation)
    std::vector<uint64_t> rep_base(n + 1);
    auto read_bases = [&]() -> bool {
      std::vector<uint32_t> h_nid(n + 1);
      int retry = 0;
      SVDAG_CUDA(cudaMemcpyAsync(h_nid.data(), d_bases.get(), 4ull * (n + 1), cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaMemcpyAsync(&retry, d_retry.get(), 4, cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
      for (uint32_t e = 0; e <= n; ++e) rep_base[e] = h_nid[e];
      return retry == 0;
    };
    dedup(size);
    if (!read_bases()) {
      ++B.table_retries;
      SVDAG_CUDA(cudaMemsetAsync(d_retry.get(), 0, 4, st));
      dedup(full);
      read_bases();
    }
    if (B.distinct_share.size() <= h) B.distinct_share.resize(h + 1, 0.0);
    B.distinct_share[h] = std::max(B.distinct_share[h], double(rep_base[n]) / double(total));
    DBuf<uint64_t> d_rep_base(n, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_rep_base.get(), rep_base.data(), 8ull * n, cudaMemcpyHostToDevice, st));
    // each entry's level, sized now that its node count is known; the emit
    // kernel fills them in place
    std::vector<uint32_t*> h_hdr(n), h_ch(n);
    for (uint32_t e = 0; e < n; ++e) {
      const uint32_t c = part[e];
      Ctx& X = RES(c).dag->c;
      Level& L = X.lev[CH(c).depth - 1 - h];
      L.n = rep_base[e + 1] - rep_base[e];
      L.hdr.alloc(L.n ? L.n : 1, st);
      L.ch.alloc(8 * (L.n ? L.n : 1), st);
      h_hdr[e] = L.hdr.get();
      h_ch[e] = L.ch.get();
    }
    DBuf<uint32_t*> d_hdr(n, st), d_ch(n, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_hdr.get(), h_hdr.data(), sizeof(uint32_t*) * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_ch.get(), h_ch.data(), sizeof(uint32_t*) * n, cudaMemcpyHostToDevice, st));
    DBuf<uint32_t> ids(total, st);
    SVDAG_LAUNCH(ex, k_batch_emit, grid_for(ex, total, tb, 8), tb, 0, V, total, rep.get(), flags.get(), woff.get(),
                 d_rep_base.get(), ids.get(), d_hdr.get(), d_ch.get());
    below_ids = std::move(ids);
    below_base_h.assign(base.begin(), base.end() - 1);
    below_part = part;
  }
  check_err(ex, d_err.get(), "batch toDAG");
  for (uint32_t c = 0; c < N; ++c) {
    Ctx& X = RES(c).dag->c;
    uint64_t nodes = 0;
    for (auto& L : X.lev) nodes += L.n;
    X.st.n_nodes = nodes;
    X.st.n_nodes_dag = nodes;
  }
}

}  // namespace

// All chunks, in waves of at most 2^30 cells one height above the leaves
// (bounds the per-height tables and index arrays to a few tens of GB).
void batch_build_dags(Batch& B) {
  const uint32_t N = uint32_t(B.chunks.size());
  B.results.clear();
  B.results.resize(N);
  std::vector<uint32_t> sel;
  uint64_t cells = 0;
  auto flush = [&]() {
    if (sel.empty()) return;
    build_wave(B, sel);
    sel.clear();
    cells = 0;
  };
  for (uint32_t c = 0; c < N; ++c) {
    const uint64_t k = 1ull << (3 * (B.chunks[c].depth - 2));
    if (!sel.empty() && cells + k > (1ull << 30)) flush();
    sel.push_back(c);
    cells += k;
  }
  flush();
}

namespace {

// Chunks for the SSVDAG / CSVDAG reduction workers.
struct ReduceQueue {
  std::mutex mu;
  std::condition_variable cv;
  std::vector<uint32_t> items;
  size_t next = 0;
  bool closed = false;
  int err_code = SVDAG_OK;
  std::string err;
  std::atomic<unsigned> cap{1};  // SMs per reduction grid
  void push(const std::vector<uint32_t>& sel) {
    {
      std::lock_guard<std::mutex> lk(mu);
      items.insert(items.end(), sel.begin(), sel.end());
    }
    cv.notify_all();
  }
  void close() {
    {
      std::lock_guard<std::mutex> lk(mu);
      closed = true;
    }
    cv.notify_all();
  }
  void fail(int code, const std::string& what) {
    {
      std::lock_guard<std::mutex> lk(mu);
      if (err_code == SVDAG_OK) { err_code = code; err = what; }
    }
    cv.notify_all();
  }
  // next ready chunk; false once the queue is closed and drained, or failed
  bool pop(uint32_t& c) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return next < items.size() || closed || err_code != SVDAG_OK; });
    if (err_code != SVDAG_OK || next >= items.size()) return false;
    c = items[next++];
    return true;
  }
};

// One worker: clones of each ready chunk's DAG on its own stream, reduced
// with grids of at most q.cap SMs.
void reduce_worker(Batch& B, ReduceQueue& q, int w, bool sdag, bool csv) {
  const cudaStream_t sw = B.streams[w];
  try {
    SVDAG_CUDA(cudaSetDevice(B.device));
    uint32_t c;
    while (q.pop(c)) {
      BatchResult& R = B.results[c];
      auto clone_of = [&](const svdag_ctx* src) {
        std::unique_ptr<svdag_ctx> o(new svdag_ctx());
        Ctx& X = o->c;
        const Ctx& S = src->c;
        X.device = S.device;
        X.stream = sw;
        X.ex = B.ex;
        X.ex.stream = sw;
        X.ex.launches = &B.worker_launches[w];
        X.ex.prof = nullptr;
        X.ex.persistent_blocks = q.cap.load();
        X.levels = S.levels;
        X.state = S.state;
        X.st = S.st;
        X.lev.resize(S.lev.size());
        for (size_t l = 0; l < S.lev.size(); ++l) {
          const Level& a = S.lev[l];
          Level& b = X.lev[l];
          b.n = a.n;
          b.hdr.alloc(a.n ? a.n : 1, sw);
          if (a.n) SVDAG_CUDA(cudaMemcpyAsync(b.hdr.get(), a.hdr.get(), 4 * a.n, cudaMemcpyDeviceToDevice, sw));
          if (a.ch.get()) {
            b.ch.alloc(8 * (a.n ? a.n : 1), sw);
            if (a.n) SVDAG_CUDA(cudaMemcpyAsync(b.ch.get(), a.ch.get(), 32 * a.n, cudaMemcpyDeviceToDevice, sw));
          }
        }
        return o;
      };
      if (sdag) {
        R.sdag = clone_of(R.dag.get());
        phase_reduce_sdag(R.sdag->c);
      }
      if (csv && R.dag->c.levels >= 2) {
        R.csv = clone_of(R.dag.get());
        R.csv->c.child_levels_init = true;  // initChildLevels before the merge, as svbuilder does
        phase_cross_level_merge(R.csv->c);
      }
      SVDAG_CUDA(cudaStreamSynchronize(sw));
    }
  } catch (const Error& e) {
    q.fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    q.fail(SVDAG_ERR_OOM, "host allocation failed");
  }
}

// Worker streams live as long as the batch: the results' buffers are
// stream-ordered allocations on them.
int reduce_streams(Batch& B, uint32_t n_chunks) {
  const int W = std::max(1, std::min<int>(B.tuning.streams, int(std::max<uint32_t>(n_chunks, 1))));
  while (int(B.streams.size()) < W) {
    cudaStream_t s;
    SVDAG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    B.streams.push_back(s);
  }
  B.worker_launches.assign(W, 0);
  return W;
}

}  // namespace

// SSVDAG and CSVDAG of every chunk's DAG, on B.tuning.streams streams.
void batch_reduce(Batch& B, bool sdag, bool csv) {
  const uint32_t N = uint32_t(B.results.size());
  if (!N || (!sdag && !csv)) return;
  SVDAG_CUDA(cudaStreamSynchronize(B.stream));
  const int W = reduce_streams(B, N);
  ReduceQueue q;
  std::vector<uint32_t> all(N);
  for (uint32_t c = 0; c < N; ++c) all[c] = c;
  q.push(all);
  q.close();
  // W streams run persistent toSDAG / merge kernels side by side: each grid
  // takes at most its share of the SMs (one block per SM)
  q.cap = std::max(1u, unsigned(B.ex.sm_count / W));
  std::vector<std::thread> th;
  for (int w = 1; w < W; ++w) th.emplace_back(reduce_worker, std::ref(B), std::ref(q), w, sdag, csv);
  reduce_worker(B, q, 0, sdag, csv);
  for (auto& t : th) t.join();
  for (auto v : B.worker_launches) B.launches += v;
  if (q.err_code != SVDAG_OK) throw Error(q.err_code, q.err);
}

}  // namespace svdag

// ---------------------------------------------------------------------------
// C ABI (include/svdag_gpu.h)
namespace {

using svdag::Batch;
using svdag::Error;

template <class F>
int batch_guarded(svdag_batch* h, F&& f) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  try {
    SVDAG_CUDA(cudaSetDevice(h->b.device));
    f(h->b);
    h->b.last_error.clear();
    return SVDAG_OK;
  } catch (const Error& e) {
    h->b.last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    h->b.last_error = "host allocation failed";
    return SVDAG_ERR_OOM;
  } catch (const std::exception& e) {
    h->b.last_error = e.what();
    return SVDAG_ERR_CUDA;
  }
}

double wall_ms(const std::chrono::steady_clock::time_point& t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// The two stages one after the other: overlapping them (each wave's chunks
// reduced while the next wave builds, the SMs split between the two) was
// slower on GB300 -- 1364 against 1080 ms for the 256-chunk benchmark --
// as the DAG waves slowed from 555 to 1298 ms next to the reductions.
void run_batch(Batch& B, uint32_t flags) {
  const auto t0 = std::chrono::steady_clock::now();
  svdag::batch_build_dags(B);
  SVDAG_CUDA(cudaStreamSynchronize(B.stream));
  B.dag_ms = wall_ms(t0);
  const auto t1 = std::chrono::steady_clock::now();
  svdag::batch_reduce(B, (flags & SVDAG_BATCH_SDAG) != 0, (flags & SVDAG_BATCH_CSVDAG) != 0);
  B.reduce_ms = wall_ms(t1);
}


}  // namespace

extern "C" {

int svdag_synth_noise_bricks(void* stream, uint32_t depth, uint64_t seed, double fill, uint8_t* device_bricks,
                             float* threshold) {
  if (!device_bricks) return SVDAG_ERR_INVALID_ARG;
  try {
    const float t = svdag::synth_noise_bricks(static_cast<cudaStream_t>(stream), depth, seed, fill, device_bricks);
    if (threshold) *threshold = t;
    return SVDAG_OK;
  } catch (const Error& e) {
    return e.code;
  } catch (const std::exception&) {
    return SVDAG_ERR_CUDA;
  }
}

int svdag_import_bricks(svdag_ctx* h, uint32_t depth, const uint8_t* device_bricks) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    SVDAG_CUDA(cudaEventRecord(c.ev0, c.stream));
    svdag::phase_import_bricks(c, depth, device_bricks);
    SVDAG_CUDA(cudaEventRecord(c.ev1, c.stream));
    SVDAG_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    SVDAG_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.st.svo_ms = double(ms);
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return SVDAG_ERR_CUDA;
  }
}

int svdag_batch_create(svdag_batch** out, int device, void* stream) {
  if (!out) return SVDAG_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return SVDAG_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return SVDAG_ERR_INVALID_ARG;
  svdag_batch* h = new (std::nothrow) svdag_batch();
  if (!h) return SVDAG_ERR_OOM;
  Batch& B = h->b;
  B.device = device;
  if (cudaSetDevice(device) != cudaSuccess) { delete h; return SVDAG_ERR_CUDA; }
  if (stream) {
    B.stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return SVDAG_ERR_CUDA; }
    B.own_stream = true;
  }
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  // keep freed blocks of the stream-ordered allocator cached between waves
  // and builds (as svdag_create does): every wave allocates and frees tens
  // of GB, which the pool would otherwise unmap and map again each time
  cudaMemPool_t pool;
  uint64_t keep = ~0ull;
  if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess ||
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
    if (B.own_stream) cudaStreamDestroy(B.stream);
    delete h;
    return SVDAG_ERR_CUDA;
  }
  B.ex.stream = B.stream;
  B.ex.sm_count = sms;
  B.ex.launches = &B.launches;
  *out = h;
  return SVDAG_OK;
}

int svdag_batch_destroy(svdag_batch* h) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  Batch& B = h->b;
  cudaSetDevice(B.device);
  cudaDeviceSynchronize();
  B.results.clear();
  for (auto s : B.streams) cudaStreamDestroy(s);
  if (B.own_stream) cudaStreamDestroy(B.stream);
  delete h;
  return SVDAG_OK;
}

const char* svdag_batch_last_error(const svdag_batch* h) { return h ? h->b.last_error.c_str() : "null batch"; }

int svdag_batch_clear(svdag_batch* h) {
  return batch_guarded(h, [&](Batch& B) {
    SVDAG_CUDA(cudaStreamSynchronize(B.stream));
    B.results.clear();
    B.chunks.clear();
  });
}

int svdag_batch_add_chunk(svdag_batch* h, uint32_t depth, const uint8_t* device_bricks) {
  return batch_guarded(h, [&](Batch& B) {
    if (depth < 2 || depth > 11) throw Error(SVDAG_ERR_INVALID_ARG, "batch: chunk depth must be in [2, 11]");
    if (!device_bricks || (reinterpret_cast<uintptr_t>(device_bricks) & 7u))
      throw Error(SVDAG_ERR_INVALID_ARG, "batch: bricks must be a device pointer aligned to 8 bytes");
    B.chunks.push_back(svdag::BatchChunk{depth, device_bricks});
  });
}

int svdag_batch_chunk_count(const svdag_batch* h, uint32_t* n) {
  if (!h || !n) return SVDAG_ERR_INVALID_ARG;
  *n = uint32_t(h->b.chunks.size());
  return SVDAG_OK;
}

int svdag_batch_build(svdag_batch* h, uint32_t flags) {
  return batch_guarded(h, [&](Batch& B) { run_batch(B, flags); });
}

int svdag_batch_result(svdag_batch* h, uint32_t chunk, uint32_t kind, svdag_ctx** view) {
  return batch_guarded(h, [&](Batch& B) {
    if (!view) throw Error(SVDAG_ERR_INVALID_ARG, "batch_result: null view");
    if (chunk >= B.results.size()) throw Error(SVDAG_ERR_INVALID_ARG, "batch_result: no such chunk (build first)");
    svdag::BatchResult& R = B.results[chunk];
    svdag_ctx* v = kind == SVDAG_BATCH_RESULT_DAG ? R.dag.get()
                   : kind == SVDAG_BATCH_RESULT_SDAG ? R.sdag.get()
                   : kind == SVDAG_BATCH_RESULT_CSVDAG ? R.csv.get() : nullptr;
    if (!v) throw Error(SVDAG_ERR_INVALID_STATE, "batch_result: this result was not built");
    *view = v;
  });
}

int svdag_batch_set_tuning(svdag_batch* h, const svdag_batch_tuning* t) {
  return batch_guarded(h, [&](Batch& B) {
    if (!t || !(t->table_factor >= 1.25 && t->table_factor <= 16.0) || t->threads < 64 || t->threads > 1024 ||
        (t->threads & 31u) || t->streams < 1 || t->streams > 64)
      throw Error(SVDAG_ERR_INVALID_ARG, "batch tuning out of range");
    B.tuning.table_factor = t->table_factor;
    B.tuning.threads = t->threads;
    B.tuning.streams = int(t->streams);
  });
}

int svdag_batch_get_tuning(const svdag_batch* h, svdag_batch_tuning* t) {
  if (!h || !t) return SVDAG_ERR_INVALID_ARG;
  t->table_factor = h->b.tuning.table_factor;
  t->threads = h->b.tuning.threads;
  t->streams = uint32_t(h->b.tuning.streams);
  return SVDAG_OK;
}

// Coordinate search over the three settings on the current chunks (each trial
// is a full build); keeps the fastest and leaves its results in place.
int svdag_batch_autotune(svdag_batch* h, uint32_t flags, uint32_t max_trials) {
  return batch_guarded(h, [&](Batch& B) {
    auto trial = [&]() {
      const auto t0 = std::chrono::steady_clock::now();
      run_batch(B, flags);
      return wall_ms(t0);
    };
    uint32_t trials = 0;
    double best = trial();
    ++trials;
    const double tf[] = {1.5, 2.0, 3.0, 4.0};
    const unsigned th[] = {128, 256, 512};
    const int sm[] = {1, 2, 4, 8, 16};
    for (int pass = 0; pass < 2 && trials < max_trials; ++pass) {
      for (double v : tf) {
        if (trials >= max_trials || v == B.tuning.table_factor) continue;
        const double old = B.tuning.table_factor;
        B.tuning.table_factor = v;
        const double t = trial();
        ++trials;
        if (t < best) best = t; else B.tuning.table_factor = old;
      }
      for (unsigned v : th) {
        if (trials >= max_trials || v == B.tuning.threads) continue;
        const unsigned old = B.tuning.threads;
        B.tuning.threads = v;
        const double t = trial();
        ++trials;
        if (t < best) best = t; else B.tuning.threads = old;
      }
      for (int v : sm) {
        if (trials >= max_trials || v == B.tuning.streams) continue;
        const int old = B.tuning.streams;
        B.tuning.streams = v;
        const double t = trial();
        ++trials;
        if (t < best) best = t; else B.tuning.streams = old;
      }
    }
    run_batch(B, flags);  // results of the chosen setting
  });
}

int svdag_batch_get_stats(const svdag_batch* h, svdag_batch_stats* out) {
  if (!h || !out) return SVDAG_ERR_INVALID_ARG;
  out->dag_ms = h->b.dag_ms;
  out->reduce_ms = h->b.reduce_ms;
  out->gpu_launches = h->b.launches;
  out->table_retries = h->b.table_retries;
  return SVDAG_OK;
}

}  // extern "C"
