// EncodedSVDAG / EncodedUSSVDAG streams on the GPU
// (src/symvox/encoded_svdag.cpp:105-199, encoded_ussvdag.cpp:86-170).
//
// Both formats are one u32 stream with the nodes in level order: a header
// word (the child mask; USSVDAG adds the three mirror masks above it), then
// for inner nodes one absolute word offset per existing child, children
// 7..0; leaves are the header word alone.  A node's offset is the exclusive
// prefix of the word counts (1 + child pointers, or 1 on the leaf level) over
// all earlier nodes, so the stream is one scan and one scatter.  Child
// pointers follow the child level (childLevels after a cross-level merge,
// else the next level); a CSVDAG pointer the merge left unresolved
// (0xFFFFFFFF) is written as 0xFFFFFFFF, as the host encoder does.  The
// reference writes the total word count as its "first leaf pointer" field.
#include <algorithm>
#include <utility>

#include "ctx.cuh"

namespace svdag {
namespace {

struct EncLevels {
  const uint32_t* hdr[32];
  const uint32_t* ch[32];
  const uint8_t* clev[32];
  uint64_t off[33];  // first global node index of each level
  uint32_t levels;
};

__device__ __forceinline__ uint32_t level_of_node(const EncLevels& E, uint64_t g) {
  uint32_t l = 0;
  while (l + 1 < E.levels && E.off[l + 1] <= g) ++l;
  return l;
}

struct WordsIn {
  EncLevels E;
  __device__ __forceinline__ uint64_t operator()(uint64_t g) const {
    const uint32_t l = level_of_node(E, g);
    if (l + 1 >= E.levels) return 1;
    const uint64_t i = g - E.off[l];
    uint64_t w = 1;
#pragma unroll
    for (int k = 0; k < 8; ++k) w += (E.ch[l][8 * i + k] != kNull) ? 1 : 0;
    return w;
  }
};
struct PtrOut {
  uint32_t* ptr;
  __device__ __forceinline__ void operator()(uint64_t g, uint64_t v) const { ptr[g] = uint32_t(v); }
};

__global__ void k_encode(EncLevels E, uint64_t n, const uint32_t* __restrict__ ptr, int ussvdag, int init_levels,
                         uint32_t* __restrict__ out) {
  for (uint64_t g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; g < n; g += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t l = level_of_node(E, g);
    const uint64_t i = g - E.off[l];
    const uint32_t h = E.hdr[l][i];
    uint32_t p = ptr[g];
    out[p++] = ussvdag ? h : (h & 0xFFu);
    if (l + 1 >= E.levels) continue;
    for (int k = 7; k >= 0; --k) {
      const uint32_t c = E.ch[l][8 * i + k];
      if (c == kNull) continue;
      uint32_t tl = l + 1;
      if (E.clev[l]) tl = E.clev[l][8 * i + k];
      else if (!init_levels) tl = l + 1;
      const uint64_t tg = (tl == 0 ? 0 : E.off[tl]) + uint64_t(c);
      out[p++] = (c != 0xFFFFFFFFu && tl < E.levels && tg < E.off[E.levels]) ? ptr[tg] : 0xFFFFFFFFu;
    }
  }
}

}  // namespace

// Stream of the context's octree; returns the word count.  out may be null
// (size query).
uint64_t encode_stream(Ctx& c, bool ussvdag, uint32_t* host_out, uint64_t capacity) {
  if (ussvdag && c.state != SVDAG_S_SDAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "encode: USSVDAG needs an SDAG (encoded_ussvdag.cpp:90-93)");
  if (!ussvdag && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "encode: SVDAG needs a DAG (encoded_svdag.cpp:109-112)");
  if (c.levels > 32) throw Error(SVDAG_ERR_INVALID_ARG, "encode: too many levels");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  EncLevels E{};
  E.levels = c.levels;
  uint64_t n = 0;
  bool explicit_levels = false;
  for (uint32_t l = 0; l < c.levels; ++l) {
    E.off[l] = n;
    E.hdr[l] = c.lev[l].hdr.get();
    E.ch[l] = c.lev[l].ch.get();
    E.clev[l] = c.lev[l].clev.get();
    explicit_levels = explicit_levels || E.clev[l];
    n += c.lev[l].n;
  }
  E.off[c.levels] = n;
  if (!ussvdag && !c.child_levels_init && !explicit_levels)
    throw Error(SVDAG_ERR_INVALID_STATE, "encode: child levels not initialised (initChildLevels)");
  DBuf<uint32_t> ptr(n ? n : 1, st);
  DBuf<uint64_t> d_total(1, st);
  device_exclusive_scan<uint64_t>(ex, WordsIn{E}, n, PtrOut{ptr.get()}, d_total.get());
  const uint64_t words = read_scalar(ex, d_total.get());
  if (words >= (1ull << 32)) throw Error(SVDAG_ERR_OVERFLOW, "encode: stream above 2^32 words");
  if (!host_out) return words;
  if (capacity < words) throw Error(SVDAG_ERR_INVALID_ARG, "encode: output buffer too small");
  DBuf<uint32_t> out(words ? words : 1, st);
  if (n)
    SVDAG_LAUNCH(ex, k_encode, grid_for(ex, n, 256), 256, 0, E, n, ptr.get(), ussvdag ? 1 : 0,
                 c.child_levels_init ? 1 : 0, out.get());
  if (words) SVDAG_CUDA(cudaMemcpyAsync(host_out, out.get(), 4 * words, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  return words;
}

// ---------------------------------------------------------------------------
// EncodedSSVDAG::encode (src/symvox/encoded_ssvdag.cpp:194-466).  Bottom-up
// from the level above the leaves: each level's nodes are ordered by how many
// pointers reach them from the level above, in the order the reference's
// std::sort over (index, count) pairs leaves them -- an unstable sort whose
// order for equal counts is libstdc++'s introsort's, reproduced on the GPU
// (refsort.cu).  The level above the leaves becomes 4^3 bricks of 8 bytes (the 8
// children's masks, mirrored, in voxel-matrix order: octree voxel (X, Y, Z)
// of the brick at bit Z + 4Y + 16X); every other level becomes u16 nodes (a
// header with 2 bits per child, then 16- or 32-bit pointers, high half
// first, carrying the mirror bits) whose word offsets are a scan of their
// sizes in the sorted order.
namespace {

__global__ void k_ss_refcount(const uint32_t* __restrict__ pch, uint64_t np, uint32_t* __restrict__ cnt) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < np; i += uint64_t(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t k = pch[8 * i + c];
      if (k != kNull) atomicAdd(&cnt[k], 1u);
    }
  }
}

__global__ void k_ss_iota(uint32_t* __restrict__ perm, uint64_t n) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    perm[i] = uint32_t(i);
}

__device__ __forceinline__ uint32_t mirror_mask8(uint32_t m, uint32_t flip) {
  uint32_t r = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) r |= ((m >> c) & 1u) << (c ^ flip);
  return r;
}

// brick k = the node perm[k] of the level above the leaves
__global__ void k_ss_leaves(const uint32_t* __restrict__ perm, uint64_t n, const uint32_t* __restrict__ hdr,
                            const uint32_t* __restrict__ ch, const uint32_t* __restrict__ leaf_hdr,
                            uint32_t* __restrict__ addr, uint64_t* __restrict__ out) {
  for (uint64_t k = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; k < n; k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t i = perm[k];
    addr[i] = uint32_t(k);
    const uint32_t h = hdr[i];
    uint32_t buf[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t q = ch[8ull * i + c];
      const uint32_t flip = (((h >> (8 + c)) & 1u) << 2) | (((h >> (16 + c)) & 1u) << 1) | ((h >> (24 + c)) & 1u);
      buf[c] = q != kNull ? mirror_mask8(leaf_hdr[q] & 0xFFu, flip) : 0u;
    }
    uint64_t w = 0;
    for (int b = 0; b < 64; ++b) {  // b = x + 4y + 16z in the reference's matrix loop
      const int x = b & 3, y = (b >> 2) & 3, z = b >> 4;
      const int byte_id = (x >> 1) + 2 * (y >> 1) + 4 * (z >> 1), bit_id = (x & 1) + 2 * (y & 1) + 4 * (z & 1);
      w |= uint64_t((buf[byte_id] >> bit_id) & 1u) << b;
    }
    out[k] = w;
  }
}

struct SsSizeIn {
  const uint32_t* perm;
  const uint32_t* hdr;
  const uint32_t* ch;
  const uint32_t* child_addr;
  __device__ __forceinline__ uint32_t operator()(uint64_t k) const {
    const uint32_t i = perm[k];
    const uint32_t m = hdr[i] & 0xFFu;
    uint32_t w = 1;
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if ((m >> c) & 1u) w += child_addr[ch[8ull * i + c]] < (1u << 13) ? 1u : 2u;
    return w;
  }
};
struct U32Store {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};

__global__ void k_ss_inner(const uint32_t* __restrict__ perm, uint64_t n, const uint32_t* __restrict__ hdr,
                           const uint32_t* __restrict__ ch, const uint32_t* __restrict__ child_addr,
                           const uint32_t* __restrict__ woff, uint16_t* __restrict__ out, uint32_t* __restrict__ addr,
                           int* __restrict__ err) {
  for (uint64_t k = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; k < n; k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t i = perm[k];
    const uint32_t h = hdr[i];
    uint32_t o = woff[k];
    addr[i] = o;
    uint16_t* node = out + o;
    uint32_t head = 0;
    uint32_t p = o + 1;
    for (int c = 7; c >= 0; --c) {
      if (!((h >> c) & 1u)) continue;
      const uint32_t a = child_addr[ch[8ull * i + c]];
      const uint32_t mx = (h >> (8 + c)) & 1u, my = (h >> (16 + c)) & 1u, mz = (h >> (24 + c)) & 1u;
      if (a < (1u << 13)) {
        head |= 1u << (2 * c);
        out[p++] = uint16_t(a | (mx << 13) | (my << 14) | (mz << 15));
      } else if (a < (1u << 30)) {
        uint32_t v = a;
        if (v & (1u << 29)) {
          head |= 3u << (2 * c);
          v &= ~(1u << 29);
        } else {
          head |= 2u << (2 * c);
        }
        v |= (mx << 29) | (my << 30) | (mz << 31);
        out[p++] = uint16_t(v >> 16);
        out[p++] = uint16_t(v & 0xFFFFu);
      } else {
        atomicExch(err, 1);
      }
    }
    node[0] = uint16_t(head);
  }
}

}  // namespace

void encode_ssvdag(Ctx& c) {
  if (c.state != SVDAG_S_SDAG && c.state != SVDAG_S_DAG)
    throw Error(SVDAG_ERR_INVALID_STATE, "encode SSVDAG: needs a DAG or SDAG (encoded_ssvdag.cpp:218-221)");
  const uint32_t L = c.levels;
  if (L < 3) throw Error(SVDAG_ERR_INVALID_ARG, "encode SSVDAG: fewer than 3 levels");
  for (const Level& Lv : c.lev)
    if (Lv.clev.get())  // children on other levels: the format has no room for them
      throw Error(SVDAG_ERR_INVALID_STATE, "encode SSVDAG: the octree is cross-level merged");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  c.ss_inner.clear();
  c.ss_inner.resize(L - 2);
  c.ss_words.assign(L - 2, 0);
  DBuf<uint32_t> addr_child, addr_cur;
  DBuf<int> d_err(1, st);
  SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, st));
  for (int lev = int(L) - 2; lev >= 0; --lev) {
    const Level& Lv = c.lev[lev];
    const uint64_t n = Lv.n;
    if (n > (1ull << 30)) throw Error(SVDAG_ERR_OVERFLOW, "encode SSVDAG: a level above 2^30 nodes");
    // order: std::sort of (index, pointers reaching it) by count, descending
    // (reproduced on the device, refsort.cu); the root level keeps index order
    DBuf<uint32_t> perm(n ? n : 1, st);
    if (n && lev > 0) {
      DBuf<uint32_t> cnt(n, st);
      SVDAG_CUDA(cudaMemsetAsync(cnt.get(), 0, 4 * n, st));
      const Level& P = c.lev[lev - 1];
      if (P.n) SVDAG_LAUNCH(ex, k_ss_refcount, grid_for(ex, P.n, 256), 256, 0, P.ch.get(), P.n, cnt.get());
      refcount_order(ex, cnt.get(), n, perm.get());
    } else if (n) {
      SVDAG_LAUNCH(ex, k_ss_iota, grid_for(ex, n, 256), 256, 0, perm.get(), n);
    }
    addr_cur = DBuf<uint32_t>(n ? n : 1, st);
    if (lev == int(L) - 2) {
      c.ss_leaves = DBuf<uint64_t>(n ? n : 1, st);
      c.ss_bricks = n;
      if (n)
        SVDAG_LAUNCH(ex, k_ss_leaves, grid_for(ex, n, 256), 256, 0, perm.get(), n, Lv.hdr.get(), Lv.ch.get(),
                     c.lev[lev + 1].hdr.get(), addr_cur.get(), c.ss_leaves.get());
    } else {
      DBuf<uint32_t> woff(n ? n : 1, st);
      DBuf<uint32_t> d_total(1, st);
      device_exclusive_scan<uint32_t>(ex, SsSizeIn{perm.get(), Lv.hdr.get(), Lv.ch.get(), addr_child.get()}, n,
                                      U32Store{woff.get()}, d_total.get());
      const uint32_t words = read_scalar(ex, d_total.get());
      c.ss_words[lev] = words;
      c.ss_inner[lev] = DBuf<uint16_t>(words ? words : 1, st);
      if (n)
        SVDAG_LAUNCH(ex, k_ss_inner, grid_for(ex, n, 256), 256, 0, perm.get(), n, Lv.hdr.get(), Lv.ch.get(),
                     addr_child.get(), woff.get(), c.ss_inner[lev].get(), addr_cur.get(), d_err.get());
    }
    addr_child = std::move(addr_cur);
  }
  int err = 0;
  SVDAG_CUDA(cudaMemcpyAsync(&err, d_err.get(), 4, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  if (err) throw Error(SVDAG_ERR_OVERFLOW, "encode SSVDAG: a pointer above 2^30");
}

}  // namespace svdag

extern "C" int svdag_encode_ssvdag(svdag_ctx* h, uint64_t* n_inner_words, uint64_t* n_leaf_bytes,
                                   uint32_t* n_level_offsets) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    svdag::encode_ssvdag(c);
    uint64_t words = 0;
    for (uint64_t w : c.ss_words) words += w;
    if (n_inner_words) *n_inner_words = words;
    if (n_leaf_bytes) *n_leaf_bytes = 8 * c.ss_bricks;
    if (n_level_offsets) *n_level_offsets = uint32_t(c.ss_words.size());
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  }
}

extern "C" int svdag_download_ssvdag(svdag_ctx* h, uint16_t* inner, uint8_t* leaves, uint32_t* level_offsets) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    if (c.ss_words.empty()) throw svdag::Error(SVDAG_ERR_INVALID_STATE, "download SSVDAG: nothing encoded");
    uint64_t at = 0;
    for (size_t l = 0; l < c.ss_words.size(); ++l) {
      if (level_offsets) level_offsets[l] = uint32_t(at);
      if (inner && c.ss_words[l])
        SVDAG_CUDA(cudaMemcpyAsync(inner + at, c.ss_inner[l].get(), 2 * c.ss_words[l], cudaMemcpyDeviceToHost,
                                   c.stream));
      at += c.ss_words[l];
    }
    if (leaves && c.ss_bricks)
      SVDAG_CUDA(cudaMemcpyAsync(leaves, c.ss_leaves.get(), 8 * c.ss_bricks, cudaMemcpyDeviceToHost, c.stream));
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  }
}

extern "C" int svdag_encode(svdag_ctx* h, uint32_t format, uint32_t* host_words, uint64_t capacity, uint64_t* n_words) {
  if (!h || !n_words) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    if (format > SVDAG_FORMAT_USSVDAG) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "encode: unknown format");
    *n_words = svdag::encode_stream(c, format == SVDAG_FORMAT_USSVDAG, host_words, capacity);
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return SVDAG_ERR_CUDA;
  }
}
