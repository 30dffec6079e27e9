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

}  // namespace svdag

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
