// Shared device utilities of the SVDAG build: error handling, stream-ordered
// device buffers, launch accounting, node-key hashing and a device-wide
// exclusive scan.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "svdag_gpu.h"

namespace svdag {

constexpr uint32_t kNull = 0xFFFFFFFEu;   // Octree::nullNode (src/symvox/octree.cpp:22)
constexpr uint32_t kNone = 0xFFFFFFFFu;   // "no entry" in internal tables
constexpr uint64_t kEmpty64 = ~0ull;      // empty hash-table slot

struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SVDAG_CUDA(expr)                                                                   \
  do {                                                                                     \
    cudaError_t e__ = (expr);                                                              \
    if (e__ != cudaSuccess) {                                                              \
      throw ::svdag::Error(e__ == cudaErrorMemoryAllocation ? SVDAG_ERR_OOM : SVDAG_ERR_CUDA, \
                           std::string(#expr) + ": " + cudaGetErrorString(e__));          \
    }                                                                                      \
  } while (0)

// Optional per-launch device timing: each launch is bracketed by two CUDA
// events on the context stream; durations are summed per kernel name when
// the report is read.
struct Profiler {
  struct Rec { const char* name; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    SVDAG_CUDA(cudaEventCreate(&e));
    return e;
  }
  ~Profiler() {
    for (auto& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Per-context execution environment handed to every launch helper.
struct Exec {
  cudaStream_t stream = nullptr;
  int sm_count = 152;
  uint64_t* launches = nullptr;  // incremented once per kernel launch
  Profiler* prof = nullptr;      // non-null while kernel timing is enabled
  unsigned persistent_blocks = 0;  // cap on a persistent kernel's grid (0 = one block per SM)
  // Launch with programmatic stream serialisation: the kernel may be
  // scheduled while the previous kernel on the stream is still running; it
  // must begin with pdl_wait() (which returns once that kernel has completed
  // and its memory operations are visible) before touching global memory.
  bool pdl = false;
};

// Programmatic dependent launch (sm_90+): the wait blocks until the grid this
// one depends on has completed (a no-op for a grid launched without the
// attribute); the trigger lets the next grid on the stream be scheduled once
// every block of this one has issued it (or exited).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(cudaStream_t st, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// Grid for a grid-stride loop over n items.
inline unsigned grid_for(const Exec& ex, uint64_t n, unsigned threads, unsigned per_sm = 16) {
  uint64_t want = (n + threads - 1) / threads;
  uint64_t cap = uint64_t(ex.sm_count) * per_sm;
  if (want < 1) want = 1;
  return unsigned(want < cap ? want : cap);
}

#define SVDAG_LAUNCH(ex, kernel, grid, block, smem, ...)                 \
  do {                                                                   \
    ::svdag::Profiler* p__ = (ex).prof;                                  \
    cudaEvent_t a__ = nullptr, b__ = nullptr;                            \
    if (p__) {                                                           \
      a__ = p__->get();                                                  \
      b__ = p__->get();                                                  \
      SVDAG_CUDA(cudaEventRecord(a__, (ex).stream));                     \
    }                                                                    \
    if ((ex).pdl)                                                        \
      SVDAG_CUDA(::svdag::launch_pdl((ex).stream, kernel, dim3(grid),     \
                                     dim3(block), (smem), __VA_ARGS__)); \
    else                                                                 \
      kernel<<<(grid), (block), (smem), (ex).stream>>>(__VA_ARGS__);     \
    if ((ex).launches) ++*(ex).launches;                                 \
    SVDAG_CUDA(cudaPeekAtLastError());                                   \
    if (p__) {                                                           \
      SVDAG_CUDA(cudaEventRecord(b__, (ex).stream));                     \
      p__->recs.push_back({#kernel, a__, b__});                          \
    }                                                                    \
  } while (0)

// Stream-ordered device allocations made by this library in the process
// (every DBuf::alloc of a non-empty buffer); read by
// svdag_device_alloc_count().
inline std::atomic<uint64_t> g_device_allocs{0};

// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync).
template <class T>
struct DBuf {
  T* p = nullptr;
  uint64_t n = 0;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(uint64_t count, cudaStream_t st) { alloc(count, st); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(uint64_t count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count) {
      g_device_allocs.fetch_add(1, std::memory_order_relaxed);
      SVDAG_CUDA(cudaMallocAsync((void**)&p, sizeof(T) * (count ? count : 1), st));
    }
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
  uint64_t bytes() const { return n * sizeof(T); }
};

// ---------------------------------------------------------------------------
// 64-bit hash of a node key (hdr word + 8 child words).
__host__ __device__ __forceinline__ uint64_t mix_word(uint64_t h, uint32_t w) {
  h ^= w;
  h *= 0xFF51AFD7ED558CCDull;
  h ^= h >> 32;
  return h;
}
__host__ __device__ __forceinline__ uint64_t finish_hash(uint64_t h) {
  h ^= h >> 29;
  h *= 0xC4CEB9FE1A85EC53ull;
  h ^= h >> 32;
  return h;
}
__device__ __forceinline__ uint64_t hash_key9(uint32_t hdr, const uint32_t ch[8]) {
  uint64_t h = mix_word(0x9E3779B97F4A7C15ull, hdr);
#pragma unroll
  for (int c = 0; c < 8; ++c) h = mix_word(h, ch[c]);
  return finish_hash(h);
}

__device__ __forceinline__ void load_children(const uint32_t* ch, uint64_t i, uint32_t out[8]) {
  const uint4* p = reinterpret_cast<const uint4*>(ch + 8 * i);
  uint4 a = p[0], b = p[1];
  out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
  out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
}
// The same through L2 only (data written by other blocks of the running kernel).
__device__ __forceinline__ void load_children_cg(const uint32_t* ch, uint64_t i, uint32_t out[8]) {
  const uint4* p = reinterpret_cast<const uint4*>(ch + 8 * i);
  const uint4 a = __ldcg(p), b = __ldcg(p + 1);
  out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
  out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
}
__device__ __forceinline__ void store_children(uint32_t* ch, uint64_t i, const uint32_t v[8]) {
  uint4* p = reinterpret_cast<uint4*>(ch + 8 * i);
  p[0] = make_uint4(v[0], v[1], v[2], v[3]);
  p[1] = make_uint4(v[4], v[5], v[6], v[7]);
}

inline uint64_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan.  `In` maps an index to a value; `Out` receives
// (index, exclusive prefix) for every index.  One tile: one kernel (scan +
// emit + total).  More tiles: tile reduce, (recursive) scan of the tile sums,
// tile scan + emit; the last tile of the emit writes the grand total.

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T n = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) >= o) v += n;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total
// in *total (all threads).
// Any block size that is a multiple of 32 (up to 1024).
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* total) {
  __shared__ T warp_sums[32];
  __shared__ T tot;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = int(blockDim.x >> 5);
  T inc = warp_incl_scan(v);
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    T s = (lane < nw) ? warp_sums[lane] : T(0);
    T si = warp_incl_scan(s);
    if (lane < nw) warp_sums[lane] = si - s;
    if (lane == nw - 1) tot = si;
  }
  __syncthreads();
  T excl = warp_sums[w] + inc - v;
  *total = tot;
  __syncthreads();
  return excl;
}

template <class T, class In>
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(In in, uint64_t n, T* sums) {
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
  T s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint64_t i = base + uint64_t(j) * kScanThreads + threadIdx.x;
    if (i < n) s += T(in(i));
  }
  T tot;
  block_excl_scan<T>(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class T, class In, class Out>
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_emit(In in, uint64_t n, const T* offs, Out out,
                                                                   T* total) {
  __shared__ T sv[kScanTile];
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint64_t i = base + uint64_t(j) * kScanThreads + threadIdx.x;
    sv[j * kScanThreads + threadIdx.x] = (i < n) ? T(in(i)) : T(0);
  }
  __syncthreads();
  T loc[kScanItems];
  T run = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    loc[j] = sv[threadIdx.x * kScanItems + j];
    run += loc[j];
  }
  T tot;
  const T off = offs ? offs[blockIdx.x] : T(0);
  T pre = block_excl_scan<T>(run, &tot) + off;
  if (total && threadIdx.x == 0 && blockIdx.x == gridDim.x - 1) *total = off + tot;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    T v = loc[j];
    sv[threadIdx.x * kScanItems + j] = pre;
    pre += v;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint64_t i = base + uint64_t(j) * kScanThreads + threadIdx.x;
    if (i < n) out(i, sv[j * kScanThreads + threadIdx.x]);
  }
}

template <class T>
struct ArrayIn {
  const T* a;
  __device__ __forceinline__ T operator()(uint64_t i) const { return a[i]; }
};
template <class T>
struct ArrayOut {
  T* a;
  __device__ __forceinline__ void operator()(uint64_t i, T v) const { a[i] = v; }
};

// Exclusive scan of in(0..n-1); out(i, prefix) for every i; the grand total
// is written to *d_total (device) when d_total != nullptr.
template <class T, class In, class Out>
void device_exclusive_scan(const Exec& ex, In in, uint64_t n, Out out, T* d_total) {
  if (n == 0) {
    if (d_total) SVDAG_CUDA(cudaMemsetAsync(d_total, 0, sizeof(T), ex.stream));
    return;
  }
  const uint64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    SVDAG_LAUNCH(ex, (k_scan_tile_emit<T, In, Out>), 1, kScanThreads, 0, in, n, (const T*)nullptr, out, d_total);
    return;
  }
  DBuf<T> sums(nb, ex.stream), offs(nb, ex.stream);
  SVDAG_LAUNCH(ex, (k_scan_tile_sums<T, In>), unsigned(nb), kScanThreads, 0, in, n, sums.get());
  device_exclusive_scan<T>(ex, ArrayIn<T>{sums.get()}, nb, ArrayOut<T>{offs.get()}, (T*)nullptr);
  SVDAG_LAUNCH(ex, (k_scan_tile_emit<T, In, Out>), unsigned(nb), kScanThreads, 0, in, n, (const T*)offs.get(), out,
               d_total);
}

template <class T>
inline T read_scalar(const Exec& ex, const T* d) {
  T h;
  SVDAG_CUDA(cudaMemcpyAsync(&h, d, sizeof(T), cudaMemcpyDeviceToHost, ex.stream));
  SVDAG_CUDA(cudaStreamSynchronize(ex.stream));
  return h;
}

template <class T>
__global__ void k_fill(T* p, uint64_t n, T v) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) p[i] = v;
}
template <class T>
inline void fill(const Exec& ex, T* p, uint64_t n, T v) {
  if (n) SVDAG_LAUNCH(ex, k_fill<T>, grid_for(ex, n, 256), 256, 0, p, n, v);
}

}  // namespace svdag
