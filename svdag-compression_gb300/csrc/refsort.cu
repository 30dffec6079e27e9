// Reference-count order of a level on the GPU: the permutation libstdc++'s
// std::sort gives EncodedSSVDAG::encode (src/symvox/encoded_ssvdag.cpp:266-276),
// reproduced exactly (refsort.cuh states the algorithm and the parallel form
// of its partition step).
//
// Rounds over the segments that still hold more than kSmall elements, one
// host read per round:
//   pivot   one thread per segment: median of three to the front;
//   count   one block per chunk of kChunk elements of a partition range:
//           its L- and R-candidates;
//   scans   of the chunk counts (a segment's chunks are consecutive);
//   classify  per element its candidate ranks, exchanged or not; exchanged
//           L- and R-candidates record their positions by rank, the
//           segment's cut and exchange count are reduced with atomics;
//   swap    the K exchanges of each segment (disjoint position pairs);
//   split   the two parts of each segment: more than kSmall elements -> next
//           round (or, with the depth budget spent, a heap sort), else one
//           thread sorts the part in shared memory with the sequential
//           introsort and the final insertion pass.
// The chunk kernels are launched over an upper bound of the chunk count;
// blocks past the true count (known on the device) write zero counts.

#include "common.cuh"
#include "refsort.cuh"

namespace svdag {
namespace {

using refsort::before;

constexpr uint32_t kSmall = 512;  // parts up to this size: one thread, shared memory
constexpr int kRsThreads = 256;
constexpr int kRsItems = 4;
constexpr uint32_t kChunk = kRsThreads * kRsItems;
constexpr int kSmallBlocksPerSm = 32;

struct Seg {
  uint32_t lo, hi, depth, pad;
};

__global__ void k_rs_init(const uint32_t* __restrict__ counts, uint64_t n, uint64_t* __restrict__ keys) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    keys[i] = refsort::make_elem(uint32_t(i), counts[i]);
}

__global__ void k_rs_seed(Seg* s, uint32_t lo, uint32_t hi, uint32_t depth) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *s = Seg{lo, hi, depth, 0};
}

// Pivot of every segment of the round; chunk counts; cut and exchange count reset.
__global__ void k_rs_pivot(uint64_t* keys, const Seg* __restrict__ segs, uint32_t ns, uint32_t* __restrict__ nchunks,
                           uint32_t* __restrict__ cut, uint32_t* __restrict__ nswap) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
    const Seg g = segs[s];
    refsort::pivot_to_front(keys, int64_t(g.lo), int64_t(g.hi));
    nchunks[s] = (g.hi - g.lo - 1 + kChunk - 1) / kChunk;
    cut[s] = g.hi;
    nswap[s] = 0;
  }
}

struct U32In {
  const uint32_t* a;
  __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return a[i]; }
};
struct U32Put {
  uint32_t* a;
  __device__ __forceinline__ void operator()(uint64_t i, uint32_t v) const { a[i] = v; }
};

// The chunk a block works on: its segment (binary search over the chunk
// bases, which increase strictly) and element range.
struct ChunkAt {
  uint32_t s, c0, c1, start, end;
  Seg g;
};
__device__ __forceinline__ bool chunk_at(uint32_t c, const Seg* segs, uint32_t ns, const uint32_t* cbase,
                                         const uint32_t* ctotal, ChunkAt& A) {
  const uint32_t total = *ctotal;
  if (c >= total) return false;
  uint32_t lo = 0, hi = ns;  // largest s with cbase[s] <= c
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (cbase[mid] <= c) lo = mid;
    else hi = mid;
  }
  A.s = lo;
  A.g = segs[lo];
  A.c0 = cbase[lo];
  A.c1 = (lo + 1 < ns) ? cbase[lo + 1] : total;
  A.start = A.g.lo + 1 + (c - A.c0) * kChunk;
  A.end = min(A.start + kChunk, A.g.hi);
  return true;
}

template <class T>
__device__ __forceinline__ T block_sum(T v) {
  T tot;
  block_excl_scan<T>(v, &tot);
  return tot;
}

__device__ __forceinline__ uint32_t block_min(uint32_t v) {
  __shared__ uint32_t wmin[32];
  v = __reduce_min_sync(0xFFFFFFFFu, v);
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t m = 0xFFFFFFFFu;
  for (int w = 0; w < int(blockDim.x >> 5); ++w) m = min(m, wmin[w]);
  __syncthreads();
  return m;
}

// L- and R-candidates of each chunk (zero past the true chunk count).
__global__ void __launch_bounds__(kRsThreads) k_rs_count(const uint64_t* __restrict__ keys, const Seg* __restrict__ segs,
                                                         uint32_t ns, const uint32_t* __restrict__ cbase,
                                                         const uint32_t* __restrict__ ctotal,
                                                         uint32_t* __restrict__ cnt_l, uint32_t* __restrict__ cnt_r) {
  ChunkAt A;
  if (!chunk_at(blockIdx.x, segs, ns, cbase, ctotal, A)) {
    if (threadIdx.x == 0) { cnt_l[blockIdx.x] = 0; cnt_r[blockIdx.x] = 0; }
    return;
  }
  const uint64_t p = keys[A.g.lo];
  uint32_t nl = 0, nr = 0;
#pragma unroll
  for (int j = 0; j < kRsItems; ++j) {
    const uint32_t i = A.start + j * kRsThreads + threadIdx.x;
    if (i < A.end) {
      const uint64_t x = keys[i];
      nl += before(x, p) ? 0u : 1u;
      nr += before(p, x) ? 0u : 1u;
    }
  }
  nl = block_sum(nl);
  nr = block_sum(nr);
  if (threadIdx.x == 0) { cnt_l[blockIdx.x] = nl; cnt_r[blockIdx.x] = nr; }
}

// Ranks, exchange roles, recorded positions, cut and exchange count.
__global__ void __launch_bounds__(kRsThreads) k_rs_classify(const uint64_t* __restrict__ keys, const Seg* __restrict__ segs,
                                                            uint32_t ns, const uint32_t* __restrict__ cbase,
                                                            const uint32_t* __restrict__ ctotal,
                                                            const uint32_t* __restrict__ pre_l,
                                                            const uint32_t* __restrict__ pre_r,
                                                            uint32_t* __restrict__ pos_l, uint32_t* __restrict__ pos_r,
                                                            uint32_t* __restrict__ cut, uint32_t* __restrict__ nswap) {
  ChunkAt A;
  if (!chunk_at(blockIdx.x, segs, ns, cbase, ctotal, A)) return;
  const uint32_t c = blockIdx.x;
  const uint64_t p = keys[A.g.lo];
  const uint32_t l_chunk = pre_l[c] - pre_l[A.c0];      // L-candidates in earlier chunks of the segment
  const uint32_t r_chunk = pre_r[A.c1] - pre_r[c + 1];  // R-candidates in later chunks
  // each thread takes kRsItems consecutive elements
  const uint32_t i0 = A.start + threadIdx.x * kRsItems;
  uint64_t x[kRsItems];
  uint32_t fl = 0, fr = 0, tl = 0, tr = 0;
#pragma unroll
  for (int j = 0; j < kRsItems; ++j) {
    const uint32_t i = i0 + j;
    x[j] = (i < A.end) ? keys[i] : 0;
    const bool is_l = i < A.end && !before(x[j], p);
    const bool is_r = i < A.end && !before(p, x[j]);
    fl |= uint32_t(is_l) << j;
    fr |= uint32_t(is_r) << j;
    tl += is_l;
    tr += is_r;
  }
  uint32_t TL, TR;
  const uint32_t el = block_excl_scan<uint32_t>(tl, &TL);
  const uint32_t er = block_excl_scan<uint32_t>(tr, &TR);
  uint32_t l_before = l_chunk + el;               // L-candidates before the current element
  uint32_t r_incl = er;                           // R-candidates in the chunk up to and including it
  uint32_t my_cut = 0xFFFFFFFFu, my_swaps = 0;
#pragma unroll
  for (int j = 0; j < kRsItems; ++j) {
    const uint32_t i = i0 + j;
    const bool is_l = (fl >> j) & 1u, is_r = (fr >> j) & 1u;
    r_incl += is_r;
    if (is_l || is_r) {
      const uint32_t r_after = r_chunk + (TR - r_incl);
      bool cc;
      const int role = refsort::classify(is_l, is_r, l_before, r_after, cc);
      if (role == refsort::kSwapL) { pos_l[A.g.lo + l_before] = i; ++my_swaps; }
      if (role == refsort::kSwapR) pos_r[A.g.lo + r_after] = i;
      if (cc) my_cut = min(my_cut, i);
    }
    l_before += is_l;
  }
  const uint32_t bc = block_min(my_cut);
  const uint32_t bs = block_sum(my_swaps);
  if (threadIdx.x == 0) {
    if (bc != 0xFFFFFFFFu) atomicMin(&cut[A.s], bc);
    if (bs) atomicAdd(&nswap[A.s], bs);
  }
}

// The exchanges L[k] <-> R[k], k < K, of every segment.
__global__ void __launch_bounds__(kRsThreads) k_rs_swap(uint64_t* __restrict__ keys, const Seg* __restrict__ segs,
                                                        uint32_t ns, const uint32_t* __restrict__ cbase,
                                                        const uint32_t* __restrict__ ctotal,
                                                        const uint32_t* __restrict__ pos_l,
                                                        const uint32_t* __restrict__ pos_r,
                                                        const uint32_t* __restrict__ nswap, uint32_t* counters) {
  ChunkAt A;
  if (!chunk_at(blockIdx.x, segs, ns, cbase, ctotal, A)) return;
  const uint32_t K = min(nswap[A.s], A.g.hi - A.g.lo - 1);
  const uint32_t r0 = (blockIdx.x - A.c0) * kChunk;
  for (uint32_t t = threadIdx.x; t < kChunk; t += kRsThreads) {
    const uint32_t r = r0 + t;
    if (r >= K) break;
    const uint32_t a = pos_l[A.g.lo + r], b = pos_r[A.g.lo + r];
    // both positions lie in the partition range and L[k] < R[k]
    if (!(a > A.g.lo && a < b && b < A.g.hi)) {
      atomicExch(&counters[3], 1u);
      continue;
    }
    const uint64_t va = keys[a], vb = keys[b];
    keys[a] = vb;
    keys[b] = va;
  }
}

// The two parts of every segment.  counters: [0] next round, [1] small
// parts, [2] parts to heap-sort, [3] error.  `cap`: capacity of the next
// list; the small and heap lists hold 2 cap.
__device__ __forceinline__ void push_seg(Seg* list, uint32_t* count, uint32_t cap, const Seg& v, uint32_t* err) {
  const uint32_t k = atomicAdd(count, 1u);
  if (k < cap) list[k] = v;
  else atomicExch(err, 1u);
}
__global__ void k_rs_split(const Seg* __restrict__ segs, uint32_t ns, const uint32_t* __restrict__ cut,
                           Seg* __restrict__ next, Seg* __restrict__ small, Seg* __restrict__ heap, uint32_t cap,
                           uint32_t* counters) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
    const Seg g = segs[s];
    const uint32_t ct = cut[s];
    if (ct <= g.lo || ct >= g.hi || g.depth == 0) {
      atomicExch(&counters[3], 1u);
      continue;
    }
    const uint32_t d = g.depth - 1;
    const uint32_t b[3] = {g.lo, ct, g.hi};
    for (int k = 0; k < 2; ++k) {
      const Seg part{b[k], b[k + 1], d, 0};
      if (part.hi - part.lo > kSmall) {
        if (d == 0) push_seg(heap, &counters[2], 2 * cap, part, &counters[3]);
        else push_seg(next, &counters[0], cap, part, &counters[3]);
      } else {
        push_seg(small, &counters[1], 2 * cap, part, &counters[3]);
      }
    }
  }
}

// Sequential introsort + final pass of each small part, in shared memory.
__global__ void __launch_bounds__(32) k_rs_small(uint64_t* __restrict__ keys, const Seg* __restrict__ small,
                                                 uint32_t n_small, uint32_t* counters) {
  __shared__ uint64_t buf[kSmall];
  uint64_t* a = buf;
  for (uint32_t s = blockIdx.x; s < n_small; s += gridDim.x) {
    const Seg g = small[s];
    const uint32_t len = g.hi - g.lo;
    if (len > kSmall || g.hi < g.lo) {
      if (threadIdx.x == 0) atomicExch(&counters[3], 1u);
      continue;
    }
    for (uint32_t t = threadIdx.x; t < len; t += 32) buf[t] = keys[g.lo + t];
    __syncwarp();
    if (threadIdx.x == 0 && !refsort::sort_segment(a, 0, int64_t(len), g.depth)) atomicExch(&counters[3], 1u);
    __syncwarp();
    for (uint32_t t = threadIdx.x; t < len; t += 32) keys[g.lo + t] = buf[t];
    __syncwarp();
  }
}

// Heap sort of the parts whose depth budget ran out (the order of a sorted
// part needs no final pass).
__global__ void k_rs_heap(uint64_t* keys, const Seg* __restrict__ heap, uint32_t n_heap) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n_heap; s += gridDim.x * blockDim.x) {
    const Seg g = heap[s];
    refsort::heap_sort(keys, int64_t(g.lo), int64_t(g.hi));
  }
}

__global__ void k_rs_emit(const uint64_t* __restrict__ keys, uint64_t n, uint32_t* __restrict__ order) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    order[i] = uint32_t(keys[i]);
}

}  // namespace

// order[k] = index of the k-th node in the reference's ref-count order.
void refcount_order(const Exec& ex, const uint32_t* counts, uint64_t n, uint32_t* order) {
  if (n == 0) return;
  if (n > (1ull << 31)) throw Error(SVDAG_ERR_OVERFLOW, "refcount order: more than 2^31 nodes");
  const cudaStream_t st = ex.stream;
  DBuf<uint64_t> keys(n, st);
  SVDAG_LAUNCH(ex, k_rs_init, grid_for(ex, n, 256), 256, 0, counts, n, keys.get());
  const uint32_t depth = refsort::depth_budget(n);
  const uint64_t max_segs = n / (kSmall + 1) + 1;  // disjoint segments of more than kSmall elements
  DBuf<Seg> cur(max_segs, st), next(max_segs, st), small(2 * max_segs, st), heap(2 * max_segs, st);
  DBuf<uint32_t> counters(4, st);
  uint32_t h_cnt[4] = {0, 0, 0, 0};
  SVDAG_CUDA(cudaMemsetAsync(counters.get(), 0, 16, st));
  if (n <= kSmall) {
    SVDAG_LAUNCH(ex, k_rs_seed, 1, 32, 0, small.get(), 0u, uint32_t(n), depth);
    SVDAG_LAUNCH(ex, k_rs_small, 1, 32, 0, keys.get(), small.get(), 1u, counters.get());
  } else {
    SVDAG_LAUNCH(ex, k_rs_seed, 1, 32, 0, cur.get(), 0u, uint32_t(n), depth);
    DBuf<uint32_t> pos_l(n, st), pos_r(n, st);
    DBuf<uint32_t> nchunks(max_segs, st), cbase(max_segs, st), cut(max_segs, st), nswap(max_segs, st);
    DBuf<uint32_t> ctotal(1, st);
    const uint64_t max_chunks = n / kChunk + max_segs + 1;
    DBuf<uint32_t> cnt_l(max_chunks, st), cnt_r(max_chunks, st), pre_l(max_chunks + 1, st), pre_r(max_chunks + 1, st);
    uint32_t ns = 1;
    for (uint32_t round = 0; ns > 0; ++round) {
      if (round > 64) throw Error(SVDAG_ERR_CUDA, "refcount order: more rounds than the depth budget allows");
      const uint64_t chunks_ub = std::min<uint64_t>(max_chunks, n / kChunk + ns + 1);
      SVDAG_CUDA(cudaMemsetAsync(counters.get(), 0, 12, st));
      SVDAG_LAUNCH(ex, k_rs_pivot, grid_for(ex, ns, 256), 256, 0, keys.get(), cur.get(), ns, nchunks.get(), cut.get(),
                   nswap.get());
      device_exclusive_scan<uint32_t>(ex, U32In{nchunks.get()}, ns, U32Put{cbase.get()}, ctotal.get());
      SVDAG_LAUNCH(ex, k_rs_count, unsigned(chunks_ub), kRsThreads, 0, keys.get(), cur.get(), ns, cbase.get(),
                   ctotal.get(), cnt_l.get(), cnt_r.get());
      device_exclusive_scan<uint32_t>(ex, U32In{cnt_l.get()}, chunks_ub, U32Put{pre_l.get()}, pre_l.get() + chunks_ub);
      device_exclusive_scan<uint32_t>(ex, U32In{cnt_r.get()}, chunks_ub, U32Put{pre_r.get()}, pre_r.get() + chunks_ub);
      SVDAG_LAUNCH(ex, k_rs_classify, unsigned(chunks_ub), kRsThreads, 0, keys.get(), cur.get(), ns, cbase.get(),
                   ctotal.get(), pre_l.get(), pre_r.get(), pos_l.get(), pos_r.get(), cut.get(), nswap.get());
      SVDAG_LAUNCH(ex, k_rs_swap, unsigned(chunks_ub), kRsThreads, 0, keys.get(), cur.get(), ns, cbase.get(),
                   ctotal.get(), pos_l.get(), pos_r.get(), nswap.get(), counters.get());
      SVDAG_LAUNCH(ex, k_rs_split, grid_for(ex, ns, 256), 256, 0, cur.get(), ns, cut.get(), next.get(), small.get(),
                   heap.get(), uint32_t(max_segs), counters.get());
      SVDAG_CUDA(cudaMemcpyAsync(h_cnt, counters.get(), 16, cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
      if (h_cnt[3] || h_cnt[0] > max_segs || h_cnt[1] > 2 * max_segs || h_cnt[2] > 2 * max_segs)
        throw Error(SVDAG_ERR_CUDA, "refcount order: inconsistent partition");
      if (h_cnt[1])
        SVDAG_LAUNCH(ex, k_rs_small, unsigned(std::min<uint64_t>(h_cnt[1], uint64_t(ex.sm_count) * kSmallBlocksPerSm)),
                     32, 0, keys.get(), small.get(), h_cnt[1], counters.get());
      if (h_cnt[2])
        SVDAG_LAUNCH(ex, k_rs_heap, grid_for(ex, h_cnt[2], 32), 32, 0, keys.get(), heap.get(), h_cnt[2]);
      ns = h_cnt[0];
      std::swap(cur, next);
    }
  }
  SVDAG_CUDA(cudaMemcpyAsync(h_cnt, counters.get(), 16, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  if (h_cnt[3]) throw Error(SVDAG_ERR_CUDA, "refcount order: a part's sort left its bounds");
  SVDAG_LAUNCH(ex, k_rs_emit, grid_for(ex, n, 256), 256, 0, keys.get(), n, order);
}

}  // namespace svdag

extern "C" int svdag_refcount_order(void* stream, const uint32_t* device_counts, uint64_t n, uint32_t* device_order) {
  if (n && (!device_counts || !device_order)) return SVDAG_ERR_INVALID_ARG;
  try {
    svdag::Exec ex;
    ex.stream = static_cast<cudaStream_t>(stream);
    int dev = 0;
    SVDAG_CUDA(cudaGetDevice(&dev));
    SVDAG_CUDA(cudaDeviceGetAttribute(&ex.sm_count, cudaDevAttrMultiProcessorCount, dev));
    svdag::refcount_order(ex, device_counts, n, device_order);
    SVDAG_CUDA(cudaStreamSynchronize(ex.stream));
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    return e.code;
  }
}
