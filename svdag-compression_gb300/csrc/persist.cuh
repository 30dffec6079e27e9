// Persistent reduction kernels: one cooperative launch runs every level of a
// reduction phase (toDAG, toSDAG, the cross-level merge), its sub-steps
// separated by a software grid barrier, so a phase costs one launch and one
// read of its per-level counts instead of a few launches and a host
// round trip per level.
//
// The barrier's wait is bounded: a block that waits longer than
// kBarSpinLimit polls sets the phase's error word to kErrBarrier and returns,
// and the blocks still inside give up at their next barrier the same way, so
// a grid that could not become co-resident ends with an error instead of
// hanging.  Grids are one block per SM at most (see persistent_grid).
#pragma once

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <type_traits>
#include <vector>

#include "common.cuh"

namespace svdag {

// Error words written by the persistent kernels (0 = none).
constexpr int kErrProbe = 1;    // hash table probe limit
constexpr int kErrBarrier = 2;  // grid barrier wait limit

constexpr int kDagThreads = 1024;  // block size of the persistent toDAG
constexpr int kRedThreads = 1024;  // block size of the persistent toSDAG and merge
constexpr int kMaxRedLevels = 24;
constexpr unsigned kBarSpinLimit = 1u << 26;  // polls of >= 32 ns: seconds

struct GridBar {
  unsigned int count;  // zero before the launch
};

// All blocks of the grid arrive before any leaves; writes before the barrier
// are visible to plain loads after it (a gpu-scope fence before the arrival
// and after the wait, with the block barrier around them: the release /
// acquire pattern of the PTX memory model, as in cooperative groups' grid
// sync).  Data that other threads change within a step is read through L2
// (__ldcg) or atomically.  One atomic per block: block 0
// adds 2^31 - (G - 1), the others 1, so the sum of one barrier's arrivals is
// 2^31 and the counter's top bit flips exactly when the last block arrives
// (no partial sum reaches it); a block waits for the top bit to differ from
// the value it saw when it arrived.  Returns false on a timed-out wait.
__device__ __forceinline__ bool grid_sync(GridBar* bar, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int inc = (blockIdx.x == 0) ? (0x80000000u - (gridDim.x - 1)) : 1u;
    __threadfence();
    const unsigned int old = atomicAdd(&bar->count, inc);
    volatile unsigned int* v = &bar->count;
    int ok = 1;
    unsigned int spins = 0;
    while (((old ^ *v) & 0x80000000u) == 0) {
      if (++spins > kBarSpinLimit) {
        atomicCAS(err, 0, kErrBarrier);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Optional step trace (SVDAG_PHASE_TRACE set in the environment): block 0
// records (level << 8 | step, %globaltimer) after every barrier; the host
// prints each step's total time.  Step codes:
enum TraceStep : uint32_t {
  kStPrologue, kStLeafFirst, kStLeafRank, kStInsert, kStCount, kStEmit, kStCompact, kStCandidates, kStRound,
  kStSerial, kStTid0First, kStTid0Assign, kStKeys, kStTidAssign, kStCheck, kStOwnerMin, kStOwnerPath,
  kStOwnerBdesc, kStPrefix, kStNewidx, kStEmitLevels, kStEntry, kStNumSteps
};
constexpr unsigned kTraceCap = 8192;

__device__ __forceinline__ void trace_mark(unsigned long long* trace, unsigned& pos, uint32_t code) {
  if (trace && blockIdx.x == 0 && threadIdx.x == 0 && pos < kTraceCap) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    trace[2 * pos] = code;
    trace[2 * pos + 1] = t;
    ++pos;
  }
}

// Ends a step: grid barrier (return from the kernel on a timed-out wait),
// then the trace mark.  Needs `trace_pos` in scope.
#define SVDAG_STEP(a, lev, step)                                       \
  do {                                                                 \
    if (!grid_sync((a).bar, (a).err)) return;                          \
    trace_mark((a).trace, trace_pos, (uint32_t(lev) << 8) | (step));   \
  } while (0)

// Sum of v over the block (all threads receive it).
template <class T>
__device__ __forceinline__ T block_sum(T v) {
  T tot;
  block_excl_scan<T>(v, &tot);
  return tot;
}

// Contiguous share [b0, b1) of [0, n) for this block (block-ordered scans).
__device__ __forceinline__ void block_share(uint64_t n, uint64_t& b0, uint64_t& b1) {
  const uint64_t per = (n + gridDim.x - 1) / gridDim.x;
  b0 = min(n, uint64_t(blockIdx.x) * per);
  b1 = min(n, b0 + per);
}

// Exclusive offset of this block's share and the grand total from the
// per-block counts bsum[0..gridDim.x) (written by every block before the
// last barrier).
__device__ __forceinline__ uint32_t block_offset(const uint32_t* bsum, uint32_t* total) {
  uint32_t before = 0, all = 0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    const uint32_t v = __ldcg(&bsum[k]);
    all += v;
    if (k < blockIdx.x) before += v;
  }
  before = block_sum(before);
  *total = block_sum(all);
  return before;
}

#define SVDAG_BLOCK_STRIDE(i, b0, b1) for (uint64_t i = (b0) + threadIdx.x; i < (b1); i += blockDim.x)
#define SVDAG_GRID_STRIDE(i, n) \
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < (n); i += uint64_t(gridDim.x) * blockDim.x)

__device__ __forceinline__ void clear_slots(unsigned long long* slots, uint64_t n) {
  SVDAG_GRID_STRIDE(s, n) slots[s] = kEmpty64;
}

template <class T>
struct NoDeduce {
  using type = T;
};

// Cooperative launch of a persistent kernel with `grid` blocks of `threads`
// threads and `smem` bytes of dynamic shared memory, counted and (when
// profiling) timed like SVDAG_LAUNCH.
template <class... KArgs>
void launch_persistent(const Exec& ex, const char* name, void (*kern)(KArgs...), unsigned grid, unsigned threads,
                       size_t smem, typename NoDeduce<KArgs>::type... args) {
  void* params[] = {(void*)&args...};
  cudaEvent_t a = nullptr, b = nullptr;
  if (ex.prof) {
    a = ex.prof->get();
    b = ex.prof->get();
    SVDAG_CUDA(cudaEventRecord(a, ex.stream));
  }
  SVDAG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(threads), params, smem, ex.stream));
  if (ex.launches) ++*ex.launches;
  if (ex.prof) {
    SVDAG_CUDA(cudaEventRecord(b, ex.stream));
    ex.prof->recs.push_back({name, a, b});
  }
}

// Blocks for a persistent kernel of `threads` threads per block over at most
// `work` items per pass: no more than the work needs (an item per thread: the
// passes are latency-bound gathers),
// one per SM at most, and at most ex.persistent_blocks when the caller runs
// several persistent phases side by side.  A block of 1024 threads at <= 64
// registers fills an SM; a cooperative launch starts only when all of its
// blocks can be resident, so persistent kernels on different streams that
// do not fit together run one after the other rather than deadlock.
// Largest dynamic shared memory of a persistent launch.
constexpr size_t kMaxPersistentSmem = 160 * 1024;

// Raises a kernel's dynamic shared-memory limit to kMaxPersistentSmem, once
// per (kernel, device): host threads that launch the same kernel with
// different sizes must not lower the limit under each other's launches.
inline void allow_persistent_smem(const void* kern) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, int>> done;
  int dev = 0;
  SVDAG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& d : done)
    if (d.first == kern && d.second == dev) return;
  SVDAG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxPersistentSmem)));
  done.emplace_back(kern, dev);
}

template <class K>
unsigned persistent_grid(const Exec& ex, K kern, unsigned threads, uint64_t work, size_t smem = 0) {
  if (smem > kMaxPersistentSmem) throw Error(SVDAG_ERR_INVALID_ARG, "persistent kernel: shared memory above the limit");
  if (smem > 48 * 1024) allow_persistent_smem((const void*)kern);
  int per_sm = 0;
  SVDAG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, int(threads), smem));
  if (per_sm < 1) throw Error(SVDAG_ERR_CUDA, "persistent kernel cannot be resident");
  uint64_t cap = uint64_t(ex.sm_count);
  if (ex.persistent_blocks) cap = std::min<uint64_t>(cap, ex.persistent_blocks);
  const uint64_t want = std::max<uint64_t>(1, (work + threads - 1) / threads);
  return unsigned(std::min<uint64_t>(want, cap));
}

// Control block of a persistent phase: error word, barrier, reduced counts.
struct RedCtl {
  int err;
  GridBar bar;
  uint32_t cnt[kMaxRedLevels];
};

inline uint64_t table_slots(uint64_t n) { return next_pow2(n < 16 ? 32 : 2 * n); }

// Reads the control block after the phase kernel (the phase's one host
// synchronisation) and maps its error word.
inline RedCtl finish_persistent(const Exec& ex, const RedCtl* d_ctl, const char* what) {
  RedCtl h;
  SVDAG_CUDA(cudaMemcpyAsync(&h, d_ctl, sizeof(RedCtl), cudaMemcpyDeviceToHost, ex.stream));
  SVDAG_CUDA(cudaStreamSynchronize(ex.stream));
  if (h.err == kErrProbe) throw Error(SVDAG_ERR_OVERFLOW, std::string(what) + ": hash table probe limit reached");
  if (h.err == kErrBarrier)
    throw Error(SVDAG_ERR_TIMEOUT, std::string(what) + ": grid barrier wait limit reached (grid not co-resident)");
  if (h.err) throw Error(SVDAG_ERR_CUDA, std::string(what) + ": device error word " + std::to_string(h.err));
  return h;
}

// Host side of the step trace.
struct PhaseTrace {
  DBuf<unsigned long long> buf;
  PhaseTrace(cudaStream_t st) {
    if (!std::getenv("SVDAG_PHASE_TRACE")) return;
    buf.alloc(2 * kTraceCap, st);
    SVDAG_CUDA(cudaMemsetAsync(buf.get(), 0, 16ull * kTraceCap, st));
  }
  unsigned long long* ptr() const { return buf.get(); }
  // After the phase's synchronisation: per step, the time from the previous
  // mark to its own (summed over levels and rounds) and how often it ran.
  void report(const Exec& ex, const char* phase) const {
    if (!buf.get()) return;
    static const char* kNames[kStNumSteps] = {
        "prologue", "leaf first", "leaf rank+remap", "insert", "count", "emit ids", "compact+remap", "candidates",
        "round", "serial", "tid0 first", "tid0 assign", "keys", "tid assign", "check", "owner min", "owner path",
        "owner bdesc", "prefix", "newidx", "emit levels", "entry"};
    std::vector<unsigned long long> h(2 * kTraceCap);
    SVDAG_CUDA(cudaMemcpyAsync(h.data(), buf.get(), 16ull * kTraceCap, cudaMemcpyDeviceToHost, ex.stream));
    SVDAG_CUDA(cudaStreamSynchronize(ex.stream));
    constexpr int kLv = 32;
    double tot[kStNumSteps] = {}, per[kStNumSteps][kLv] = {};
    unsigned cnt[kStNumSteps] = {};
    unsigned n = 0;
    while (n < kTraceCap && h[2 * n + 1]) ++n;
    for (unsigned k = 1; k < n; ++k) {
      const uint32_t step = uint32_t(h[2 * k] & 0xFFu), lev = uint32_t(h[2 * k] >> 8);
      if (step >= kStNumSteps) continue;
      const double us = double(h[2 * k + 1] - h[2 * k - 1]) * 1e-3;
      tot[step] += us;
      if (lev < kLv) per[step][lev] += us;
      ++cnt[step];
    }
    std::fprintf(stderr, "[svdag trace] %s: %.1f us over %u marks\n", phase,
                 n > 1 ? double(h[2 * (n - 1) + 1] - h[1]) * 1e-3 : 0.0, n);
    for (int s = 0; s < int(kStNumSteps); ++s) {
      if (!cnt[s]) continue;
      std::fprintf(stderr, "[svdag trace]   %-16s %9.1f us  x%-3u", kNames[s], tot[s], cnt[s]);
      for (int l = 0; l < kLv; ++l)
        if (per[s][l] > 0) std::fprintf(stderr, " %d:%.0f", l, per[s][l]);
      std::fprintf(stderr, "\n");
    }
  }
};

// A level buffer of capacity `cap` holding `live` entries: kept when at
// least half is live, else replaced by an exact copy.
template <class T>
void fit_buffer(DBuf<T>& b, uint64_t live, cudaStream_t st) {
  if (!b.get() || 2 * live >= b.n) return;
  DBuf<T> t(live ? live : 1, st);
  if (live) SVDAG_CUDA(cudaMemcpyAsync(t.get(), b.get(), live * sizeof(T), cudaMemcpyDeviceToDevice, st));
  b = std::move(t);
}

}  // namespace svdag
