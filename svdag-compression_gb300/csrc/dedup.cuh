// Open-addressing hash table of node keys shared by the DAG, SDAG and
// CSVDAG reductions.  Keys never change while a table is built or read, so
// they are plain (L1-cached) loads; inserts read slots through L2 (__ldcg),
// as other threads fill them concurrently; lookups run after all inserts and
// read them plainly.  A key is (hdr word, 8 child words) read from
// structure-of-arrays level buffers; a slot packs (hash tag << 32 | index).
// Equal keys converge on their minimum index (atomicMin), so after all
// inserts every slot holds its key's first occurrence.
#pragma once

#include "common.cuh"

namespace svdag {
namespace {

__device__ __forceinline__ uint64_t ld_cg64(const unsigned long long* p) { return __ldcg(p); }
__device__ __forceinline__ uint32_t ld_cg32(const uint32_t* p) { return __ldcg(p); }

__device__ __forceinline__ void load_key(const uint32_t* hdr, const uint32_t* ch, uint64_t i, uint32_t& h, uint32_t c[8]) {
  h = hdr[i];
  if (ch) {
    load_children(ch, i, c);
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = kNull;
  }
}

__device__ __forceinline__ bool key_equal_at(const uint32_t* hdr, const uint32_t* ch, uint64_t j, uint32_t h,
                                             const uint32_t c[8]) {
  if (hdr[j] != h) return false;
  if (!ch) return true;
  uint32_t d[8];
  load_children(ch, j, d);
  bool eq = true;
#pragma unroll
  for (int k = 0; k < 8; ++k) eq &= (d[k] == c[k]);
  return eq;
}

struct Table {
  unsigned long long* slots;
  uint64_t mask;  // size - 1 (power of two)
};

// Slots are probed linearly, an aligned pair per 16-byte load (tables have
// at least 32 slots, a power of two, so pairs never wrap).
constexpr int kGroup = 2;
template <bool kL2>
__device__ __forceinline__ void load_group(const unsigned long long* slots, uint64_t g, unsigned long long w[kGroup]) {
  const ulonglong2* p = reinterpret_cast<const ulonglong2*>(slots + g);
  const ulonglong2 x = kL2 ? __ldcg(p) : *p;
  w[0] = x.x;
  w[1] = x.y;
}

// Insert node i's key; equal keys keep the minimum index.  Returns the slot.
__device__ uint64_t table_insert(Table T, const uint32_t* hdr, const uint32_t* ch, uint32_t i, uint32_t h,
                                 const uint32_t c[8], int* err) {
  const uint64_t hk = hash_key9(h, c);
  const uint64_t tag = hk >> 32;
  const unsigned long long mine = (tag << 32) | i;
  uint64_t pos = hk & T.mask;
  uint64_t probe = 0;
  while (probe <= T.mask) {
    const uint64_t g = pos & ~uint64_t(kGroup - 1);
    unsigned long long w[kGroup];
    load_group<true>(T.slots, g, w);
    const int k0 = int(pos - g);
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {  // unrolled: w stays in registers
      if (k < k0) continue;
      ++probe;
      const uint64_t sp = g + uint64_t(k);
      unsigned long long cur = w[k];
      if (cur == kEmpty64) {
        const unsigned long long prev = atomicCAS(&T.slots[sp], kEmpty64, mine);
        if (prev == kEmpty64) return sp;
        cur = prev;
      }
      if ((cur >> 32) == tag) {
        const uint32_t j = uint32_t(cur);
        if (key_equal_at(hdr, ch, j, h, c)) {
          if (i < j) atomicMin(&T.slots[sp], mine);
          return sp;
        }
      }
    }
    pos = (g + kGroup) & T.mask;
  }
  atomicExch(err, 1);
  return kEmpty64;
}

// Look a key up; returns the minimum index stored for it or kNone.
__device__ uint32_t table_find(Table T, const uint32_t* hdr, const uint32_t* ch, uint32_t h, const uint32_t c[8]) {
  const uint64_t hk = hash_key9(h, c);
  const uint64_t tag = hk >> 32;
  uint64_t pos = hk & T.mask;
  uint64_t probe = 0;
  while (probe <= T.mask) {
    const uint64_t g = pos & ~uint64_t(kGroup - 1);
    unsigned long long w[kGroup];
    load_group<false>(T.slots, g, w);
    const int k0 = int(pos - g);
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
      if (k < k0) continue;
      ++probe;
      const unsigned long long cur = w[k];
      if (cur == kEmpty64) return kNone;
      if ((cur >> 32) == tag) {
        const uint32_t j = uint32_t(cur);
        if (key_equal_at(hdr, ch, j, h, c)) return j;
      }
    }
    pos = (g + kGroup) & T.mask;
  }
  return kNone;
}

__global__ void k_insert(Table T, const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                         uint32_t* __restrict__ slot_of, int* err) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t h, c[8];
    load_key(hdr, ch, i, h, c);
    if ((h & 0xFFu) == 0) { slot_of[i] = kNone; continue; }  // empty nodes are skipped (geom_octree.cpp:495)
    const uint64_t s = table_insert(T, hdr, ch, uint32_t(i), h, c, err);
    slot_of[i] = uint32_t(s);
  }
}

__global__ void k_rep(Table T, const uint32_t* __restrict__ slot_of, uint64_t n, uint32_t* __restrict__ rep) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t s = slot_of[i];
    rep[i] = (s == kNone) ? kNone : uint32_t(T.slots[s]);
  }
}

Table make_table(const Exec& ex, uint64_t n, DBuf<unsigned long long>& buf) {
  const uint64_t size = next_pow2(n < 16 ? 32 : 2 * n);
  buf.alloc(size, ex.stream);
  SVDAG_CUDA(cudaMemsetAsync(buf.get(), 0xFF, size * 8, ex.stream));
  return Table{buf.get(), size - 1};
}

void check_err(const Exec& ex, const int* d_err, const char* what) {
  if (read_scalar(ex, d_err)) throw Error(SVDAG_ERR_OVERFLOW, std::string(what) + ": hash table probe limit reached");
}


}  // namespace
}  // namespace svdag
