// Reference-count order of one level's nodes, as EncodedSSVDAG::encode
// (src/symvox/encoded_ssvdag.cpp:259-276) makes it: a vector of
// (index, count) pairs, initially in index order, sorted by std::sort with
// "count(a) > count(b)" as the only comparison.  std::sort is not stable, so
// the order of nodes with equal counts -- and with it every byte of the
// .ssvdag file -- is whatever libstdc++'s introsort leaves.  This header
// restates that published algorithm (GCC 13 libstdc++, bits/stl_algo.h and
// bits/stl_heap.h) step for step:
//   * introsort loop: while a segment has more than 16 elements, either
//     (depth budget spent) heap-sort it, or spend one unit of depth budget,
//     move the median of the elements at first+1, middle, last-1 to first,
//     Hoare-partition [first+1, last) around it and continue on both parts;
//     the initial budget is 2 floor(log2 n);
//   * final pass: insertion sort over the whole array.  Every element of a
//     part is ordered no later than every element of the parts to its right,
//     so the strict insertion never crosses a part boundary: the pass is a
//     stable sort of each final part (heap-sorted parts are already sorted).
// The GPU runs the partitions of large segments in parallel (refsort.cu) with
// the swap pattern characterised below; small segments are finished by one
// thread with the sequential steps of this header.  Elements are 64-bit
// words (count << 32) | index.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define RS_HD __host__ __device__ __forceinline__
#else
#define RS_HD inline
#endif

namespace svdag {
namespace refsort {

constexpr uint32_t kThreshold = 16;  // parts of at most this size are left to the final pass

// "a is ordered before b": the reference's comparator on the counts
RS_HD bool before(uint64_t a, uint64_t b) { return (a >> 32) > (b >> 32); }

RS_HD uint64_t make_elem(uint32_t index, uint32_t count) { return (uint64_t(count) << 32) | index; }

// initial depth budget 2 floor(log2 n)
RS_HD uint32_t depth_budget(uint64_t n) {
  uint32_t l = 0;
  while (n > 1) { n >>= 1; ++l; }
  return 2 * l;
}

template <class A>
RS_HD void swap_at(A& a, int64_t i, int64_t j) {
  const uint64_t t = a[i];
  a[i] = a[j];
  a[j] = t;
}

// Pivot choice of one partition step of [lo, hi) (hi - lo > 16): the median
// (under `before`) of the elements at lo+1, lo+(hi-lo)/2 and hi-1 is
// exchanged with the element at lo, with the reference's tie-breaking.
template <class A>
RS_HD void pivot_to_front(A& a, int64_t lo, int64_t hi) {
  const int64_t x = lo + 1, y = lo + (hi - lo) / 2, z = hi - 1;
  int64_t m;
  if (before(a[x], a[y])) {
    if (before(a[y], a[z])) m = y;
    else if (before(a[x], a[z])) m = z;
    else m = x;
  } else if (before(a[x], a[z])) {
    m = x;
  } else if (before(a[y], a[z])) {
    m = z;
  } else {
    m = y;
  }
  swap_at(a, lo, m);
}

// Hoare partition of [lo+1, hi) around the pivot at lo; returns the cut.
// A left scan stops at the first element not ordered before the pivot, a
// right scan at the first element the pivot is not ordered before; the two
// are exchanged until the scans cross.  The pivot choice guarantees both
// scans stop inside the segment; `ok` turns false if a scan would leave it.
template <class A>
RS_HD int64_t partition_seq(A& a, int64_t lo, int64_t hi, bool& ok) {
  const uint64_t p = a[lo];
  int64_t f = lo + 1, l = hi;
  for (;;) {
    while (f < hi && before(a[f], p)) ++f;
    --l;
    while (l > lo && before(p, a[l])) --l;
    if (f >= hi) { ok = false; return hi - 1; }
    if (!(f < l)) return f;
    swap_at(a, f, l);
    ++f;
  }
}

// One step of the heap sort's sift: the hole at `hole` of the heap
// a[base, base+len) moves down along the child that is not ordered before
// its sibling (the right one on ties) to the bottom, then `v` climbs back up
// from there while its parent is ordered before it.
template <class A>
RS_HD void sift(A& a, int64_t base, int64_t hole, int64_t len, uint64_t v) {
  const int64_t top = hole;
  int64_t child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (before(a[base + child], a[base + child - 1])) --child;
    a[base + hole] = a[base + child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    a[base + hole] = a[base + child - 1];
    hole = child - 1;
  }
  int64_t parent = (hole - 1) / 2;
  while (hole > top && before(a[base + parent], v)) {
    a[base + hole] = a[base + parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[base + hole] = v;
}

// Heap sort of [lo, hi) (the introsort's fallback once the depth budget is
// spent): heapify from the last parent down to the root, then repeatedly
// move the root behind the shrinking heap.
template <class A>
RS_HD void heap_sort(A& a, int64_t lo, int64_t hi) {
  const int64_t len = hi - lo;
  if (len < 2) return;
  for (int64_t parent = (len - 2) / 2;; --parent) {
    sift(a, lo, parent, len, a[lo + parent]);
    if (parent == 0) break;
  }
  for (int64_t end = len - 1; end > 0; --end) {
    const uint64_t v = a[lo + end];
    a[lo + end] = a[lo];
    sift(a, lo, 0, end, v);
  }
}

// Stable insertion sort of [lo, hi) under `before` (the final pass).
template <class A>
RS_HD void insertion_sort(A& a, int64_t lo, int64_t hi) {
  for (int64_t i = lo + 1; i < hi; ++i) {
    const uint64_t v = a[i];
    int64_t j = i;
    while (j > lo && before(v, a[j - 1])) {
      a[j] = a[j - 1];
      --j;
    }
    a[j] = v;
  }
}

// The whole introsort of one segment [lo, hi) with depth budget `depth`,
// followed by the final pass over it.  Parts wait on an explicit stack (the
// order in which disjoint parts are sorted does not matter); the budgets on
// the stack decrease strictly from bottom to top, so it never holds more
// than depth + 1 <= 63 parts.
constexpr int kStack = 64;
template <class A>
RS_HD bool sort_segment(A& a, int64_t lo, int64_t hi, uint32_t depth) {
  int64_t s_lo[kStack], s_hi[kStack];
  uint32_t s_d[kStack];
  int top = 0;
  bool ok = true;
  s_lo[0] = lo; s_hi[0] = hi; s_d[0] = depth; top = 1;
  while (top > 0) {
    --top;
    int64_t l = s_lo[top], h = s_hi[top];
    uint32_t d = s_d[top];
    while (h - l > int64_t(kThreshold)) {
      if (d == 0) {
        heap_sort(a, l, h);
        break;
      }
      --d;
      pivot_to_front(a, l, h);
      const int64_t cut = partition_seq(a, l, h, ok);
      if (!ok) return false;
      if (top == kStack) return false;
      s_lo[top] = cut; s_hi[top] = h; s_d[top] = d; ++top;
      h = cut;
    }
  }
  insertion_sort(a, lo, hi);
  return true;
}

// Parallel form of one partition step.  For the range [lo+1, hi) with pivot
// p, call an element an L-candidate when it is not ordered before p (the
// left scan stops there) and an R-candidate when p is not ordered before it
// (the right scan stops there); an element equal to p is both.  With L[k]
// the k-th L-candidate from the left and R[k] the k-th R-candidate from the
// right, the sequential partition exchanges L[k] with R[k] for k = 0, 1, ...
// while L[k] < R[k] (L ascends and R descends, so this holds for exactly the
// first K ranks), and returns cut = L[0] if K = 0, else
// min(L[K], R[K-1]) (L[K] taken as infinite when absent): after the last
// exchange the left scan stops at the next original L-candidate or at an
// exchanged R position, whichever comes first.  Per element, from counts
// over the range only:
//   L-candidate of rank kL (kL L-candidates before it) is exchanged iff at
//     least kL + 1 R-candidates lie after it;
//   R-candidate of rank kR (kR R-candidates after it) is exchanged iff at
//     least kR + 1 L-candidates lie before it;
// an element is never exchanged in both roles, and the cut is the smallest
// position among the L-candidates that are not exchanged and the
// R-candidates that are.
enum Role : int { kStay = 0, kSwapL = 1, kSwapR = 2 };
RS_HD int classify(bool is_l, bool is_r, uint64_t l_before, uint64_t r_after, bool& cut_candidate) {
  if (is_l && r_after >= l_before + 1) { cut_candidate = false; return kSwapL; }
  if (is_r && l_before >= r_after + 1) { cut_candidate = true; return kSwapR; }
  cut_candidate = is_l;
  return kStay;
}

}  // namespace refsort
}  // namespace svdag
