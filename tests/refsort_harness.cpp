// CPU check of the reference-count order restatement (refsort.cuh) against
// libstdc++'s std::sort itself, as EncodedSSVDAG::encode calls it
// (src/symvox/encoded_ssvdag.cpp:266-276): a vector of (index, count) pairs
// sorted by "count(a) > count(b)".
//
// Three forms are compared on many seeded count arrays:
//   seq    sort_segment over the whole array (the sequential introsort);
//   par    the GPU's round structure run sequentially: parallel-form
//          partitions (classify) of parts above a size limit, sequential
//          sort of the parts below it, heap sort when the budget runs out;
//   heap   heap_sort against std::partial_sort(first, last, last).
// Prints one line per failing case and "ok <cases>" at the end.  With
// arguments "adversary N FILE" it writes the adversary counts below instead.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <string>
#include <utility>
#include <vector>

#include "refsort.cuh"

using namespace svdag::refsort;

static std::vector<uint32_t> reference_order(const std::vector<uint32_t>& counts) {
  std::vector<std::pair<uint32_t, uint32_t>> hist(counts.size());
  for (uint32_t i = 0; i < counts.size(); ++i) hist[i] = std::make_pair(i, counts[i]);
  std::sort(hist.begin(), hist.end(),
            [](std::pair<uint32_t, uint32_t> a, std::pair<uint32_t, uint32_t> b) { return a.second > b.second; });
  std::vector<uint32_t> o(counts.size());
  for (size_t k = 0; k < hist.size(); ++k) o[k] = hist[k].first;
  return o;
}

static std::vector<uint64_t> elems(const std::vector<uint32_t>& counts) {
  std::vector<uint64_t> a(counts.size());
  for (uint32_t i = 0; i < counts.size(); ++i) a[i] = make_elem(i, counts[i]);
  return a;
}

static std::vector<uint32_t> order_of(const std::vector<uint64_t>& a) {
  std::vector<uint32_t> o(a.size());
  for (size_t k = 0; k < a.size(); ++k) o[k] = uint32_t(a[k]);
  return o;
}

static std::vector<uint32_t> seq_order(const std::vector<uint32_t>& counts) {
  std::vector<uint64_t> a = elems(counts);
  uint64_t* p = a.data();
  if (!a.empty() && !sort_segment(p, 0, int64_t(a.size()), depth_budget(a.size()))) return {};
  return order_of(a);
}

// The GPU's rounds, one segment after another.
static std::vector<uint32_t> par_order(const std::vector<uint32_t>& counts, int64_t small_limit) {
  std::vector<uint64_t> a = elems(counts);
  uint64_t* p = a.data();
  const int64_t n = int64_t(a.size());
  if (n == 0) return {};
  struct Seg { int64_t lo, hi; uint32_t d; };
  std::vector<Seg> cur, next;
  if (n <= small_limit) {
    sort_segment(p, 0, n, depth_budget(n));
    return order_of(a);
  }
  cur.push_back({0, n, depth_budget(n)});
  std::vector<int64_t> pos_l(n), pos_r(n);
  while (!cur.empty()) {
    next.clear();
    for (const Seg& g : cur) {
      pivot_to_front(p, g.lo, g.hi);
      const uint64_t pv = a[g.lo];
      uint64_t TR = 0;
      for (int64_t i = g.lo + 1; i < g.hi; ++i) TR += !before(pv, a[i]);
      uint64_t l_before = 0, r_seen = 0, K = 0;
      int64_t cut = g.hi;
      for (int64_t i = g.lo + 1; i < g.hi; ++i) {
        const bool is_l = !before(a[i], pv), is_r = !before(pv, a[i]);
        r_seen += is_r;
        const uint64_t r_after = TR - r_seen;
        bool cc = false;
        const int role = classify(is_l, is_r, l_before, r_after, cc);
        if (role == kSwapL) { pos_l[g.lo + l_before] = i; ++K; }
        if (role == kSwapR) pos_r[g.lo + r_after] = i;
        if (cc) cut = std::min(cut, i);
        l_before += is_l;
      }
      for (uint64_t k = 0; k < K; ++k) std::swap(a[pos_l[g.lo + k]], a[pos_r[g.lo + k]]);
      if (cut <= g.lo || cut >= g.hi) return {};
      const uint32_t d = g.d - 1;
      const int64_t b[3] = {g.lo, cut, g.hi};
      for (int k = 0; k < 2; ++k) {
        const Seg part{b[k], b[k + 1], d};
        if (part.hi - part.lo > small_limit) {
          if (d == 0) heap_sort(p, part.lo, part.hi);
          else next.push_back(part);
        } else if (!sort_segment(p, part.lo, part.hi, d)) {
          return {};
        }
      }
    }
    std::swap(cur, next);
  }
  return order_of(a);
}

static bool heap_ok(const std::vector<uint32_t>& counts) {
  std::vector<std::pair<uint32_t, uint32_t>> hist(counts.size());
  for (uint32_t i = 0; i < counts.size(); ++i) hist[i] = std::make_pair(i, counts[i]);
  std::partial_sort(hist.begin(), hist.end(), hist.end(),
                    [](std::pair<uint32_t, uint32_t> x, std::pair<uint32_t, uint32_t> y) { return x.second > y.second; });
  std::vector<uint64_t> a = elems(counts);
  uint64_t* p = a.data();
  heap_sort(p, 0, int64_t(a.size()));
  for (size_t k = 0; k < a.size(); ++k)
    if (uint32_t(a[k]) != hist[k].first) return false;
  return true;
}

// Counts that drive the introsort into its heap-sort fallback: McIlroy's
// adversary ("A Killer Adversary for Quicksort", 1999) assigns values lazily
// while std::sort runs, so that every pivot is as bad as possible; the
// values it fixes are consistent with every comparison made, hence a fixed
// input with the same comparison sequence.
static std::vector<uint32_t> adversary_counts(size_t n) {
  std::vector<int64_t> val(n);
  const int64_t gas = int64_t(n);
  for (auto& v : val) v = gas;
  int64_t nsolid = 0, candidate = 0;
  std::vector<std::pair<uint32_t, uint32_t>> hist(n);
  for (uint32_t i = 0; i < n; ++i) hist[i] = std::make_pair(i, 0u);
  auto less = [&](std::pair<uint32_t, uint32_t> a, std::pair<uint32_t, uint32_t> b) {
    const uint32_t x = a.first, y = b.first;
    if (val[x] == gas && val[y] == gas) {
      if (int64_t(x) == candidate) val[x] = nsolid++;
      else val[y] = nsolid++;
    }
    if (val[x] == gas) candidate = x;
    else if (val[y] == gas) candidate = y;
    return val[x] < val[y];
  };
  std::sort(hist.begin(), hist.end(), less);
  std::vector<uint32_t> c(n);
  for (size_t i = 0; i < n; ++i) c[i] = uint32_t(gas - val[i]);  // "before" = smaller value
  return c;
}

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "adversary") {
    // writes the adversary's counts for n elements as raw u32
    const std::vector<uint32_t> c = adversary_counts(std::stoull(argv[2]));
    FILE* f = std::fopen(argv[3], "wb");
    if (!f || std::fwrite(c.data(), 4, c.size(), f) != c.size()) return 2;
    std::fclose(f);
    return 0;
  }
  std::mt19937_64 rng(0x5eed);
  int cases = 0, bad = 0;
  const size_t sizes[] = {0, 1, 2, 3, 15, 16, 17, 18, 31, 32, 33, 100, 511, 512, 513, 1000, 1024, 1025, 4097,
                          10000, 65537, 200003};
  for (size_t n : sizes) {
    for (int kind = 0; kind < 9; ++kind) {
      std::vector<uint32_t> c(n);
      if (kind == 8) c = adversary_counts(n);
      for (size_t i = 0; i < n && kind < 8; ++i) {
        switch (kind) {
          case 0: c[i] = 1 + uint32_t(rng() % 3); break;                  // few distinct counts
          case 1: c[i] = uint32_t(rng() % 1000); break;                   // many distinct
          case 2: c[i] = 1; break;                                        // all equal
          case 3: c[i] = uint32_t(i); break;                              // ascending
          case 4: c[i] = uint32_t(n - i); break;                          // descending
          case 5: c[i] = uint32_t(i < n / 2 ? i : n - i); break;          // organ pipe
          case 6: c[i] = 1u + uint32_t(__builtin_ctzll(rng() | (1ull << 20))); break;  // geometric
          default: c[i] = (rng() % 10 == 0) ? uint32_t(rng() % 50000) : 1u; break;   // heavy tail
        }
      }
      const std::vector<uint32_t> ref = reference_order(c);
      const std::vector<uint32_t> s = seq_order(c);
      ++cases;
      if (s != ref) { ++bad; std::printf("seq mismatch n=%zu kind=%d\n", n, kind); }
      for (int64_t lim : {int64_t(16), int64_t(40), int64_t(512)}) {
        const std::vector<uint32_t> q = par_order(c, lim);
        ++cases;
        if (q != ref) { ++bad; std::printf("par mismatch n=%zu kind=%d limit=%lld\n", n, kind, (long long)lim); }
      }
      if (n <= 65537) {
        ++cases;
        if (!heap_ok(c)) { ++bad; std::printf("heap mismatch n=%zu kind=%d\n", n, kind); }
      }
    }
  }
  if (bad) { std::printf("FAILED %d of %d\n", bad, cases); return 1; }
  std::printf("ok %d\n", cases);
  return 0;
}
