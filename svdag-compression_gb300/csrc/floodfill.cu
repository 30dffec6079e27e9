// Hidden-geometry flood fill on the GPU: the outside masks of
// GeomOctree::hiddenGeometryFloodfill (src/symvox/geom_octree_extension.cpp:
// 1651-1891) for an SVO.
//
// The reference walks leaf cells (empty child slots at any level and the
// voxel slots of the deepest nodes) from a start cell, visiting face
// neighbours found by octree neighbour search: every neighbour of a reached
// cell is marked outside, and the empty ones are reached in turn.  The
// marked set is therefore
//   C = the empty leaf cells face-connected to the start cell through empty
//       leaf cells, plus every set voxel sharing a face with a cell of C,
// whatever the visiting order, and it is computed here as connected
// components:
//   1. per node its parent and its integer coordinates (top-down);
//   2. every empty leaf cell links to the leaf of size >= its own across each
//      of its 6 faces (up from the cell to the lowest common ancestor, down
//      along the neighbour's coordinates; a subdivided neighbour is skipped:
//      its smaller leaves link back), union-find over the links;
//   3. a node's outside mask: its empty leaf cells in the start cell's
//      component, and its set voxels with a face neighbour there;
//   4. bottom-up, a child node with any outside bit marks its slot.
// The start cell is slot 7 of the deepest node on the child-7 path
// (:1788-1814); when that voxel is set the reference aborts, and here the
// call returns SVDAG_ERR_INVALID_STATE.
//
// Cells are numbered cell(l, n, c) = base_l + 8 n + c over the node levels.
// The union-find links larger roots under smaller ones with atomicCAS and
// halves paths on the way; every pointer goes to a smaller index, so each
// find ends, and the retry loops have iteration limits that raise an error.
#include "ctx.cuh"

namespace svdag {
namespace {

constexpr uint32_t kFFMaxLevels = 21;
constexpr int kFFMaxIters = 1 << 22;

struct FFView {
  const uint32_t* hdr[kFFMaxLevels];
  const uint32_t* ch[kFFMaxLevels];
  uint32_t* par[kFFMaxLevels];
  uint64_t* coord[kFFMaxLevels];  // 21 bits per axis: x << 42 | y << 21 | z
  uint64_t n[kFFMaxLevels];
  uint64_t base[kFFMaxLevels + 1];
  uint32_t levels;
};

__device__ __forceinline__ uint32_t axis_of(uint64_t p, int a) { return uint32_t(p >> (42 - 21 * a)) & 0x1FFFFFu; }

__device__ __forceinline__ bool is_leaf(const FFView& V, uint32_t l, uint64_t node, int c) {
  return l + 1 == V.levels || V.ch[l][8 * node + c] == kNull;
}

__device__ __forceinline__ bool is_set(const FFView& V, uint32_t l, uint64_t node, int c) {
  return (V.hdr[l][node] >> c) & 1u;
}

__global__ void k_ff_links(FFView V, uint32_t l) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < V.n[l]; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t p = V.coord[l][i];
    for (int c = 0; c < 8; ++c) {
      const uint32_t k = V.ch[l][8 * i + c];
      if (k == kNull) continue;
      V.par[l + 1][k] = uint32_t(i);
      const uint64_t x = 2ull * axis_of(p, 0) + ((c >> 2) & 1), y = 2ull * axis_of(p, 1) + ((c >> 1) & 1),
                     z = 2ull * axis_of(p, 2) + (c & 1);
      V.coord[l + 1][k] = (x << 42) | (y << 21) | z;
    }
  }
}

// The leaf cell of size >= that of cell (l, node, c) across its face
// (axis a, direction s = +-1), or kNone64 outside the root or when the
// neighbour of equal size is subdivided.
constexpr uint64_t kNone64 = ~0ull;

__device__ uint64_t face_neighbour(const FFView& V, uint32_t l, uint64_t node, int c, int a, int s,
                                   uint32_t* found_level = nullptr) {
  const uint32_t d = l + 1;  // depth of the cell
  const uint64_t p = V.coord[l][node];
  uint32_t x[3] = {2 * axis_of(p, 0) + ((c >> 2) & 1), 2 * axis_of(p, 1) + ((c >> 1) & 1), 2 * axis_of(p, 2) + (c & 1)};
  const uint32_t xa = x[a];
  if (s < 0 ? xa == 0 : xa + 1 >= (1u << d)) return kNone64;
  x[a] = s < 0 ? xa - 1 : xa + 1;
  const uint32_t k = 32 - __clz(xa ^ x[a]);  // levels up to the common ancestor (>= 1)
  uint32_t m = l;
  uint64_t nd = node;
  for (uint32_t i = 1; i < k; ++i) {
    nd = V.par[m][nd];
    --m;
  }
  for (;;) {
    const uint32_t sh = d - 1 - m;
    const int cc = int((((x[0] >> sh) & 1u) << 2) | (((x[1] >> sh) & 1u) << 1) | ((x[2] >> sh) & 1u));
    if (found_level) *found_level = m;
    if (m + 1 == V.levels) return V.base[m] + 8 * nd + cc;
    const uint32_t q = V.ch[m][8 * nd + cc];
    if (q == kNull) return V.base[m] + 8 * nd + cc;
    if (m + 1 == d) return kNone64;
    nd = q;
    ++m;
  }
}

__device__ __forceinline__ bool empty_leaf_cell(const FFView& V, uint64_t g) {
  uint32_t l = 0;
  while (l + 1 < V.levels && V.base[l + 1] <= g) ++l;
  const uint64_t r = g - V.base[l];
  return is_leaf(V, l, r >> 3, int(r & 7)) && !is_set(V, l, r >> 3, int(r & 7));
}

__device__ uint32_t uf_find(uint32_t* P, uint32_t x, uint32_t* err) {
  for (int it = 0; it < kFFMaxIters; ++it) {
    const uint32_t p = __ldcg(&P[x]);
    if (p == x) return x;
    const uint32_t gp = __ldcg(&P[p]);
    if (gp != p) P[x] = gp;  // path halving: gp is an ancestor of x
    x = gp;
  }
  atomicOr(err, 1u);
  return x;
}

__device__ void uf_unite(uint32_t* P, uint32_t a, uint32_t b, uint32_t* err) {
  for (int it = 0; it < kFFMaxIters; ++it) {
    a = uf_find(P, a, err);
    b = uf_find(P, b, err);
    if (a == b) return;
    if (a < b) {
      const uint32_t t = a;
      a = b;
      b = t;
    }
    const uint32_t old = atomicCAS(&P[a], a, b);
    if (old == a) return;
    a = old;
  }
  atomicOr(err, 1u);
}

__global__ void k_ff_init(uint32_t* P, uint64_t n) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    P[i] = uint32_t(i);
}

__global__ void k_ff_unite(FFView V, uint32_t l, uint32_t* P, uint32_t* err) {
  const uint64_t cells = 8 * V.n[l];
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < cells; r += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t node = r >> 3;
    const int c = int(r & 7);
    if (!is_leaf(V, l, node, c) || is_set(V, l, node, c)) continue;
    const uint32_t g = uint32_t(V.base[l] + r);
    for (int dir = 0; dir < 6; ++dir) {
      uint32_t fl = 0;
      const uint64_t nb = face_neighbour(V, l, node, c, dir % 3, dir < 3 ? -1 : 1, &fl);
      // a neighbour of the same size links to this cell across its + face
      if (nb == kNone64 || (dir < 3 && fl == l) || !empty_leaf_cell(V, nb)) continue;
      uf_unite(P, g, uint32_t(nb), err);
    }
  }
}

__global__ void k_ff_flatten(uint32_t* P, uint64_t n, uint32_t* err) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    P[i] = uf_find(P, uint32_t(i), err);
}

// The start cell and whether its voxel / slot is set (one thread).
__global__ void k_ff_start(FFView V, uint64_t* start, uint32_t* start_set) {
  uint64_t nd = 0;
  for (uint32_t m = 0; m < V.levels; ++m) {
    if (m + 1 == V.levels || V.ch[m][8 * nd + 7] == kNull) {
      *start = V.base[m] + 8 * nd + 7;
      *start_set = is_set(V, m, nd, 7) ? 1u : 0u;
      return;
    }
    nd = V.ch[m][8 * nd + 7];
  }
}

__global__ void k_ff_masks(FFView V, uint32_t l, const uint32_t* __restrict__ P, const uint64_t* start,
                           uint8_t* __restrict__ out, unsigned long long* counts) {
  const uint32_t root = P[*start];
  unsigned long long ne = 0, ns = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < V.n[l]; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t mask = 0;
    for (int c = 0; c < 8; ++c) {
      if (!is_leaf(V, l, i, c)) continue;
      if (!is_set(V, l, i, c)) {
        if (P[V.base[l] + 8 * i + c] == root) {
          mask |= 1u << c;
          ++ne;
        }
        continue;
      }
      for (int dir = 0; dir < 6; ++dir) {  // a set voxel: outside when a face neighbour is
        const uint64_t nb = face_neighbour(V, l, i, c, dir % 3, dir < 3 ? -1 : 1);
        if (nb != kNone64 && empty_leaf_cell(V, nb) && P[nb] == root) {
          mask |= 1u << c;
          ++ns;
          break;
        }
      }
    }
    out[i] = uint8_t(mask);
  }
  for (int o = 16; o; o >>= 1) {
    ne += __shfl_down_sync(0xFFFFFFFFu, ne, o);
    ns += __shfl_down_sync(0xFFFFFFFFu, ns, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (ne) atomicAdd(&counts[0], ne);
    if (ns) atomicAdd(&counts[1], ns);
  }
}

__global__ void k_ff_propagate(const uint32_t* __restrict__ ch, uint64_t n, const uint8_t* __restrict__ below,
                               uint8_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t mask = out[i];
    for (int c = 0; c < 8; ++c) {
      const uint32_t k = ch[8 * i + c];
      if (k != kNull && below[k] != 0) mask |= 1u << c;
    }
    out[i] = uint8_t(mask);
  }
}

}  // namespace

void phase_flood_fill(Ctx& c, uint64_t* n_empty, uint64_t* n_surface) {
  if (c.state != SVDAG_S_SVO) throw Error(SVDAG_ERR_INVALID_STATE, "hiddenGeometryFloodfill: not in SVO state");
  if (c.levels < 1 || c.levels > kFFMaxLevels) throw Error(SVDAG_ERR_INVALID_ARG, "flood fill: levels must be 1..21");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t L = c.levels;
  FFView V{};
  V.levels = L;
  std::vector<DBuf<uint32_t>> par(L);
  std::vector<DBuf<uint64_t>> coord(L);
  uint64_t cells = 0;
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t n = c.lev[l].n;
    V.hdr[l] = c.lev[l].hdr.get();
    V.ch[l] = l + 1 < L ? c.lev[l].ch.get() : nullptr;
    V.n[l] = n;
    V.base[l] = cells;
    cells += 8 * n;
    par[l].alloc(n ? n : 1, st);
    coord[l].alloc(n ? n : 1, st);
    V.par[l] = par[l].get();
    V.coord[l] = coord[l].get();
  }
  V.base[L] = cells;
  if (cells >= (1ull << 32)) throw Error(SVDAG_ERR_OVERFLOW, "flood fill: more than 2^32 cells");
  SVDAG_CUDA(cudaMemsetAsync(V.coord[0], 0, 8, st));
  for (uint32_t l = 0; l + 1 < L; ++l)
    if (V.n[l]) SVDAG_LAUNCH(ex, k_ff_links, grid_for(ex, V.n[l], 256), 256, 0, V, l);
  DBuf<uint32_t> P(cells ? cells : 1, st);
  DBuf<uint32_t> d_err(2, st);
  DBuf<uint64_t> d_start(1, st);
  DBuf<unsigned long long> d_counts(2, st);
  SVDAG_CUDA(cudaMemsetAsync(d_err.get(), 0, 8, st));
  SVDAG_CUDA(cudaMemsetAsync(d_counts.get(), 0, 16, st));
  SVDAG_LAUNCH(ex, k_ff_start, 1, 1, 0, V, d_start.get(), d_err.get() + 1);
  SVDAG_LAUNCH(ex, k_ff_init, grid_for(ex, cells, 256), 256, 0, P.get(), cells);
  for (uint32_t l = 0; l < L; ++l)
    if (V.n[l]) SVDAG_LAUNCH(ex, k_ff_unite, grid_for(ex, 8 * V.n[l], 256), 256, 0, V, l, P.get(), d_err.get());
  SVDAG_LAUNCH(ex, k_ff_flatten, grid_for(ex, cells, 256), 256, 0, P.get(), cells, d_err.get());
  uint32_t err[2];
  SVDAG_CUDA(cudaMemcpyAsync(err, d_err.get(), 8, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  if (err[0]) throw Error(SVDAG_ERR_TIMEOUT, "flood fill: union-find iteration limit reached");
  if (err[1])
    throw Error(SVDAG_ERR_INVALID_STATE, "hiddenGeometryFloodfill: the corner cell intersects geometry");
  for (uint32_t l = 0; l < L; ++l) {
    c.lev[l].outm.alloc(V.n[l] ? V.n[l] : 1, st);
    if (V.n[l])
      SVDAG_LAUNCH(ex, k_ff_masks, grid_for(ex, V.n[l], 256), 256, 0, V, l, P.get(), d_start.get(),
                   c.lev[l].outm.get(), d_counts.get());
  }
  for (int l = int(L) - 2; l >= 0; --l)
    if (V.n[l])
      SVDAG_LAUNCH(ex, k_ff_propagate, grid_for(ex, V.n[l], 256), 256, 0, V.ch[l], V.n[l], c.lev[l + 1].outm.get(),
                   c.lev[l].outm.get());
  unsigned long long counts[2];
  SVDAG_CUDA(cudaMemcpyAsync(counts, d_counts.get(), 16, cudaMemcpyDeviceToHost, st));
  SVDAG_CUDA(cudaStreamSynchronize(st));
  if (n_empty) *n_empty = counts[0];
  if (n_surface) *n_surface = counts[1];
}

}  // namespace svdag

extern "C" int svdag_flood_fill(svdag_ctx* h, uint64_t* n_outside_empty, uint64_t* n_outside_surface) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    svdag::phase_flood_fill(c, n_outside_empty, n_outside_surface);
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    for (auto& L : c.lev) L.outm.release();
    c.last_error = e.what();
    return e.code;
  }
}

extern "C" int svdag_download_outside_masks(svdag_ctx* h, uint32_t level, uint8_t* masks) {
  if (!h || !masks) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    if (level >= c.lev.size()) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "outside masks: no such level");
    const svdag::Level& L = c.lev[level];
    if (c.state != SVDAG_S_SVO || !L.outm.get())
      throw svdag::Error(SVDAG_ERR_INVALID_STATE, "outside masks: no flood fill on the current SVO");
    if (L.n) SVDAG_CUDA(cudaMemcpyAsync(masks, L.outm.get(), L.n, cudaMemcpyDeviceToHost, c.stream));
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  }
}
