// GeomOctree::buildDAG on the GPU (src/symvox/geom_octree.cpp:289-435).
//
// The reference builds a top SVO of step_level+1 levels, then one sub-octree
// per voxel of the top tree's leaf level -- buildSVO over that voxel's box
// with levels - (step_level+1) levels, then toDAG -- and joins the sub-DAGs
// level by level (top leaf i ascending, voxel j descending), adding each
// sub-DAG's offset to its child pointers, before one toDAG over the whole
// tree.  Node order therefore differs from a single buildSVO + toDAG, and the
// result is kept bit for bit: the chunks here run in the same order through
// the same voxelization and reduction kernels, each on the triangles that
// can touch its box (a conservative box filter in front of the exact test,
// which keeps the triangles' order), and are joined the same way.  Only one
// chunk's SVO is resident at a time; the joined DAG levels are assembled at
// the end.
#include <algorithm>

#include "ctx.cuh"

namespace svdag {
namespace {

// Float AABB of every triangle (min xyz, max xyz).
__global__ void k_tri_aabb(const float* __restrict__ tris, uint64_t n, float* __restrict__ box) {
  for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < n; t += uint64_t(gridDim.x) * blockDim.x) {
    const float* p = tris + 9 * t;
    float b[6];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      b[q] = fminf(fminf(p[q], p[3 + q]), p[6 + q]);
      b[3 + q] = fmaxf(fmaxf(p[q], p[3 + q]), p[6 + q]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) box[6 * t + q] = b[q];
  }
}

// Triangles whose AABB meets the chunk box grown by a margin.  A triangle
// outside it fails the reference's bounding-box test against every child box
// of the chunk's root, so it adds nothing to the chunk (NaN boxes compare
// false and are kept, so the exact test sees them).
struct ChunkBox {
  float lo[3], hi[3];
};
__device__ __forceinline__ bool meets(const float* b, const ChunkBox& c) {
  return !(b[0] > c.hi[0] || b[3] < c.lo[0] || b[1] > c.hi[1] || b[4] < c.lo[1] || b[2] > c.hi[2] || b[5] < c.lo[2]);
}
struct ChunkFlagIn {
  const float* box;
  ChunkBox c;
  __device__ __forceinline__ uint32_t operator()(uint64_t t) const { return meets(box + 6 * t, c) ? 1u : 0u; }
};
struct ChunkListOut {
  const float* box;
  ChunkBox c;
  uint32_t* list;
  __device__ __forceinline__ void operator()(uint64_t t, uint32_t pos) const {
    if (meets(box + 6 * t, c)) list[pos] = uint32_t(t);
  }
};

// Child pointers of one sub-DAG level shifted by the nodes already joined on
// the level below (null pointers stay null).
__global__ void k_offset_children(const uint32_t* __restrict__ src, uint64_t n8, uint32_t off, uint32_t* __restrict__ dst) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n8; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t v = src[i];
    dst[i] = (v == kNull) ? kNull : v + off;
  }
}

struct Chunk {
  std::vector<Level> lev;
};

}  // namespace

void phase_build_dag(Ctx& c, uint32_t levels, uint32_t step_level, const double bb[6]) {
  if (step_level < 1 || step_level + 1 >= levels)
    throw Error(SVDAG_ERR_INVALID_ARG, "buildDAG: need 1 <= stepLevel and stepLevel + 1 < levels");
  const Exec& ex = c.ex;
  const cudaStream_t st = c.stream;
  const uint32_t top = step_level + 1;

  // --- top SVO
  phase_voxelize(c, top, bb);
  const svdag_stats top_st = c.st;
  const double root_side = c.root_side;

  // centres of the top tree's leaf nodes, as its DFS computes them
  // (leavesCenters, geom_octree.cpp:245-246): walk the (small) top tree
  std::vector<std::vector<uint32_t>> thdr(top), tch(top);
  for (uint32_t l = 0; l < top; ++l) {
    const Level& L = c.lev[l];
    thdr[l].resize(L.n);
    if (L.n) SVDAG_CUDA(cudaMemcpyAsync(thdr[l].data(), L.hdr.get(), 4 * L.n, cudaMemcpyDeviceToHost, st));
    if (l + 1 < top) {
      tch[l].resize(8 * L.n);
      if (L.n) SVDAG_CUDA(cudaMemcpyAsync(tch[l].data(), L.ch.get(), 32 * L.n, cudaMemcpyDeviceToHost, st));
    }
  }
  SVDAG_CUDA(cudaStreamSynchronize(st));
  const uint64_t n_top = c.lev[top - 1].n;
  std::vector<double> centers(3 * n_top);
  {
    struct W { uint32_t lev, id; double c[3]; };
    W root{0, 0, {(bb[0] + bb[3]) * 0.5, (bb[1] + bb[4]) * 0.5, (bb[2] + bb[5]) * 0.5}};
    std::vector<W> stack{root};
    while (!stack.empty()) {
      const W w = stack.back();
      stack.pop_back();
      if (w.lev + 1 >= top) continue;
      const double k = root_side / double(1ull << (w.lev + 2));  // getHalfSideD(lev+1)
      for (int i = 0; i < 8; ++i) {
        const uint32_t ch = tch[w.lev][8ull * w.id + i];
        if (ch == kNull) continue;
        W n{w.lev + 1, ch, {w.c[0] + ((i & 4) ? k : -k), w.c[1] + ((i & 2) ? k : -k), w.c[2] + ((i & 1) ? k : -k)}};
        if (n.lev == top - 1)
          for (int q = 0; q < 3; ++q) centers[3ull * ch + q] = n.c[q];
        stack.push_back(n);
      }
    }
  }
  const double lhs = root_side / double(1ull << top);  // getHalfSideD(stepLevels - 1)

  // --- triangle boxes for the chunk filter
  DBuf<float> tbox(6 * (c.n_tris ? c.n_tris : 1), st);
  if (c.n_tris) SVDAG_LAUNCH(ex, k_tri_aabb, grid_for(ex, c.n_tris, 256), 256, 0, c.tris, c.n_tris, tbox.get());
  DBuf<uint32_t> list(c.n_tris ? c.n_tris : 1, st), d_cnt(1, st);

  // --- one sub-octree per top voxel, in join order
  std::vector<Chunk> chunks;
  std::vector<uint32_t> top_children(8 * n_top, kNull);
  std::vector<uint64_t> count(levels, 0);  // nodes joined so far per level
  uint64_t svo_nodes = top_st.n_nodes_svo, svo_last = 0, vox = top_st.n_total_voxels;
  uint64_t pairs = top_st.frontier_pairs, fallbacks = top_st.sat_fallbacks;
  for (uint64_t i = 0; i < n_top; ++i) {
    for (int j = 7; j >= 0; --j) {
      if (!((thdr[top - 1][i] >> j) & 1u)) continue;
      const double* cc = &centers[3 * i];
      double sb[6];
      for (int q = 0; q < 3; ++q) {
        const double e = cc[q] + (((j >> (2 - q)) & 1) ? lhs : -lhs);
        sb[q] = std::min(cc[q], e);
        sb[3 + q] = std::max(cc[q], e);
      }
      // candidate triangles: float box of the chunk grown by a margin far
      // above the float / double roundings of its root box and centres
      ChunkBox cb;
      for (int q = 0; q < 3; ++q) {
        const double m = 1e-5 * (sb[3 + q] - sb[q]) + 1e-6 * std::max(std::fabs(sb[q]), std::fabs(sb[3 + q])) + 1e-30;
        cb.lo[q] = float(sb[q] - m);
        cb.hi[q] = float(sb[3 + q] + m);
        cb.lo[q] = std::nextafter(cb.lo[q], -INFINITY);
        cb.hi[q] = std::nextafter(cb.hi[q], INFINITY);
      }
      device_exclusive_scan<uint32_t>(ex, ChunkFlagIn{tbox.get(), cb}, c.n_tris, ChunkListOut{tbox.get(), cb, list.get()},
                                      d_cnt.get());
      const uint64_t n_list = read_scalar(ex, d_cnt.get());

      Ctx sub;
      sub.device = c.device;
      sub.stream = st;
      sub.ex = c.ex;
      sub.tris = c.tris;
      sub.n_tris = c.n_tris;
      phase_voxelize(sub, levels - top, sb, list.get(), n_list);
      svo_nodes += sub.st.n_nodes_svo;
      svo_last += sub.st.n_nodes_last_lev_svo;
      vox += sub.st.n_total_voxels - 1;  // the sub-root is the top voxel itself (wraps like the reference's size_t)
      pairs += sub.st.frontier_pairs;
      fallbacks += sub.st.sat_fallbacks;
      phase_reduce_dag(sub);

      top_children[8 * i + j] = uint32_t(count[top]);
      Chunk ch;
      ch.lev = std::move(sub.lev);
      for (uint32_t k = 0; k < levels - top; ++k) {
        count[top + k] += ch.lev[k].n;
        if (count[top + k] >= 0xFFFFFFF0ull) throw Error(SVDAG_ERR_OVERFLOW, "buildDAG: more than 2^32 nodes on a level");
        ch.lev[k].ctr.release();
        ch.lev[k].nbox.release();
      }
      chunks.push_back(std::move(ch));
    }
  }
  tbox.release();
  list.release();

  // --- join: top levels stay, the top leaf level gets child pointers, and
  // every deeper level is the concatenation of the sub-DAG levels
  c.lev.resize(levels);
  {
    Level& T = c.lev[top - 1];
    T.ch.alloc(8 * (n_top ? n_top : 1), st);
    if (n_top)
      SVDAG_CUDA(cudaMemcpyAsync(T.ch.get(), top_children.data(), 32 * n_top, cudaMemcpyHostToDevice, st));
  }
  for (uint32_t k = top; k < levels; ++k) {
    Level& L = c.lev[k];
    L = Level();
    L.n = count[k];
    L.hdr.alloc(L.n ? L.n : 1, st);
    const bool inner = k + 1 < levels;
    if (inner) L.ch.alloc(8 * (L.n ? L.n : 1), st);
    uint64_t base = 0, base_next = 0;
    for (auto& ch : chunks) {
      const Level& S = ch.lev[k - top];
      if (S.n) {
        SVDAG_CUDA(cudaMemcpyAsync(L.hdr.get() + base, S.hdr.get(), 4 * S.n, cudaMemcpyDeviceToDevice, st));
        if (inner)
          SVDAG_LAUNCH(ex, k_offset_children, grid_for(ex, 8 * S.n, 256), 256, 0, S.ch.get(), 8 * S.n,
                       uint32_t(base_next), L.ch.get() + 8 * base);
      }
      base += S.n;
      if (inner) base_next += ch.lev[k + 1 - top].n;
    }
  }
  SVDAG_CUDA(cudaStreamSynchronize(st));
  chunks.clear();

  c.levels = levels;
  c.state = SVDAG_S_SVO;
  c.child_levels_init = false;
  c.st.levels = levels;
  c.st.n_nodes_svo = svo_nodes;
  c.st.n_nodes_last_lev_svo = svo_last;
  c.st.n_total_voxels = vox;
  c.st.frontier_pairs = pairs;
  c.st.sat_fallbacks = fallbacks;
  phase_reduce_dag(c);
}

}  // namespace svdag
