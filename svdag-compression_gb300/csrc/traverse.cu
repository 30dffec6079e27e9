// Point queries of an encoded SSVDAG on the GPU: EncodedSSVDAG::traverse
// (src/symvox/encoded_ssvdag.cpp:527-574), one query per thread.
//
// The walk mirrors the query point about the node centre when the pointer it
// followed carries mirror bits, picks the child by comparing with the centre,
// and stops at the first missing child; it returns the depth reached, which
// equals the number of levels when the voxel is set.  The float arithmetic is
// the reference's, operation by operation, with explicitly rounded
// intrinsics (no contraction), so results match its CPU walk bit for bit.
// Inner nodes: a u16 header with a 2-bit pointer-size code per child (0 none,
// 1 one word with mirror bits 13-15, 2/3 two words with mirror bits 29-31 and
// bit 29 taken from the code), pointers for children 7..0; the last two
// levels are 4^3 leaf bricks of 8 bytes (encoded_ssvdag.cpp:580-625).
// One departure, in the leaf lookup: traverse() reads a brick as one byte
// per 2^3 sub-brick, the layout the encoder writes only with its voxel-matrix
// order switched off; by default (encoded_ssvdag.cpp:32) it writes the 64
// voxels in matrix order (:317-345, xyz_to_byte_voxel :119-135) -- local
// voxel (x, y, z) in [0, 4)^3 at bit z + 4y + 16x -- which is what the viewer
// reads and what is read here, so a query reports exactly the built voxels.
#include "ctx.cuh"

namespace svdag {
namespace {

__device__ __forceinline__ uint32_t child_code(const uint16_t* node, int c) { return (node[0] >> (2 * c)) & 3u; }

// Child pointer `c` of the node at `node`; false when its pointer words
// would lie past the end of the inner-node array (`avail` words from `node`).
__device__ bool get_child(const uint16_t* node, uint64_t avail, int c, uint32_t& idx, bool& mx, bool& my, bool& mz) {
  uint64_t off = 1;
  for (int i = 7; i > c; --i) {
    const uint32_t code = child_code(node, i);
    off += code == 0 ? 0 : (code == 1 ? 1 : 2);
  }
  const uint32_t code = child_code(node, c);
  if (off + (code >= 2 ? 2 : 1) > avail) return false;
  const uint16_t* p = node + off;
  idx = 0;
  if (code == 1) {
    idx = p[0];
    mx = (idx >> 13) & 1u;
    my = (idx >> 14) & 1u;
    mz = (idx >> 15) & 1u;
    idx &= ~(7u << 13);
  } else if (code >= 2) {
    // the encoder stores the high half first (encoded_ssvdag.cpp:395-403)
    idx = (uint32_t(p[0]) << 16) | uint32_t(p[1]);
    mx = (idx >> 29) & 1u;
    my = (idx >> 30) & 1u;
    mz = (idx >> 31) & 1u;
    idx &= ~(7u << 29);
    idx |= (code & 1u) << 29;
  }
  return true;
}

struct SsvdagView {
  const uint16_t* inner;
  const uint8_t* leaves;
  const uint32_t* level_off;
  uint64_t n_inner, n_leaves;
  uint32_t n_level_off;
  uint32_t levels;
  float bmin[3], bmax[3];
  float root_side;
};

__device__ __forceinline__ float half_side(const SsvdagView& S, uint32_t level) {
  return __fdiv_rn(S.root_side, float(1u << (level + 1)));
}

// A pointer that leads outside the arrays ends the query with depth -2 and
// raises *bad; the host turns that into an error status.
__global__ void k_traverse(SsvdagView S, const float* __restrict__ pts, uint64_t n, int32_t* __restrict__ out,
                           uint32_t* __restrict__ bad) {
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < n; q += uint64_t(gridDim.x) * blockDim.x) {
    float p[3] = {pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]};
    bool inside = true;
    for (int k = 0; k < 3; ++k) inside = inside && !(p[k] < S.bmin[k] || p[k] > S.bmax[k]);
    if (!inside) { out[q] = -1; continue; }
    uint64_t node_idx = 0;
    uint32_t level = 0;
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = __fmul_rn(__fadd_rn(S.bmin[k], S.bmax[k]), 0.5f);
    bool mx = false, my = false, mz = false;
    bool broken = false;
    while (level < S.levels) {
      if (node_idx >= S.n_inner) { broken = true; break; }
      const uint16_t* node = S.inner + node_idx;
      if (mx) p[0] = __fsub_rn(__fmul_rn(2.f, c[0]), p[0]);
      if (my) p[1] = __fsub_rn(__fmul_rn(2.f, c[1]), p[1]);
      if (mz) p[2] = __fsub_rn(__fmul_rn(2.f, c[2]), p[2]);
      int sel = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
      if (child_code(node, sel) == 0) break;
      ++level;
      float hs = half_side(S, level);
      for (int k = 0; k < 3; ++k) c[k] = __fadd_rn(c[k], (p[k] > c[k]) ? hs : __fmul_rn(-1.f, hs));
      uint32_t child = 0;
      if (!get_child(node, S.n_inner - node_idx, sel, child, mx, my, mz)) { broken = true; break; }
      if (level < S.levels - 2) {
        if (level >= S.n_level_off) { broken = true; break; }
        node_idx = uint64_t(S.level_off[level]) + child;
      } else if (level == S.levels - 2) {
        const uint64_t leaf = uint64_t(child) * 8;
        if (leaf + 8 > S.n_leaves) { broken = true; break; }
        if (mx) p[0] = __fsub_rn(__fmul_rn(2.f, c[0]), p[0]);
        if (my) p[1] = __fsub_rn(__fmul_rn(2.f, c[1]), p[1]);
        if (mz) p[2] = __fsub_rn(__fmul_rn(2.f, c[2]), p[2]);
        sel = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
        // the 2^3 sub-brick `sel` is empty when its 8 voxel bits are
        uint32_t any = 0;
        for (int v = 0; v < 8; ++v) {
          const int b = (2 * (sel & 1) + (v & 1)) + 4 * (2 * ((sel >> 1) & 1) + ((v >> 1) & 1)) +
                        16 * (2 * ((sel >> 2) & 1) + ((v >> 2) & 1));
          any |= (S.leaves[leaf + b / 8] >> (b % 8)) & 1u;
        }
        if (!any) break;
        ++level;
        hs = half_side(S, level);
        for (int k = 0; k < 3; ++k) c[k] = __fadd_rn(c[k], (p[k] > c[k]) ? hs : __fmul_rn(-1.f, hs));
        const int vox = 4 * int(p[0] > c[0]) + 2 * int(p[1] > c[1]) + int(p[2] > c[2]);
        const int bi = 2 * ((sel >> 2) & 1) + ((vox >> 2) & 1), bj = 2 * ((sel >> 1) & 1) + ((vox >> 1) & 1),
                  bk = 2 * (sel & 1) + (vox & 1);
        const int bit = bk + 4 * bj + 16 * bi;  // voxel-matrix order (see the file comment)
        if ((S.leaves[leaf + bit / 8] >> (bit % 8)) & 1u) ++level;
        break;
      }
    }
    if (broken) atomicOr(bad, 1u);
    out[q] = broken ? -2 : int32_t(level);
  }
}

}  // namespace
}  // namespace svdag

extern "C" int svdag_ssvdag_traverse(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                                     const uint32_t* level_offsets, uint32_t n_level_offsets, uint32_t levels,
                                     const float bbox[6], float root_side, const float* points, uint64_t n_points,
                                     int32_t* depth) {
  if (!inner || !leaves || !level_offsets || !bbox || !depth || (n_points && !points) || levels < 3)
    return SVDAG_ERR_INVALID_ARG;
  using svdag::DBuf;
  int status = SVDAG_OK;
  try {
    cudaStream_t st;
    SVDAG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    {
      DBuf<uint16_t> d_inner(n_inner ? n_inner : 1, st);
      DBuf<uint8_t> d_leaves(n_leaves ? n_leaves : 1, st);
      DBuf<uint32_t> d_off(n_level_offsets ? n_level_offsets : 1, st);
      DBuf<float> d_pts(3 * (n_points ? n_points : 1), st);
      DBuf<int32_t> d_out(n_points ? n_points : 1, st);
      DBuf<uint32_t> d_bad(1, st);
      SVDAG_CUDA(cudaMemsetAsync(d_bad.get(), 0, 4, st));
      SVDAG_CUDA(cudaMemcpyAsync(d_inner.get(), inner, 2 * n_inner, cudaMemcpyHostToDevice, st));
      SVDAG_CUDA(cudaMemcpyAsync(d_leaves.get(), leaves, n_leaves, cudaMemcpyHostToDevice, st));
      SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), level_offsets, 4ull * n_level_offsets, cudaMemcpyHostToDevice, st));
      SVDAG_CUDA(cudaMemcpyAsync(d_pts.get(), points, 12 * n_points, cudaMemcpyHostToDevice, st));
      svdag::SsvdagView S{d_inner.get(), d_leaves.get(), d_off.get(), n_inner, n_leaves, n_level_offsets, levels,
                          {bbox[0], bbox[1], bbox[2]}, {bbox[3], bbox[4], bbox[5]}, root_side};
      if (n_points) {
        const unsigned grid = unsigned(std::min<uint64_t>((n_points + 255) / 256, 152 * 16));
        svdag::k_traverse<<<grid, 256, 0, st>>>(S, d_pts.get(), n_points, d_out.get(), d_bad.get());
        SVDAG_CUDA(cudaPeekAtLastError());
        SVDAG_CUDA(cudaMemcpyAsync(depth, d_out.get(), 4 * n_points, cudaMemcpyDeviceToHost, st));
      }
      uint32_t bad = 0;
      SVDAG_CUDA(cudaMemcpyAsync(&bad, d_bad.get(), 4, cudaMemcpyDeviceToHost, st));
      SVDAG_CUDA(cudaStreamSynchronize(st));
      if (bad) status = SVDAG_ERR_INVALID_ARG;
    }
    cudaStreamDestroy(st);
    return status;
  } catch (const svdag::Error& e) {
    return e.code;
  }
}
