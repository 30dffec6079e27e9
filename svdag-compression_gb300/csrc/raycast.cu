// Ray casting of an encoded SSVDAG on the GPU: the viewer's fragment-shader
// traversal (shaders/octree_dda.frag.glsl, SSVDAG variant) as a CUDA kernel
// writing a headless per-pixel buffer, one ray per thread.
//
// Per pixel the kernel builds the camera ray (computeCameraRay, :587-604),
// moves it into the octree's unit cube and clips it to the scene box
// (transform_ray, :480-507), and walks the octree with the shader's
// hierarchical DDA (init / dda_next / down_in / up_in, :373-537) over the
// u16 inner nodes and 4^3 leaf bricks, accumulating child mirror flags and
// mirroring local cell indices (voxel_to_linear_idx, :149-152).  Its result
// is trace_ray's (:539-581): the hit distance in world units (or -1 no hit
// inside the box, -2 past t_max, -3 iteration limit, -4 outside the box),
// the shader level of the hit, the iterations used and the node index, plus
// the hit cell's grid coordinates and the entry face normal.
//
// The float arithmetic is the shader's, operation by operation, in IEEE
// single precision with explicit rounding (no contraction): mat4 x vec4 sums
// the column products left to right; normalize divides by a correctly
// rounded square root; min / max / sign follow the GLSL definitions.  One
// departure: transform_ray replaces a direction component below 1e-4 in
// magnitude by sign(d) * 1e-4, which leaves an exact zero at zero (sign 0)
// and divides by it; here an exact zero becomes +1e-4.  Every array access
// is bounds-checked; a pointer outside the arrays ends the ray with the
// status -5 and the call returns SVDAG_ERR_INVALID_ARG.
#include "ctx.cuh"

namespace svdag {

struct SsvdagDev {
  int device = 0;
  cudaStream_t stream = nullptr;
  DBuf<uint16_t> inner;
  DBuf<uint8_t> leaves;
  DBuf<uint32_t> level_off;
  uint64_t n_inner = 0, n_leaves = 0;
  uint32_t n_level_off = 0, levels = 0;
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  float root_side = 0.f;
};

namespace {

constexpr int kMaxStack = 30;  // one entry per inner level at most (levels <= 30)

#ifndef SVDAG_RAY_MIN_BLOCKS
#define SVDAG_RAY_MIN_BLOCKS 8
#endif

struct RayView {
  const uint16_t* inner;
  const uint32_t* leaves;  // two words per 4^3 brick
  const uint32_t* level_off;
  uint64_t n_inner, n_bricks;
  uint32_t n_level_off, inner_levels;
  float bmin[3], bmax[3], center[3], root_half;
  float view_inv[16], proj_inv[16];
  float res[2];
  uint32_t width, height, max_iters, draw_level;
  float proj_factor, t_min, t_max;
};

__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gsign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }

// column-major M (M[4c + r]) times (x, y, z, w)
__device__ void mat_vec(const float* M, const float v[4], float out[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r)
    out[r] = add(add(add(mul(M[r], v[0]), mul(M[4 + r], v[1])), mul(M[8 + r], v[2])), mul(M[12 + r], v[3]));
}

__device__ void normalize3(float v[3]) {
  const float l = __fsqrt_rn(add(add(mul(v[0], v[0]), mul(v[1], v[1])), mul(v[2], v[2])));
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = dvd(v[k], l);
}

struct Trav {
  float t;
  int node;
  uint32_t hdr;
  int mir[3];
  uint32_t leaf[2];
  int idx[3], loc[3];
  uint32_t lin;
  float tn[3], inv[3];
  int step[3];
  int size;
  float cell;
  uint32_t level;
};

__device__ __forceinline__ uint32_t code_of(uint32_t hdr, uint32_t c) { return (hdr >> (c << 1)) & 3u; }

__device__ __forceinline__ uint32_t linear_index(const Trav& s) {
  int l[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (s.loc[k] < 0 || s.loc[k] >= s.size) return 0xFFFFFFFFu;
    l[k] = (1 - 2 * s.mir[k]) * s.loc[k] + s.mir[k] * (s.size - 1);
  }
  return uint32_t(l[2] + s.size * (l[1] + s.size * l[0]));
}

__device__ __forceinline__ bool fetch_data(const RayView& V, Trav& s) {
  if (s.level < V.inner_levels) {
    if (s.level >= V.n_level_off) return false;
    const uint64_t g = uint64_t(V.level_off[s.level]) + uint32_t(s.node);
    if (g >= V.n_inner) return false;
    s.hdr = V.inner[g];
  } else {
    if (uint64_t(uint32_t(s.node)) >= V.n_bricks) return false;
    s.leaf[0] = V.leaves[2 * uint64_t(uint32_t(s.node))];
    s.leaf[1] = V.leaves[2 * uint64_t(uint32_t(s.node)) + 1];
  }
  return true;
}

__device__ __forceinline__ bool voxel_bit(const RayView& V, const Trav& s) {
  if (s.level < V.inner_levels) return s.lin < 8 && code_of(s.hdr, s.lin) != 0;
  if (s.lin >= 64) return false;
  return ((s.lin & 32) == 0 ? s.leaf[0] : s.leaf[1]) & (1u << (s.lin & 31));
}

__device__ __forceinline__ bool child_in(const RayView& V, Trav& s) {
  if (s.level >= V.n_level_off || s.lin >= 8) return false;
  uint64_t off = 1 + uint64_t(V.level_off[s.level]) + uint32_t(s.node);
  for (uint32_t i = 7; i > s.lin; --i) off += min(code_of(s.hdr, i), 2u);
  const uint32_t code = code_of(s.hdr, s.lin);
  if (off + (code > 1 ? 2 : 1) > V.n_inner) return false;
  int x = V.inner[off];
  const int m[3] = {(x >> 13) & 1, (x >> 14) & 1, (x >> 15) & 1};
  x &= ~(7 << 13);
  if (code > 1) {
    x = (x << 16) | int(V.inner[off + 1]);
    x |= int(code & 1u) << 29;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) s.mir[k] ^= m[k];
  s.node = x;
  return true;
}

__device__ __forceinline__ void crossings(const float o[3], Trav& s) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float p_next = mul(float(s.idx[k] + max(0, s.step[k])), s.cell);
    s.tn[k] = mul(sub(p_next, o[k]), s.inv[k]);
  }
}

__device__ __forceinline__ void go_down_one_level(const float o[3], const float d[3], Trav& s) {
  ++s.level;
  s.cell = mul(s.cell, 0.5f);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float p_a = add(o[k], mul(s.t, d[k]));
    const float p_center = mul(float(s.idx[k] * 2 + 1), s.cell);
    s.idx[k] = s.idx[k] * 2 + int(p_center < p_a);
  }
  crossings(o, s);
#pragma unroll
  for (int k = 0; k < 3; ++k) s.loc[k] = s.idx[k] & (s.size - 1);
}

// the axis of the next crossing as a 0/1 mask (all zero on ties that the
// shader's comparisons leave unresolved)
__device__ __forceinline__ void next_mask(const Trav& s, int m[3]) {
  m[0] = (s.tn[0] < s.tn[1]) && (s.tn[0] <= s.tn[2]);
  m[1] = (s.tn[1] < s.tn[2]) && (s.tn[1] <= s.tn[0]);
  m[2] = (s.tn[2] < s.tn[0]) && (s.tn[2] <= s.tn[1]);
}

struct Stack {
  int node[kMaxStack];
  uint32_t hdr[kMaxStack];
  int mask[kMaxStack];
  uint32_t n;
};

// Pixels go to threads in 16 x 8 tiles per block, 8 x 4 per warp: rays of
// one warp start close together and stay in step longer than along a row.
constexpr int kRayThreads = 128;
constexpr uint32_t kTileW = 16, kTileH = 8;

__global__ void __launch_bounds__(kRayThreads, SVDAG_RAY_MIN_BLOCKS)
    k_raycast(RayView V, svdag_ray_hit* __restrict__ out, uint32_t* __restrict__ bad) {
  const uint32_t tiles_x = (V.width + kTileW - 1) / kTileW;
  const uint64_t tiles = uint64_t(tiles_x) * ((V.height + kTileH - 1) / kTileH);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ox = (warp & 1) * 8 + (lane & 7), oy = (warp >> 1) * 4 + (lane >> 3);
  for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t px = uint32_t(tile % tiles_x) * kTileW + ox, py = uint32_t(tile / tiles_x) * kTileH + oy;
    if (px >= V.width || py >= V.height) continue;
    const uint64_t q = uint64_t(py) * V.width + px;
    svdag_ray_hit h{};
    h.node = -1;
    // computeCameraRay
    const float sx = sub(mul(dvd(add(float(px), 0.5f), V.res[0]), 2.f), 1.f);
    const float sy = sub(mul(dvd(add(float(py), 0.5f), V.res[1]), 2.f), 1.f);
    float o[3], d[3];
    {
      const float s0[4] = {sx, sy, 0.f, 1.f}, s1[4] = {sx, sy, 1.f, 1.f};
      float w0[4], w1[4];
      mat_vec(V.proj_inv, s0, w0);
      mat_vec(V.proj_inv, s1, w1);
      float dd[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) dd[k] = sub(dvd(w1[k], w1[3]), dvd(w0[k], w0[3]));
      normalize3(dd);
      const float z4[4] = {0.f, 0.f, 0.f, 1.f}, e4[4] = {dd[0], dd[1], dd[2], 1.f};
      float op[4], ep[4];
      mat_vec(V.view_inv, z4, op);
      mat_vec(V.view_inv, e4, ep);
#pragma unroll
      for (int k = 0; k < 3; ++k) { o[k] = op[k]; d[k] = sub(ep[k], op[k]); }
      normalize3(d);
    }
    // transform_ray
    float tmin = V.t_min, tmax = V.t_max;
    bool inside;
    {
      const float eps = 1e-4f;
      const float scale = dvd(1.f, mul(2.f, V.root_half));
      float omin[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        omin[k] = sub(V.center[k], V.root_half);
        o[k] = mul(sub(o[k], omin[k]), scale);
        const float sg = gsign(d[k]);
        if (sg == 0.f) d[k] = eps;
        else if (mul(d[k], sg) < eps) d[k] = mul(sg, eps);
      }
      tmin = mul(tmin, scale);
      tmax = mul(tmax, scale);
      float t1[3], t2[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float cmin = mul(sub(V.bmin[k], omin[k]), scale), cmax = mul(sub(V.bmax[k], omin[k]), scale);
        t1[k] = dvd(sub(cmin, o[k]), d[k]);
        t2[k] = dvd(sub(cmax, o[k]), d[k]);
      }
      float tlo[3], thi[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) { tlo[k] = gmin(t1[k], t2[k]); thi[k] = gmax(t1[k], t2[k]); }
      const float ti0 = gmax(gmax(tlo[0], 0.f), gmax(tlo[1], tlo[2]));
      const float ti1 = gmin(thi[0], gmin(thi[1], thi[2]));
      tmin = gmax(ti0, add(tmin, 1e-10f));
      tmax = gmin(ti1, tmax);
      inside = ti0 < ti1;
    }
    if (!inside) {
      h.t = -4.f;
      out[q] = h;
      continue;
    }
    const float wscale = mul(2.f, V.root_half);
    Trav s;
    Stack st;
    st.n = 0;
    s.t = tmin;
    // init
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      s.inv[k] = dvd(1.f, d[k]);
      s.step[k] = int(gsign(d[k]));
      s.mir[k] = 0;
    }
    s.level = 0;
    s.cell = 0.5f;
    {  // dda_init
      const float voxel_eps = dvd(1.f, mul(256.f, 1024.f));
      const float tt = add(s.t, voxel_eps);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float p_a = add(o[k], mul(tt, d[k]));
        s.idx[k] = f2i(dvd(p_a, s.cell));
      }
      crossings(o, s);
#pragma unroll
      for (int k = 0; k < 3; ++k) s.loc[k] = s.idx[k] % 2;
    }
    s.size = 2;
    s.node = 0;
    bool broken = !fetch_data(V, s);
    s.lin = linear_index(s);
    int stepdir[3] = {0, 0, 0};
    uint32_t iters = 0;
    const uint32_t max_level = min(V.inner_levels, V.draw_level - 1u);
    bool done = false;
    while (!broken) {
      if (!voxel_bit(V, s)) {
        int m[3];
        next_mask(s, m);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          stepdir[k] = m[k] * s.step[k];
          s.idx[k] += stepdir[k];
          s.loc[k] += stepdir[k];
        }
        s.t = add(add(mul(float(m[0]), s.tn[0]), mul(float(m[1]), s.tn[1])), mul(float(m[2]), s.tn[2]));
#pragma unroll
        for (int k = 0; k < 3; ++k) s.tn[k] = add(s.tn[k], mul(mul(float(m[k]), s.cell), fabsf(s.inv[k])));
        bool inb = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) inb = inb && s.loc[k] >= 0 && s.loc[k] < s.size;
        if (!inb) {
          if (st.n == 0) {
            h.t = -1.f;
            h.iterations = int32_t(iters);
            done = true;
            break;
          }
          // up_in
          uint32_t dl = s.level;
          --st.n;
          s.node = st.node[st.n];
          s.hdr = st.hdr[st.n];
          const int msk = st.mask[st.n];
          s.mir[0] = msk & 1;
          s.mir[1] = (msk >> 1) & 1;
          s.mir[2] = (msk >> 2) & 1;
          s.level = uint32_t(msk >> 3) & 255u;
          dl -= s.level;
#pragma unroll
          for (int k = 0; k < 3; ++k) s.idx[k] >>= dl;
          s.cell = mul(s.cell, float(1 << dl));
          s.size = s.level < V.inner_levels ? 2 : 4;
#pragma unroll
          for (int k = 0; k < 3; ++k) s.loc[k] = s.idx[k] & 1;
          crossings(o, s);
        }
      } else {
        const bool hit = s.level >= max_level || mul(s.cell, V.proj_factor) < s.t;
        if (hit) {
          h.t = mul(s.t, wscale);
          h.level = int32_t(s.level);
          h.iterations = int32_t(iters);
          h.node = s.node;
#pragma unroll
          for (int k = 0; k < 3; ++k) h.voxel[k] = s.idx[k];
          h.normal = (uint32_t(uint8_t(int8_t(-stepdir[0])))) | (uint32_t(uint8_t(int8_t(-stepdir[1]))) << 8) |
                     (uint32_t(uint8_t(int8_t(-stepdir[2]))) << 16);
          done = true;
          break;
        }
        // down_in
        int m[3];
        next_mask(s, m);
        bool push = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int nl = s.loc[k] + m[k] * s.step[k];
          push = push && nl >= 0 && nl < 2;
        }
        if (push) {
          if (st.n >= kMaxStack) { broken = true; break; }
          st.node[st.n] = s.node;
          st.hdr[st.n] = s.hdr;
          st.mask[st.n] = s.mir[0] | (s.mir[1] << 1) | (s.mir[2] << 2) | int(s.level << 3);
          ++st.n;
        }
        if (!child_in(V, s)) { broken = true; break; }
        go_down_one_level(o, d, s);
        if (s.level == V.inner_levels) {
          s.size = 4;
          go_down_one_level(o, d, s);
        }
        if (!fetch_data(V, s)) { broken = true; break; }
      }
      s.lin = linear_index(s);
      ++iters;
      if (!(s.t < tmax && iters < V.max_iters)) break;
    }
    if (broken) {
      atomicOr(bad, 1u);
      h = svdag_ray_hit{};
      h.t = -5.f;
      h.node = -1;
    } else if (!done) {
      h.t = iters >= V.max_iters ? -3.f : -2.f;
      h.iterations = int32_t(iters);
    }
    out[q] = h;
  }
}

}  // namespace
}  // namespace svdag

struct svdag_ssvdag {
  svdag::SsvdagDev d;
};

extern "C" int svdag_ssvdag_upload(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                                   const uint32_t* level_offsets, uint32_t n_level_offsets, uint32_t levels,
                                   const float bbox[6], float root_side, svdag_ssvdag** out) {
  if (!out) return SVDAG_ERR_INVALID_ARG;
  *out = nullptr;
  if ((n_inner && !inner) || (n_leaves && !leaves) || (n_level_offsets && !level_offsets) || !bbox || levels < 3 ||
      levels > 30 || n_leaves % 8 != 0 || !(root_side > 0.f))
    return SVDAG_ERR_INVALID_ARG;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return SVDAG_ERR_NO_DEVICE;
  svdag_ssvdag* h = new svdag_ssvdag;
  svdag::SsvdagDev& D = h->d;
  try {
    SVDAG_CUDA(cudaGetDevice(&D.device));
    SVDAG_CUDA(cudaStreamCreateWithFlags(&D.stream, cudaStreamNonBlocking));
    D.inner = svdag::DBuf<uint16_t>(n_inner ? n_inner : 1, D.stream);
    D.leaves = svdag::DBuf<uint8_t>(n_leaves ? n_leaves : 8, D.stream);
    D.level_off = svdag::DBuf<uint32_t>(n_level_offsets ? n_level_offsets : 1, D.stream);
    if (n_inner) SVDAG_CUDA(cudaMemcpyAsync(D.inner.get(), inner, 2 * n_inner, cudaMemcpyHostToDevice, D.stream));
    if (n_leaves) SVDAG_CUDA(cudaMemcpyAsync(D.leaves.get(), leaves, n_leaves, cudaMemcpyHostToDevice, D.stream));
    if (n_level_offsets)
      SVDAG_CUDA(cudaMemcpyAsync(D.level_off.get(), level_offsets, 4ull * n_level_offsets, cudaMemcpyHostToDevice,
                                 D.stream));
    SVDAG_CUDA(cudaStreamSynchronize(D.stream));
    D.n_inner = n_inner;
    D.n_leaves = n_leaves;
    D.n_level_off = n_level_offsets;
    D.levels = levels;
    for (int k = 0; k < 6; ++k) D.bbox[k] = bbox[k];
    D.root_side = root_side;
    *out = h;
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    cudaStream_t st = D.stream;
    delete h;
    if (st) cudaStreamDestroy(st);
    return e.code;
  }
}

extern "C" int svdag_ssvdag_free(svdag_ssvdag* h) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  cudaStream_t st = h->d.stream;
  cudaSetDevice(h->d.device);
  delete h;  // frees the buffers on the handle's stream
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  return SVDAG_OK;
}

extern "C" int svdag_ssvdag_raycast(svdag_ssvdag* h, const svdag_camera* cam, void* stream, svdag_ray_hit* hits,
                                    int device_buffer) {
  if (!h || !cam || !hits || cam->width == 0 || cam->height == 0) return SVDAG_ERR_INVALID_ARG;
  const svdag::SsvdagDev& D = h->d;
  try {
    SVDAG_CUDA(cudaSetDevice(D.device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : D.stream;
    svdag::RayView V{};
    V.inner = D.inner.get();
    V.leaves = reinterpret_cast<const uint32_t*>(D.leaves.get());
    V.level_off = D.level_off.get();
    V.n_inner = D.n_inner;
    V.n_bricks = D.n_leaves / 8;
    V.n_level_off = D.n_level_off;
    V.inner_levels = D.levels - 2;
    for (int k = 0; k < 3; ++k) {
      V.bmin[k] = D.bbox[k];
      V.bmax[k] = D.bbox[3 + k];
      V.center[k] = (D.bbox[k] + D.bbox[3 + k]) * 0.5f;
    }
    V.root_half = D.root_side * 0.5f;
    for (int k = 0; k < 16; ++k) {
      V.view_inv[k] = cam->view_inv[k];
      V.proj_inv[k] = cam->proj_inv[k];
    }
    V.res[0] = float(cam->width);
    V.res[1] = float(cam->height);
    V.width = cam->width;
    V.height = cam->height;
    V.max_iters = cam->max_iters;
    V.draw_level = cam->draw_level;
    V.proj_factor = cam->projection_factor;
    V.t_min = cam->t_min;
    V.t_max = cam->t_max;
    const uint64_t npix = uint64_t(cam->width) * cam->height;
    svdag::DBuf<uint32_t> d_bad(1, st);
    SVDAG_CUDA(cudaMemsetAsync(d_bad.get(), 0, 4, st));
    svdag::DBuf<svdag_ray_hit> tmp;
    svdag_ray_hit* dst = hits;
    if (!device_buffer) {
      tmp = svdag::DBuf<svdag_ray_hit>(npix, st);
      dst = tmp.get();
    }
    const uint64_t tiles = uint64_t((cam->width + svdag::kTileW - 1) / svdag::kTileW) *
                           ((cam->height + svdag::kTileH - 1) / svdag::kTileH);
    const unsigned grid = unsigned(std::min<uint64_t>(tiles, 152ull * 32));
    svdag::k_raycast<<<grid, svdag::kRayThreads, 0, st>>>(V, dst, d_bad.get());
    SVDAG_CUDA(cudaPeekAtLastError());
    if (!device_buffer)
      SVDAG_CUDA(cudaMemcpyAsync(hits, dst, sizeof(svdag_ray_hit) * npix, cudaMemcpyDeviceToHost, st));
    uint32_t bad = 0;
    SVDAG_CUDA(cudaMemcpyAsync(&bad, d_bad.get(), 4, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
    return bad ? SVDAG_ERR_INVALID_ARG : SVDAG_OK;
  } catch (const svdag::Error& e) {
    return e.code;
  }
}
