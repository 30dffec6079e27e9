// Test infrastructure only (the oracle): a CPU restatement of the viewer's
// ray traversal of an encoded SSVDAG, the GLSL fragment shader
// shaders/octree_dda.frag.glsl (SSVDAG variant, DEPTH_MODE main :848-859,
// trace_ray :539-581) with the uniforms OctreeDDARenderer sets
// (src/svviewer/octree_dda_renderer.cpp:199-223, 391-422).  The tests compare
// the GPU ray caster with it; the product never links it.
//
// GLSL fixes no evaluation order or rounding, so this file fixes one: IEEE
// single precision, no contraction (build with -ffp-contract=off), each
// expression evaluated left to right as written in the shader; mat4 * vec4
// as ((M0 x + M1 y) + M2 z) + M3 w over the columns; dot as (xx' + yy') + zz';
// normalize(v) = v / sqrt(dot(v, v)); min(x, y) = y < x ? y : x and
// max(x, y) = x < y ? y : x (the GLSL definitions); float -> int truncates.
// One departure from the shader: transform_ray (:480-507) keeps an exactly
// zero direction component at zero (sign(0) * 1e-4) and divides by it; here
// it becomes +1e-4.  Out-of-range reads (a corrupt file) end the ray with
// t = -5 and make the call return -2.
#include <cmath>
#include <cstdint>

#include "svdag_oracle.h"

namespace {

struct Hit {
  float t;
  int32_t level, iterations, node;
  int32_t voxel[3];
  uint32_t normal;
};
static_assert(sizeof(Hit) == 32, "hit record layout");

float fmin_g(float x, float y) { return y < x ? y : x; }
float fmax_g(float x, float y) { return x < y ? y : x; }
float sign_g(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
int to_int(float x) {
  if (x != x) return 0;
  if (x >= 2147483648.f) return 2147483647;
  if (x <= -2147483648.f) return -2147483647 - 1;
  return int(x);
}

struct Scene {
  const uint16_t* inner;
  const uint8_t* leaves;
  const uint32_t* level_off;
  uint64_t n_inner, n_leaves;
  uint32_t n_level_off, inner_levels;
};

void mat4_vec4(const float* M, const float v[4], float r[4]) {
  for (int i = 0; i < 4; ++i) {
    float a = M[i] * v[0];
    a = a + M[4 + i] * v[1];
    a = a + M[8 + i] * v[2];
    a = a + M[12 + i] * v[3];
    r[i] = a;
  }
}

void normalize(float v[3]) {
  float dd = v[0] * v[0];
  dd = dd + v[1] * v[1];
  dd = dd + v[2] * v[2];
  const float l = std::sqrt(dd);
  for (int k = 0; k < 3; ++k) v[k] = v[k] / l;
}

// traversal_status (:103-118)
struct Status {
  float t_current;
  int node_index;
  uint32_t hdr;
  int mirror_mask[3];
  uint32_t leaf_data[2];
  int idx[3], local_idx[3];
  uint32_t child_linear_index;
  float t_next[3], inv_d[3];
  int delta_idx[3];
  int node_size;
  float cell_size;
  uint32_t level;
};

uint32_t child_mask(uint32_t hdr, uint32_t c) { return (hdr >> (c << 1)) & 3u; }

// voxel_to_linear_idx (:149-152); out-of-node indices give an empty cell
uint32_t voxel_to_linear(const Status& s) {
  int v[3];
  for (int k = 0; k < 3; ++k) {
    if (s.local_idx[k] < 0 || s.local_idx[k] >= s.node_size) return 0xFFFFFFFFu;
    v[k] = (1 - 2 * s.mirror_mask[k]) * s.local_idx[k] + s.mirror_mask[k] * (s.node_size - 1);
  }
  return uint32_t(v[2] + s.node_size * (v[1] + s.node_size * v[0]));
}

// fetch_data (:305-310)
bool fetch_data(const Scene& S, Status& s) {
  if (s.level < S.inner_levels) {
    if (s.level >= S.n_level_off) return false;
    const uint64_t at = uint64_t(S.level_off[s.level]) + uint32_t(s.node_index);
    if (at >= S.n_inner) return false;
    s.hdr = S.inner[at];
    return true;
  }
  const uint64_t b = uint64_t(uint32_t(s.node_index)) * 8;
  if (b + 8 > S.n_leaves) return false;
  for (int w = 0; w < 2; ++w)
    s.leaf_data[w] = uint32_t(S.leaves[b + 4 * w]) | (uint32_t(S.leaves[b + 4 * w + 1]) << 8) |
                     (uint32_t(S.leaves[b + 4 * w + 2]) << 16) | (uint32_t(S.leaves[b + 4 * w + 3]) << 24);
  return true;
}

// fetch_voxel_bit / leaf_fetch_voxel_bit (:290-303)
bool fetch_voxel_bit(const Scene& S, const Status& s) {
  const uint32_t c = s.child_linear_index;
  if (s.level < S.inner_levels) return c < 8 && child_mask(s.hdr, c) != 0;
  if (c >= 64) return false;
  const uint32_t word = (c & 32) == 0 ? s.leaf_data[0] : s.leaf_data[1];
  return (word & (1u << (c & 31))) != 0;
}

// fetch_child_index_in (:312-347), high half of a two-word pointer first
bool fetch_child_index(const Scene& S, Status& s) {
  const uint32_t c = s.child_linear_index;
  if (s.level >= S.n_level_off || c >= 8) return false;
  uint64_t node_offset = 1 + uint64_t(S.level_off[s.level]) + uint32_t(s.node_index);
  for (uint32_t i = 7; i > c; --i) {
    const uint32_t m = child_mask(s.hdr, i);
    node_offset += m < 2 ? m : 2;
  }
  const uint32_t mask = child_mask(s.hdr, c);
  if (node_offset + (mask > 1 ? 2 : 1) > S.n_inner) return false;
  int cx = S.inner[node_offset];
  const int mirror[3] = {(cx >> 13) & 1, (cx >> 14) & 1, (cx >> 15) & 1};
  cx &= -57345;  // ~(7 << 13)
  if (mask > 1) {
    cx = (cx << 16) | int(S.inner[node_offset + 1]);
    cx |= int(mask & 1) << 29;
  }
  for (int k = 0; k < 3; ++k) s.mirror_mask[k] ^= mirror[k];
  s.node_index = cx;
  return true;
}

void next_crossings(const float o[3], Status& s) {
  for (int k = 0; k < 3; ++k) {
    const int nxt = s.idx[k] + (s.delta_idx[k] > 0 ? s.delta_idx[k] : 0);
    const float plane = float(nxt) * s.cell_size;
    s.t_next[k] = (plane - o[k]) * s.inv_d[k];
  }
}

// go_down_one_level (:434-451)
void go_down_one_level(const float o[3], const float d[3], Status& s) {
  ++s.level;
  s.cell_size = s.cell_size * 0.5f;
  for (int k = 0; k < 3; ++k) {
    const float p_a = o[k] + s.t_current * d[k];
    const float p_center = float(s.idx[k] * 2 + 1) * s.cell_size;
    s.idx[k] = s.idx[k] * 2 + (p_center < p_a ? 1 : 0);
  }
  next_crossings(o, s);
  for (int k = 0; k < 3; ++k) s.local_idx[k] = s.idx[k] & (s.node_size - 1);
}

// dda_next_delta_index (:411-416): the crossing axis as a 0/1 mask
void crossing_mask(const Status& s, int m[3]) {
  const float* t = s.t_next;
  m[0] = (t[0] < t[1]) & (t[0] <= t[2]);
  m[1] = (t[1] < t[2]) & (t[1] <= t[0]);
  m[2] = (t[2] < t[0]) & (t[2] <= t[1]);
}

Hit trace(const Scene& S, const float bbox[6], float root_half, const float view_inv[16], const float proj_inv[16],
          uint32_t width, uint32_t height, uint32_t px, uint32_t py, uint32_t max_iters, uint32_t draw_level,
          float proj_factor, float t_min, float t_max, bool& broken) {
  Hit h{};
  h.node = -1;
  broken = false;
  // main (:848-851): gl_FragCoord at the pixel centre
  const float sx = ((float(px) + 0.5f) / float(width)) * 2.f - 1.f;
  const float sy = ((float(py) + 0.5f) / float(height)) * 2.f - 1.f;
  // computeCameraRay (:587-604)
  float o[3], d[3];
  {
    const float s0[4] = {sx, sy, 0.f, 1.f}, s1[4] = {sx, sy, 1.f, 1.f};
    float a[4], b[4];
    mat4_vec4(proj_inv, s0, a);
    mat4_vec4(proj_inv, s1, b);
    float dir[3];
    for (int k = 0; k < 3; ++k) dir[k] = b[k] / b[3] - a[k] / a[3];
    normalize(dir);
    const float zero[4] = {0.f, 0.f, 0.f, 1.f}, e[4] = {dir[0], dir[1], dir[2], 1.f};
    float op[4], ep[4];
    mat4_vec4(view_inv, zero, op);
    mat4_vec4(view_inv, e, ep);
    for (int k = 0; k < 3; ++k) {
      o[k] = op[k];
      d[k] = ep[k] - op[k];
    }
    normalize(d);
  }
  // transform_ray (:480-507) with intersectAABB (:357-365)
  float center[3];
  for (int k = 0; k < 3; ++k) center[k] = (bbox[k] + bbox[3 + k]) * 0.5f;
  const float epsilon = 1e-4f;
  const float scale = 1.f / (2.f * root_half);
  float octree_min[3];
  for (int k = 0; k < 3; ++k) {
    octree_min[k] = center[k] - root_half;
    o[k] = (o[k] - octree_min[k]) * scale;
  }
  t_min = t_min * scale;
  t_max = t_max * scale;
  for (int k = 0; k < 3; ++k) {
    const float sg = sign_g(d[k]);
    if (sg == 0.f) d[k] = epsilon;
    else if (d[k] * sg < epsilon) d[k] = sg * epsilon;
  }
  float tlo[3], thi[3];
  for (int k = 0; k < 3; ++k) {
    const float clip_lo = (bbox[k] - octree_min[k]) * scale;
    const float clip_hi = (bbox[3 + k] - octree_min[k]) * scale;
    const float t1 = (clip_lo - o[k]) / d[k];
    const float t2 = (clip_hi - o[k]) / d[k];
    tlo[k] = fmin_g(t1, t2);
    thi[k] = fmax_g(t1, t2);
  }
  const float enter = fmax_g(fmax_g(tlo[0], 0.f), fmax_g(tlo[1], tlo[2]));
  const float leave = fmin_g(thi[0], fmin_g(thi[1], thi[2]));
  t_min = fmax_g(enter, t_min + 1e-10f);
  t_max = fmin_g(leave, t_max);
  if (!(enter < leave)) {
    h.t = -4.f;
    return h;
  }
  const float world = 2.f * root_half;
  // init (:509-527) with dda_init (:373-388)
  Status s{};
  s.t_current = t_min;
  for (int k = 0; k < 3; ++k) {
    s.inv_d[k] = 1.f / d[k];
    s.delta_idx[k] = int(sign_g(d[k]));
  }
  s.level = 0;
  s.cell_size = 0.5f;
  {
    const float voxel_eps = 1.f / (256.f * 1024.f);
    const float tt = s.t_current + voxel_eps;
    for (int k = 0; k < 3; ++k) {
      const float p_a = o[k] + tt * d[k];
      s.idx[k] = to_int(p_a / s.cell_size);
    }
    next_crossings(o, s);
    for (int k = 0; k < 3; ++k) s.local_idx[k] = s.idx[k] % 2;
  }
  s.node_size = 2;
  s.node_index = 0;
  if (!fetch_data(S, s)) { broken = true; }
  s.child_linear_index = voxel_to_linear(s);
  // the traversal stack (:124-147): node, header, mirror | level << 3
  int st_node[64];
  uint32_t st_hdr[64];
  int st_mask[64];
  uint32_t st_n = 0;
  int step_dir[3] = {0, 0, 0};
  uint32_t it = 0;
  const uint32_t max_level = S.inner_levels < draw_level - 1u ? S.inner_levels : draw_level - 1u;
  while (!broken) {
    if (!fetch_voxel_bit(S, s)) {
      // dda_next (:396-409)
      int m[3];
      crossing_mask(s, m);
      for (int k = 0; k < 3; ++k) {
        step_dir[k] = m[k] * s.delta_idx[k];
        s.idx[k] += step_dir[k];
        s.local_idx[k] += step_dir[k];
      }
      float tc = float(m[0]) * s.t_next[0];
      tc = tc + float(m[1]) * s.t_next[1];
      tc = tc + float(m[2]) * s.t_next[2];
      s.t_current = tc;
      for (int k = 0; k < 3; ++k) s.t_next[k] = s.t_next[k] + (float(m[k]) * s.cell_size) * std::fabs(s.inv_d[k]);
      bool in_node = true;
      for (int k = 0; k < 3; ++k) in_node = in_node && s.local_idx[k] >= 0 && s.local_idx[k] < s.node_size;
      if (!in_node) {
        if (st_n == 0) {
          h.t = -1.f;
          h.iterations = int32_t(it);
          return h;
        }
        // up_in (:418-432)
        uint32_t delta_level = s.level;
        --st_n;
        s.node_index = st_node[st_n];
        s.hdr = st_hdr[st_n];
        const int mk = st_mask[st_n];
        s.mirror_mask[0] = mk & 1;
        s.mirror_mask[1] = (mk >> 1) & 1;
        s.mirror_mask[2] = (mk >> 2) & 1;
        s.level = uint32_t(mk >> 3) & 255u;
        delta_level -= s.level;
        for (int k = 0; k < 3; ++k) s.idx[k] >>= delta_level;
        s.cell_size = s.cell_size * float(1 << delta_level);
        s.node_size = s.level < S.inner_levels ? 2 : 4;
        for (int k = 0; k < 3; ++k) s.local_idx[k] = s.idx[k] & 1;
        next_crossings(o, s);
      }
    } else {
      // resolution_ok (:367-369)
      const bool hit = s.level >= max_level || (s.cell_size * proj_factor) < s.t_current;
      if (hit) {
        h.t = s.t_current * world;
        h.level = int32_t(s.level);
        h.iterations = int32_t(it);
        h.node = s.node_index;
        for (int k = 0; k < 3; ++k) h.voxel[k] = s.idx[k];
        for (int k = 0; k < 3; ++k) h.normal |= uint32_t(uint8_t(int8_t(-step_dir[k]))) << (8 * k);
        return h;
      }
      // down_in (:453-477)
      int m[3];
      crossing_mask(s, m);
      bool stays = true;
      for (int k = 0; k < 3; ++k) {
        const int nl = s.local_idx[k] + m[k] * s.delta_idx[k];
        stays = stays && nl >= 0 && nl < 2;
      }
      if (stays) {
        if (st_n >= 64) { broken = true; break; }
        st_node[st_n] = s.node_index;
        st_hdr[st_n] = s.hdr;
        st_mask[st_n] = s.mirror_mask[0] | (s.mirror_mask[1] << 1) | (s.mirror_mask[2] << 2) | int(s.level << 3);
        ++st_n;
      }
      if (!fetch_child_index(S, s)) { broken = true; break; }
      go_down_one_level(o, d, s);
      if (s.level == S.inner_levels) {
        s.node_size = 4;  // LEAF_SIZE
        go_down_one_level(o, d, s);
      }
      if (!fetch_data(S, s)) { broken = true; break; }
    }
    s.child_linear_index = voxel_to_linear(s);
    ++it;
    if (!(s.t_current < t_max && it < max_iters)) break;
  }
  if (broken) {
    Hit b{};
    b.t = -5.f;
    b.node = -1;
    return b;
  }
  h.t = it >= max_iters ? -3.f : -2.f;
  h.iterations = int32_t(it);
  return h;
}

}  // namespace

extern "C" int ora_ssvdag_raycast(const uint16_t* inner, uint64_t n_inner, const uint8_t* leaves, uint64_t n_leaves,
                                  const uint32_t* level_off, uint32_t n_level_off, uint32_t levels,
                                  const float bbox[6], float root_side, const float view_inv[16],
                                  const float proj_inv[16], uint32_t width, uint32_t height, uint32_t max_iters,
                                  uint32_t draw_level, float projection_factor, float t_min, float t_max,
                                  void* hits) {
  if (levels < 3 || levels > 30) return -1;
  const Scene S{inner, leaves, level_off, n_inner, n_leaves, n_level_off, levels - 2};
  Hit* out = static_cast<Hit*>(hits);
  int status = 0;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t q = 0; q < int64_t(width) * height; ++q) {
    bool broken = false;
    out[q] = trace(S, bbox, root_side * 0.5f, view_inv, proj_inv, width, height, uint32_t(q % width),
                   uint32_t(q / width), max_iters, draw_level, projection_factor, t_min, t_max, broken);
    if (broken) {
#pragma omp atomic write
      status = -2;
    }
  }
  return status;
}
