// Triangle / box overlap with the reference's exact fp64 decisions
// (src/symvox/test_triangle_box.cpp:38-184), evaluated through a certified
// fp32 filter.
//
// testTriBox rejects a box as soon as one of 13 independent tests fails (9
// edge-axis tests, 3 bounding-box tests, 1 plane test); the answer is the AND
// of the 13 fp64 predicates whatever their order.  Each predicate compares
// fp64 values that the reference computes in a fixed operation order.  Here
// every predicate is first evaluated in fp32 together with a forward error
// bound that covers both the fp32 evaluation and the reference's fp64
// evaluation, relative to the exact real value of the same expression.  When
// the fp32 margin exceeds the bound the fp64 predicate provably has the same
// outcome; otherwise (near-ties, non-finite or huge inputs) that one
// predicate is recomputed in fp64 exactly as the reference does.  The result
// is identical to the reference's for every input.
//
// Error model: fl(a op b) = (a op b)(1 + d), |d| <= u (u32 = 2^-24,
// u64 = 2^-53), plus an absolute slack of 2^-100 against fp32 underflow.
// Bounds (exact-real anchors t - c, t_j - t_i; each follows from the model
// above by adding the relative errors of the operations in order):
//   edge-axis value p = a*u - b*w:  |p_f - p*| <= 4.1 u32 S + 1.02 (|a|+|b|) clo
//                                   S = |a u| + |b w|,   clo = |c - fl32(c)|
//   rad = (|a|+|b|) h:              |rad_f - rad*| <= 3.1 u32 rad
//   fp64 side:                      <= 2^-47 (V^2 + V h)
// where V bounds |t - c| over the pair.  Plane test bounds are in
// plane_decide().
//
// Compiled as host code (tests) with -ffp-contract=off and as device code
// with explicitly rounded intrinsics, so both builds make the same decisions.
#pragma once

#include <stdint.h>

#include <cmath>

#if defined(__CUDACC__)
#define SAT_HD __host__ __device__ __forceinline__
#define SAT_COLD __host__ __device__ __noinline__
#else
#define SAT_HD inline
#define SAT_COLD inline
#endif

// Optional per-predicate fallback hook (profiling builds); no-op by default.
#ifndef SVDAG_FB_HOOK
#define SVDAG_FB_HOOK(which) ((void)0)
#endif

namespace svdag {
namespace sat {

#if defined(__CUDA_ARCH__)
SAT_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
SAT_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
SAT_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
SAT_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
SAT_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
SAT_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
SAT_HD float fabsf_(float a) { return fabsf(a); }
SAT_HD double fabs_(double a) { return fabs(a); }
SAT_HD float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
SAT_HD float fadd(float a, float b) { return a + b; }
SAT_HD float fsub(float a, float b) { return a - b; }
SAT_HD float fmul(float a, float b) { return a * b; }
SAT_HD double dadd(double a, double b) { return a + b; }
SAT_HD double dsub(double a, double b) { return a - b; }
SAT_HD double dmul(double a, double b) { return a * b; }
SAT_HD float fabsf_(float a) { return std::fabs(a); }
SAT_HD double fabs_(double a) { return std::fabs(a); }
SAT_HD float ffma(float a, float b, float c) { return std::fma(a, b, c); }
#endif

// Two independent fp32 operations (one packed instruction on sm_100+; each
// lane is the ordinary IEEE-rounded operation, so host and device agree).
struct F2 {
  float x, y;
};
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
SAT_HD F2 f2add(F2 a, F2 b) { const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y)); return {r.x, r.y}; }
SAT_HD F2 f2mul(F2 a, F2 b) { const float2 r = __fmul2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y)); return {r.x, r.y}; }
#else
SAT_HD F2 f2add(F2 a, F2 b) { return {fadd(a.x, b.x), fadd(a.y, b.y)}; }
SAT_HD F2 f2mul(F2 a, F2 b) { return {fmul(a.x, b.x), fmul(a.y, b.y)}; }
#endif
#if defined(__CUDA_ARCH__)
SAT_HD int __builtin_ctz_(uint32_t m) { return __ffs(int(m)) - 1; }
#else
SAT_HD int __builtin_ctz_(uint32_t m) { return __builtin_ctz(m); }
#endif
SAT_HD float fmin_(float a, float b) { return (b < a) ? b : a; }
SAT_HD float fmax_(float a, float b) { return (a < b) ? b : a; }

constexpr float kU32 = 5.9604644775390625e-08f;  // 2^-24
constexpr float kTiny = 7.8886090522101181e-31f; // 2^-100 absolute slack
constexpr float kD64 = 7.105427357601002e-15f;   // 2^-47 (fp64-side factor)

// Three-valued outcome of one comparison.
enum Tri : int { kFalse = 0, kTrue = 1, kUnknown = 2 };

// ---------------------------------------------------------------------------
// Exact fp64 replicas of the reference's individual tests (used for the
// predicates the filter cannot decide).

// AXISTEST_* reject decision (test_triangle_box.cpp:59-102).  b_first selects
// the Z12 ordering (p2 < p1).
SAT_HD bool axis_reject64(double pa, double pb, double fa, double fb, double h, bool b_first) {
  double mn, mx;
  if (b_first) {
    if (pb < pa) { mn = pb; mx = pa; } else { mn = pa; mx = pb; }
  } else {
    if (pa < pb) { mn = pa; mx = pb; } else { mn = pb; mx = pa; }
  }
  const double rad = dmul(dadd(fa, fb), h);
  return (mn > rad || mx < -rad);
}

// p = a*u - b*w (X and Z macros) and p = -a*u + b*w (Y macros)
SAT_HD double amb64(double a, double u, double b, double w) { return dsub(dmul(a, u), dmul(b, w)); }
SAT_HD double nab64(double a, double u, double b, double w) { return dadd(dmul(-a, u), dmul(b, w)); }

// fp64 vertex offsets and edges of one box, as the reference computes them.
struct Box64 {
  double v[3][3];  // vertex, axis
  double e[3][3];  // edge, axis
};

SAT_HD void box64(const float t[9], const double c[3], Box64& b) {
  for (int i = 0; i < 3; ++i)
    for (int q = 0; q < 3; ++q) b.v[i][q] = dsub(double(t[3 * i + q]), c[q]);
  for (int q = 0; q < 3; ++q) {
    b.e[0][q] = dsub(b.v[1][q], b.v[0][q]);
    b.e[1][q] = dsub(b.v[2][q], b.v[1][q]);
    b.e[2][q] = dsub(b.v[0][q], b.v[2][q]);
  }
}

// Edge-axis test k (0..8) in the reference's order, fp64.  Returns reject.
SAT_HD bool edge_test64(const Box64& b, int k, double h) {
  const int X = 0, Y = 1, Z = 2;
  const int j = k / 3;  // edge
  const double* e = b.e[j];
  const double* v0 = b.v[0];
  const double* v1 = b.v[1];
  const double* v2 = b.v[2];
  const double fx = fabs_(e[X]), fy = fabs_(e[Y]), fz = fabs_(e[Z]);
  switch (k) {
    case 0: return axis_reject64(amb64(e[Z], v0[Y], e[Y], v0[Z]), amb64(e[Z], v2[Y], e[Y], v2[Z]), fz, fy, h, false);
    case 1: return axis_reject64(nab64(e[Z], v0[X], e[X], v0[Z]), nab64(e[Z], v2[X], e[X], v2[Z]), fz, fx, h, false);
    case 2: return axis_reject64(amb64(e[Y], v1[X], e[X], v1[Y]), amb64(e[Y], v2[X], e[X], v2[Y]), fy, fx, h, true);
    case 3: return axis_reject64(amb64(e[Z], v0[Y], e[Y], v0[Z]), amb64(e[Z], v2[Y], e[Y], v2[Z]), fz, fy, h, false);
    case 4: return axis_reject64(nab64(e[Z], v0[X], e[X], v0[Z]), nab64(e[Z], v2[X], e[X], v2[Z]), fz, fx, h, false);
    case 5: return axis_reject64(amb64(e[Y], v0[X], e[X], v0[Y]), amb64(e[Y], v1[X], e[X], v1[Y]), fy, fx, h, false);
    case 6: return axis_reject64(amb64(e[Z], v0[Y], e[Y], v0[Z]), amb64(e[Z], v1[Y], e[Y], v1[Z]), fz, fy, h, false);
    case 7: return axis_reject64(nab64(e[Z], v0[X], e[X], v0[Z]), nab64(e[Z], v1[X], e[X], v1[Z]), fz, fx, h, false);
    default: return axis_reject64(amb64(e[Y], v1[X], e[X], v1[Y]), amb64(e[Y], v2[X], e[X], v2[Y]), fy, fx, h, true);
  }
}

// FINDMINMAX test on one axis (test_triangle_box.cpp:165-174), fp64.
SAT_HD bool aabb_reject64(const Box64& b, int q, double h) {
  double mn = b.v[0][q], mx = b.v[0][q];
  if (b.v[1][q] < mn) mn = b.v[1][q];
  if (b.v[1][q] > mx) mx = b.v[1][q];
  if (b.v[2][q] < mn) mn = b.v[2][q];
  if (b.v[2][q] > mx) mx = b.v[2][q];
  return (mn > h || mx < -h);
}

// planeBoxOverlap(e0 x e1, v0, h) (test_triangle_box.cpp:38-56, 179-180), fp64.
// Returns reject (= !overlap).
SAT_HD bool plane_reject64(const Box64& b, double h) {
  const double* e0 = b.e[0];
  const double* e1 = b.e[1];
  const double n[3] = {dsub(dmul(e0[1], e1[2]), dmul(e0[2], e1[1])), dsub(dmul(e0[2], e1[0]), dmul(e0[0], e1[2])),
                       dsub(dmul(e0[0], e1[1]), dmul(e0[1], e1[0]))};
  double vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    if (n[q] > 0.0) { vmin[q] = dsub(-h, b.v[0][q]); vmax[q] = dsub(h, b.v[0][q]); }
    else            { vmin[q] = dsub(h, b.v[0][q]);  vmax[q] = dsub(-h, b.v[0][q]); }
  }
  const double dmin = dadd(dadd(dmul(n[0], vmin[0]), dmul(n[1], vmin[1])), dmul(n[2], vmin[2]));
  if (dmin > 0.0) return true;
  const double dmax = dadd(dadd(dmul(n[0], vmax[0]), dmul(n[1], vmax[1])), dmul(n[2], vmax[2]));
  return !(dmax >= 0.0);
}

// The whole reference test in fp64 (reference order).  Returns overlap.
SAT_HD bool tri_box64(const float t[9], const double c[3], double h) {
  Box64 b;
  box64(t, c, b);
  for (int k = 0; k < 9; ++k)
    if (edge_test64(b, k, h)) return false;
  for (int q = 0; q < 3; ++q)
    if (aabb_reject64(b, q, h)) return false;
  return !plane_reject64(b, h);
}

// One predicate of child `ci` of a pair in fp64, from scratch (rare path):
// which = 0..2 bounding-box axis, 3..11 edge-axis test which-3, 12 plane,
// -1 the whole test (returns !overlap).  Returns "reject".
SAT_COLD bool pred64(const float* t, const double* pc, double k, int ci, int which) {
  const double c[3] = {dadd(pc[0], (ci & 4) ? k : -k), dadd(pc[1], (ci & 2) ? k : -k),
                       dadd(pc[2], (ci & 1) ? k : -k)};
  float tt[9];
  for (int i = 0; i < 9; ++i) tt[i] = t[i];
  if (which < 0) return !tri_box64(tt, c, k);
  Box64 b;
  box64(tt, c, b);
  if (which < 3) return aabb_reject64(b, which, k);
  if (which < 12) return edge_test64(b, which - 3, k);
  return plane_reject64(b, k);
}

// ---------------------------------------------------------------------------
// Exact-arithmetic tier.  A predicate the error bound leaves undecided is
// re-evaluated in fp32 with error-free transformations: TwoSum gives the
// exact rounding error of an addition, an FMA residual that of a product.
// When every operation of the predicate is exact, the fp32 value is the real
// value of the expression on the exact inputs; the reference's fp64
// evaluation of the same expression then rounds nothing either (every fp32
// value is an fp64 value), so both make the same comparison of the same real
// numbers.  Typical case: triangles lying on octree grid planes (ties).

SAT_HD bool xsub(float a, float b, float& s) {  // s = fl(a - b); exact?
  s = fsub(a, b);
  const float bv = fsub(s, a);
  const float av = fsub(s, bv);
  return fadd(fsub(a, av), fsub(-b, bv)) == 0.f;
}
SAT_HD bool xmul(float a, float b, float& p) {  // p = fl(a * b); exact?
  p = fmul(a, b);
  if (p == 0.f) return a == 0.f || b == 0.f;
  if (fabsf_(p) < 1.0e-30f) return false;  // keep the residual out of the subnormal range
  return ffma(a, b, -p) == 0.f;
}

// which = 0..2 bounding-box axis, 3..11 edge-axis test which-3, 12 plane.
// kTrue = the reference rejects the box, kFalse = it does not, kUnknown = some
// operation was inexact.  c = the child centre, exact in fp32.
SAT_COLD int exact32(const float* tg, float cx, float cy, float cz, float h, int which) {
  float t[9];
  for (int i = 0; i < 9; ++i) t[i] = tg[i];
  const float c[3] = {cx, cy, cz};
  float v[3][3];
  bool ok = true;
  if (which < 3) {  // one axis only
    const int q = which;
    for (int i = 0; i < 3; ++i) ok = xsub(t[3 * i + q], c[q], v[i][q]) && ok;
    if (!ok) return kUnknown;
    float mn = v[0][q], mx = v[0][q];
    for (int i = 1; i < 3; ++i) { mn = (v[i][q] < mn) ? v[i][q] : mn; mx = (v[i][q] > mx) ? v[i][q] : mx; }
    return (mn > h || mx < -h) ? kTrue : kFalse;
  }
  for (int i = 0; i < 3; ++i)
    for (int q = 0; q < 3; ++q) ok = xsub(t[3 * i + q], c[q], v[i][q]) && ok;
  if (!ok) return kUnknown;
  // edges from the vertex offsets, as the reference forms them (e0 = v1 - v0, ...)
  float e[3][3];
  for (int q = 0; q < 3; ++q) {
    ok = xsub(v[1][q], v[0][q], e[0][q]) && ok;
    ok = xsub(v[2][q], v[1][q], e[1][q]) && ok;
    ok = xsub(v[0][q], v[2][q], e[2][q]) && ok;
  }
  if (!ok) return kUnknown;
  if (which < 12) {
    const int k = which - 3, j = k / 3;
    // (a axis, b axis, u axis, w axis, vertex pair, negated) per test, as
    // AXISTEST_X01/X2 (a=e.z b=e.y on y,z), Y02/Y1 (-a*x + b*z, a=e.z b=e.x),
    // Z12/Z0 (a=e.y b=e.x on x,y)
    int aa, bb, ua, wa, i0, i1;
    bool neg = false;
    switch (k) {
      case 0: case 3: aa = 2; bb = 1; ua = 1; wa = 2; i0 = 0; i1 = 2; break;
      case 1: case 4: aa = 2; bb = 0; ua = 0; wa = 2; i0 = 0; i1 = 2; neg = true; break;
      case 2: case 8: aa = 1; bb = 0; ua = 0; wa = 1; i0 = 1; i1 = 2; break;
      case 5: aa = 1; bb = 0; ua = 0; wa = 1; i0 = 0; i1 = 1; break;
      case 6: aa = 2; bb = 1; ua = 1; wa = 2; i0 = 0; i1 = 1; break;
      default: aa = 2; bb = 0; ua = 0; wa = 2; i0 = 0; i1 = 1; neg = true; break;
    }
    const float a = e[j][aa], b = e[j][bb];
    float x0, y0, x1, y1, p0, p1, sab, rad;
    ok = xmul(a, v[i0][ua], x0) && ok;
    ok = xmul(b, v[i0][wa], y0) && ok;
    ok = xmul(a, v[i1][ua], x1) && ok;
    ok = xmul(b, v[i1][wa], y1) && ok;
    ok = xsub(x0, y0, p0) && ok;
    ok = xsub(x1, y1, p1) && ok;
    ok = xsub(fabsf_(a), -fabsf_(b), sab) && ok;
    ok = xmul(sab, h, rad) && ok;
    if (!ok) return kUnknown;
    if (neg) { p0 = -p0; p1 = -p1; }
    return ((p0 > rad && p1 > rad) || (p0 < -rad && p1 < -rad)) ? kTrue : kFalse;
  }
  // plane test: n = e0 x e1, box corners by the sign of n, two dot products
  float m[6], n[3];
  ok = xmul(e[0][1], e[1][2], m[0]) && ok;
  ok = xmul(e[0][2], e[1][1], m[1]) && ok;
  ok = xmul(e[0][2], e[1][0], m[2]) && ok;
  ok = xmul(e[0][0], e[1][2], m[3]) && ok;
  ok = xmul(e[0][0], e[1][1], m[4]) && ok;
  ok = xmul(e[0][1], e[1][0], m[5]) && ok;
  ok = xsub(m[0], m[1], n[0]) && ok;
  ok = xsub(m[2], m[3], n[1]) && ok;
  ok = xsub(m[4], m[5], n[2]) && ok;
  if (!ok) return kUnknown;
  float vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    if (n[q] > 0.f) { ok = xsub(-h, v[0][q], vmin[q]) && ok; ok = xsub(h, v[0][q], vmax[q]) && ok; }
    else            { ok = xsub(h, v[0][q], vmin[q]) && ok; ok = xsub(-h, v[0][q], vmax[q]) && ok; }
  }
  float d[3], s1, dmin, dmax;
  for (int q = 0; q < 3; ++q) ok = xmul(n[q], vmin[q], d[q]) && ok;
  ok = xsub(d[0], -d[1], s1) && ok;
  ok = xsub(s1, -d[2], dmin) && ok;
  if (!ok) return kUnknown;
  if (dmin > 0.f) return kTrue;
  for (int q = 0; q < 3; ++q) ok = xmul(n[q], vmax[q], d[q]) && ok;
  ok = xsub(d[0], -d[1], s1) && ok;
  ok = xsub(s1, -d[2], dmax) && ok;
  if (!ok) return kUnknown;
  return (dmax >= 0.f) ? kFalse : kTrue;
}

// Edge tangency.  Edge-axis test k projects vertices i0, i1 onto
// p = a*u - b*w (Y tests: -a*u + b*w) with a = e_A, b = e_B of edge j and
// u = v_U, w = v_W.  When a is an exact zero (the edge's endpoints share
// coordinate A, so the reference's e_A = v - v = 0) and |w| = h exactly for
// one of the two vertices, the reference computes |p| = fl(|b|*h) = rad for
// that vertex: it lies on the slab boundary and the test cannot reject.  The
// same holds with b and u exchanged, and when a = b = 0 (p = rad = 0).
// Returns true when the rule proves test k passes for box centre c.
SAT_COLD bool edge_tangent(const float* tg, float cx, float cy, float cz, float h, int k) {
  float t[9];
  for (int i = 0; i < 9; ++i) t[i] = tg[i];
  const float c[3] = {cx, cy, cz};
  int aa, bb, ua, wa, i0, i1;
  switch (k) {
    case 0: case 3: aa = 2; bb = 1; ua = 1; wa = 2; i0 = 0; i1 = 2; break;
    case 1: case 4: aa = 2; bb = 0; ua = 0; wa = 2; i0 = 0; i1 = 2; break;
    case 2: case 8: aa = 1; bb = 0; ua = 0; wa = 1; i0 = 1; i1 = 2; break;
    case 5: aa = 1; bb = 0; ua = 0; wa = 1; i0 = 0; i1 = 1; break;
    case 6: aa = 2; bb = 1; ua = 1; wa = 2; i0 = 0; i1 = 1; break;
    default: aa = 2; bb = 0; ua = 0; wa = 2; i0 = 0; i1 = 1; break;
  }
  const int j = k / 3;                       // e0 = v1 - v0, e1 = v2 - v1, e2 = v0 - v2
  const int ea = (j + 1) % 3, eb = j;        // endpoints of edge j
  const bool a0 = t[3 * ea + aa] == t[3 * eb + aa];
  const bool b0 = t[3 * ea + bb] == t[3 * eb + bb];
  if (a0 && b0) return true;
  if (!a0 && !b0) return false;
  const int q = a0 ? wa : ua;                // the component multiplied by the non-zero coefficient
  for (int r = 0; r < 2; ++r) {
    const int i = r ? i1 : i0;
    float vq;
    if (xsub(t[3 * i + q], c[q], vq) && fabsf_(vq) == h) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// fp32 filter.

// Per node: the centres of its 8 child boxes, c_q + (+-k) per axis, as the
// fp32 head of each coordinate and the largest tail.  Computed once per node
// in fp64 (the reference's child-centre values, geom_octree.cpp:222-230).
struct NodeBoxes {
  float chi[6];  // index 2*q + s: fl32(c_q + (s ? k : -k))
  float clo;     // max |(c_q +- k) - chi|, inflated
  float ok;      // 1 when the fp32 path may be used for this node
};

SAT_HD void node_boxes(const double c[3], double k, NodeBoxes& nb) {
  float clo = 0.f;
  bool ok = (k > 1.0e-30) && (k < 1.0e18) && (double(float(k)) == k);
  for (int q = 0; q < 3; ++q) {
    for (int s = 0; s < 2; ++s) {
      const double cd = dadd(c[q], s ? k : -k);
      const float hi = float(cd);
      nb.chi[2 * q + s] = hi;
      const float alo = float(fabs_(dsub(cd, double(hi))));
      clo = (alo > clo) ? alo : clo;
      ok = ok && (fabs_(cd) < 1.0e18);
    }
  }
  nb.clo = clo * 1.0000002f;
  nb.ok = ok ? 1.f : 0.f;
}

// Where the triangle's extent on one axis lies against one child slab
// [c - h, c + h]:
//   out    : the reference's bounding-box test rejects (certain)
//   in     : strictly inside, margin >= 2^-21 h (certain pass, see below)
//   cross  : the bounding-box test passes (certain), not strictly inside
//   unsure : the bounding-box predicate needs fp64
// A triangle strictly inside a box by a margin d passes all 13 fp64 tests of
// the reference when d exceeds their rounding errors (<= 2^-40 h): every
// edge-axis projection lies within rad - d(|a|+|b|), and the plane test gives
// dmin <= -|n|_1 d < 0 <= |n|_1 d <= dmax (both zero when n = 0).
enum Slab : uint32_t { kSlabOut = 0, kSlabIn = 1, kSlabCross = 2, kSlabUnsure = 3 };

// Per (triangle, parent node) data shared by the 8 children.
struct Pair32 {
  float t[9];        // triangle (exact)
  float e[3][3];     // fp32 edges  t1-t0, t2-t1, t0-t2 (edge, axis)
  float ae[3][3];    // |e|
  NodeBoxes nb;
  float h;           // child half side (exact in fp32 when nb.ok)
  bool fast;         // fp32 path usable (finite, moderate magnitudes)
  uint32_t slab;     // 2 bits per (axis q, side s) at bit 2*(2q+s)
  uint32_t tang;     // bit 2q+s: grid-plane tangency on axis q, side s (see pair_slabs)
  uint32_t flat;     // bit q: the three vertices share coordinate q exactly (see pair_slabs)
  float vmax[6];     // max_i |fl32(t_iq - chi)| per (axis, side)
  float n[3], sn[3]; // plane normal e0 x e1 in fp32 and |m1| + |m2| per component
  float nh;          // fl32(|n|_1 h)
  const float* tp;   // the triangle in its source buffer (fp64 predicates reload it)
  const double* c;   // parent centre (fp64), for predicates decided in fp64
  double k;          // child half side (fp64)
};

// Decides x > y from fp32 values with a tolerance; kUnknown inside it.
SAT_HD Tri gt(float x, float y, float tol) {
  const float d = fsub(x, y);
  if (d > tol) return kTrue;
  if (d < -tol) return kFalse;
  return kUnknown;
}

SAT_HD Tri tri_and(Tri a, Tri b) {
  if (a == kFalse || b == kFalse) return kFalse;
  if (a == kTrue && b == kTrue) return kTrue;
  return kUnknown;
}
SAT_HD Tri tri_or(Tri a, Tri b) {
  if (a == kTrue || b == kTrue) return kTrue;
  if (a == kFalse && b == kFalse) return kFalse;
  return kUnknown;
}

// Builds the per-pair data; c = parent centre (fp64, kept by pointer),
// nb = the node's child boxes, k = child half side.
// Plane constants of a pair: n = e0 x e1 (fp32), sn_q = |m1| + |m2| of
// component q, nh = fl32(|n|_1 h).
SAT_HD void pair_plane(Pair32& P, float h) {
  const float* e0 = P.e[0];
  const float* e1 = P.e[1];
  const float m0 = fmul(e0[1], e1[2]), m1 = fmul(e0[2], e1[1]);
  const float m2 = fmul(e0[2], e1[0]), m3 = fmul(e0[0], e1[2]);
  const float m4 = fmul(e0[0], e1[1]), m5 = fmul(e0[1], e1[0]);
  P.n[0] = fsub(m0, m1); P.n[1] = fsub(m2, m3); P.n[2] = fsub(m4, m5);
  P.sn[0] = fadd(fabsf_(m0), fabsf_(m1));
  P.sn[1] = fadd(fabsf_(m2), fabsf_(m3));
  P.sn[2] = fadd(fabsf_(m4), fabsf_(m5));
  P.nh = fmul(fadd(fadd(fabsf_(P.n[0]), fabsf_(P.n[1])), fabsf_(P.n[2])), h);
}

// Edge vectors and plane constants of a pair (only the full test uses them).
SAT_HD void pair_edges(Pair32& P) {
  const float* t = P.t;
  for (int q = 0; q < 3; ++q) {
    P.e[0][q] = fsub(t[3 + q], t[q]);
    P.e[1][q] = fsub(t[6 + q], t[3 + q]);
    P.e[2][q] = fsub(t[q], t[6 + q]);
    for (int j = 0; j < 3; ++j) P.ae[j][q] = fabsf_(P.e[j][q]);
  }
  pair_plane(P, P.h);
}

// Triangle and node data of a pair (no edges, no slab classification).
SAT_HD void pair_core(const float t[9], const float* tp, const double* c, const NodeBoxes& nb, double k,
                      Pair32& P) {
  P.tp = tp;
  bool ok = nb.ok != 0.f;
  for (int i = 0; i < 9; ++i) {
    P.t[i] = t[i];
    ok = ok && (fabsf_(t[i]) < 1.0e18f);  // also false for NaN
  }
  P.nb = nb;
  P.h = float(k);
  P.fast = ok;
  P.c = c;
  P.k = k;
  P.slab = 0;
  P.tang = 0;
  P.flat = 0;
}

// Triangle, node and edge data of a pair (no slab classification).
SAT_HD void pair_basic(const float t[9], const float* tp, const double* c, const NodeBoxes& nb, double k,
                       Pair32& P) {
  P.tp = tp;
  bool ok = nb.ok != 0.f;
  for (int i = 0; i < 9; ++i) {
    P.t[i] = t[i];
    ok = ok && (fabsf_(t[i]) < 1.0e18f);  // also false for NaN
  }
  for (int q = 0; q < 3; ++q) {
    P.e[0][q] = fsub(t[3 + q], t[q]);
    P.e[1][q] = fsub(t[6 + q], t[3 + q]);
    P.e[2][q] = fsub(t[q], t[6 + q]);
    for (int j = 0; j < 3; ++j) P.ae[j][q] = fabsf_(P.e[j][q]);
  }
  pair_plane(P, float(k));
  P.nb = nb;
  P.h = float(k);
  P.fast = ok;
  P.c = c;
  P.k = k;
  P.slab = 0;
  P.tang = 0;
  P.flat = 0;
}

// Slab classification of the pair (see Slab).
// Slab classes of the pair: per axis and side, whether the triangle is
// outside, inside or across the child slab (or undecided).
SAT_HD void pair_slab_classes(Pair32& P) {
  if (!P.fast) return;
  const float* t = P.t;
  const NodeBoxes& nb = P.nb;
  // per axis: vertex extent; fl32(t - chi) is monotone in t, so the extreme
  // offsets are the offsets of the extreme coordinates
  const float h = P.h, clo = nb.clo;
  const float thr_in = fsub(fmul(h, 0.99999904632568359375f), fmul(1.02f, clo));
  uint32_t slab = 0;
  for (int q = 0; q < 3; ++q) {
    float tmn = t[q], tmx = t[q];
    tmn = (t[3 + q] < tmn) ? t[3 + q] : tmn;
    tmx = (t[3 + q] > tmx) ? t[3 + q] : tmx;
    tmn = (t[6 + q] < tmn) ? t[6 + q] : tmn;
    tmx = (t[6 + q] > tmx) ? t[6 + q] : tmx;
    for (int sd = 0; sd < 2; ++sd) {
      const float chi = nb.chi[2 * q + sd];
      const float mn = fsub(tmn, chi), mx = fsub(tmx, chi);
      // FINDMINMAX reject: min v > h or max v < -h.
      Tri r;
      if (clo == 0.f) {
        // c is an fp32 value: v_f = fl32(v*) and v_d = fl64(v*) round the same
        // exact v*, and h is an fp32 value, so v_f > h implies v* > h + ulp32/2,
        // hence v_d > h (likewise for <); only equality stays open
        if (mn > h || mx < -h) r = kTrue;
        else if (mn < h && mx > -h) r = kFalse;
        else r = kUnknown;
      } else {
        // |v_f - v*| <= 1.01 u32 |v_f| + clo, plus a one-ulp fp64 margin
        const float tl = fadd(fadd(fmul(1.1f * kU32, fabsf_(mn)), fmul(1.02f, clo)),
                              fadd(fmul(2.2e-16f, fadd(fabsf_(mn), h)), kTiny));
        const float tu = fadd(fadd(fmul(1.1f * kU32, fabsf_(mx)), fmul(1.02f, clo)),
                              fadd(fmul(2.2e-16f, fadd(fabsf_(mx), h)), kTiny));
        r = tri_or(gt(mn, h, tl), gt(-h, mx, tu));
      }
      const float am = (fabsf_(mn) > fabsf_(mx)) ? fabsf_(mn) : fabsf_(mx);
      P.vmax[2 * q + sd] = am;
      uint32_t cls;
      if (r == kTrue) cls = kSlabOut;
      else if (r == kUnknown) cls = kSlabUnsure;
      else cls = (am <= thr_in) ? kSlabIn : kSlabCross;
      slab |= cls << (2 * (2 * q + sd));
    }
  }
  P.slab = slab;
}

// Grid-plane tangency and axis-aligned triangles (only the full test reads
// them).
SAT_HD void pair_tangency(Pair32& P) {
  if (!P.fast) return;
  const float* t = P.t;
  const NodeBoxes& nb = P.nb;
  const float h = P.h, clo = nb.clo;
  // Grid-plane tangency.  When the three vertices share coordinate q
  // (t_q constant) and the child face lies exactly on that plane
  // (t_q - c_q = +-h exactly, c_q an fp32 value), the reference's fp64
  // predicates that involve axis q all pass: the bounding-box test on q
  // compares +-h with h; every edge of the triangle has e_q = 0 exactly, so an
  // edge-axis test whose projection uses v_q computes p = fl(e'*(+-h)) (the
  // e_q*v term is an exact zero) against rad = fl(|e'|*h), i.e. |p| = rad,
  // which rejects nothing; and the plane test's normal has only its q
  // component non-zero with box corner offsets {0, +-2h} on q, giving
  // dmin <= 0 <= dmax.
  uint32_t tang = 0;
  // Axis-aligned triangle.  When the three vertices share coordinate q, the
  // reference's fp64 offsets v_iq are one value v_q, so both edges have
  // e_q = 0 exactly and the normal's other two components are exact zeros;
  // its dot products reduce to dmin = fl(n_q * vmin_q), dmax = fl(n_q * vmax_q)
  // with vmin_q, vmax_q = fl(-+h - v_q) picked by sign(n_q).  Rounding keeps
  // signs, so the plane test rejects exactly when |v_q| > h (any sign of n_q;
  // n_q = 0 never rejects) -- which the bounding-box test on q rejects too.
  // The plane test therefore never decides the box and is skipped.
  uint32_t flat = 0;
  for (int q = 0; q < 3; ++q)
    if (t[q] == t[3 + q] && t[q] == t[6 + q]) flat |= 1u << q;
  P.flat = flat;
  if (clo == 0.f) {
    for (int q = 0; q < 3; ++q) {
      if (!(t[q] == t[3 + q] && t[q] == t[6 + q])) continue;
      for (int sd = 0; sd < 2; ++sd) {
        float vq;
        if (xsub(t[q], nb.chi[2 * q + sd], vq) && fabsf_(vq) == h) tang |= 1u << (2 * q + sd);
      }
    }
  }
  P.tang = tang;
}

SAT_HD void pair_slabs(Pair32& P) {
  pair_slab_classes(P);
  pair_tangency(P);
}

// child_fast() of all 8 children at once: hit = children whose three slabs
// are inside, full = children the slabs leave undecided (neither inside on
// every axis nor outside on one); the rest do not overlap.
SAT_HD void child_masks(const Pair32& P, uint32_t& hit, uint32_t& full) {
  if (!P.fast) {
    hit = 0;
    full = 0xFFu;
    return;
  }
  // children on side s of axis q: X 0x0F / 0xF0, Y 0x33 / 0xCC, Z 0x55 / 0xAA
  const uint32_t side[6] = {0x0Fu, 0xF0u, 0x33u, 0xCCu, 0x55u, 0xAAu};
  uint32_t in = 0xFFu, out = 0;
  for (int q = 0; q < 3; ++q) {
    uint32_t inq = 0;
    for (int sd = 0; sd < 2; ++sd) {
      const uint32_t c = (P.slab >> (2 * (2 * q + sd))) & 3u;
      if (c == kSlabIn) inq |= side[2 * q + sd];
      if (c == kSlabOut) out |= side[2 * q + sd];
    }
    in &= inq;
  }
  hit = in;
  full = 0xFFu & ~in & ~out;
}

SAT_HD void pair_setup(const float t[9], const float* tp, const double* c, const NodeBoxes& nb, double k,
                       Pair32& P) {
  pair_basic(t, tp, c, nb, k, P);
  pair_slabs(P);
}

// One edge-axis test in fp32: reject (kTrue), keep (kFalse) or kUnknown.
// p_i = a*u_i - b*w_i (negated for the Y tests) for the two vertices of the
// test; cd = the fp64-side and absolute error terms of the box.
// The reference rejects iff min p > rad or max p < -rad.  With tol covering
// |p_f - p*| + |rad_f - rad*| + the fp64 errors, and the roundings of
// rad +- tol (at most u32 (rad + tol), absorbed by the 4.6 / 4.3 factors):
//   min p > rad + tol or max p < -(rad + tol)   -> certain reject
//   min p < rad - tol and max p > -(rad - tol)  -> certain keep
SAT_HD Tri edge_test32(float a, float b, bool neg_a, float u0, float w0, float u1, float w1, float fa, float fb,
                       float h, float clo, float cd) {
  const F2 x = f2mul(F2{a, a}, F2{u0, u1});
  const F2 y = f2mul(F2{b, b}, F2{w0, w1});
  F2 p = f2add(x, F2{-y.x, -y.y});
  if (neg_a) p = F2{-p.x, -p.y};
  const F2 sv = f2add(F2{fabsf_(x.x), fabsf_(x.y)}, F2{fabsf_(y.x), fabsf_(y.y)});
  const float ab = fadd(fa, fb);
  const float rad = fmul(ab, h);
  const float smax = fmax_(sv.x, sv.y);
  const float tol = ffma(4.6f * kU32, smax, ffma(4.3f * kU32, rad, ffma(1.04f * clo, ab, cd)));
  const float mn = fmin_(p.x, p.y), mx = fmax_(p.x, p.y);
  const float hi = fadd(rad, tol), lo = fsub(rad, tol);
  if (mn > hi || mx < -hi) return kTrue;
  if (mn < lo && mx > -lo) return kFalse;
  return kUnknown;
}

// Edge-axis test with box-level thresholds: 1 reject, 0 keep, 2 unknown.
// ab = fl(|a| + |b|), hW = fl(h + Wp), hmW = fl(h - Wp).  With
// Wp >= 4.7 u32 V + 4.4 u32 h + 1.05 clo the thresholds
//   hi = fl(ab hW + cd) >= rad* + (|a|+|b|)(4.1 u32 V + 1.02 clo) + fp64 errors,
//   lo = fl(ab hmW - cd) <= rad* - (the same)
// hold after every rounding (|a*|+|b*| <= ab (1 + 2.02 u32)), so
//   min p > hi or max p < -hi -> certain reject,
//   min p < lo and max p > -lo -> certain keep.
SAT_HD int edge_test_box(float a, float b, bool neg_a, float u0, float w0, float u1, float w1, float ab, float hW,
                         float hmW, float cd) {
  const F2 x = f2mul(F2{a, a}, F2{u0, u1});
  const F2 y = f2mul(F2{b, b}, F2{w0, w1});
  F2 p = f2add(x, F2{-y.x, -y.y});
  if (neg_a) p = F2{-p.x, -p.y};
  const float mn = fmin_(p.x, p.y), mx = fmax_(p.x, p.y);
  const float hi = ffma(ab, hW, cd), lo = ffma(ab, hmW, -cd);
  if (mn > hi || mx < -hi) return 1;
  if (mn < lo && mx > -lo) return 0;
  return 2;
}

// Decision from the slab classes alone: 0 no overlap, 1 overlap, 2 the
// full test is needed.
SAT_HD int child_fast(const Pair32& P, int ci) {
  if (!P.fast) return 2;
  const uint32_t cx = (P.slab >> (2 * (0 + ((ci >> 2) & 1)))) & 3u;
  const uint32_t cy = (P.slab >> (2 * (2 + ((ci >> 1) & 1)))) & 3u;
  const uint32_t cz = (P.slab >> (2 * (4 + (ci & 1)))) & 3u;
  if (cx == kSlabOut || cy == kSlabOut || cz == kSlabOut) return 0;
  if (cx == kSlabIn && cy == kSlabIn && cz == kSlabIn) return 1;
  return 2;
}

// Edge and plane data of a pair, read from the Pair32 itself; the kernel
// passes a source that reads them from shared memory where they are used.
struct PairSrc {
  const Pair32& P;
  SAT_HD float t(int i) const { return P.t[i]; }
  SAT_HD float chi(int i) const { return P.nb.chi[i]; }
  SAT_HD float clo() const { return P.nb.clo; }
  SAT_HD float vmax(int i) const { return P.vmax[i]; }
  SAT_HD float e(int j, int q) const { return P.e[j][q]; }
  SAT_HD float n(int q) const { return P.n[q]; }
  SAT_HD float sn(int q) const { return P.sn[q]; }
  SAT_HD float nh() const { return P.nh; }
};

// The full test of child `ci` for a child child_fast() left undecided (the
// edges and plane constants from S, everything else from P).
template <class Src>
SAT_HD bool child_full_src(const Pair32& P, const Src& S, int ci, unsigned* fallbacks) {
  const bool sx = (ci >> 2) & 1, sy = (ci >> 1) & 1, sz = ci & 1;
  if (!P.fast) {
    if (fallbacks) ++*fallbacks;
    SVDAG_FB_HOOK(-1);
    return !pred64(P.tp, P.c, P.k, ci, -1);
  }
  const uint32_t cx = (P.slab >> (2 * (0 + sx))) & 3u;
  const uint32_t cy = (P.slab >> (2 * (2 + sy))) & 3u;
  const uint32_t cz = (P.slab >> (2 * (4 + sz))) & 3u;
  const float h = P.h;
  const float clo = S.clo();
  // fp32 vertex offsets v = t - fl32(c); |v_f - (t - c)| <= 1.01 u32 |v_f| + 1.01 clo
  float v[3][3];
  const float chi[3] = {S.chi(sx ? 1 : 0), S.chi(sy ? 3 : 2), S.chi(sz ? 5 : 4)};
  for (int i = 0; i < 3; ++i)
    for (int q = 0; q < 3; ++q) v[i][q] = fsub(S.t(3 * i + q), chi[q]);
  // V >= |t - c| and >= |v_f| over this box
  float V = S.vmax(sx ? 1 : 0);
  V = fmax_(V, S.vmax(sy ? 3 : 2));
  V = fmax_(V, S.vmax(sz ? 5 : 4));
  V = ffma(V, 1.0000003f, 1.01f * clo);
  // fp64-side and absolute error terms: 2^-47 (V^2 + V h) + 2^-100
  const float cd = ffma(kD64, fmul(V, fadd(V, h)), kTiny);

  // undecided predicate: tangency rule, then the exact fp32 tier when the box
  // centre is an fp32 value, else (or when inexact) the reference's fp64
  // evaluation
  auto need64 = [&](int which) {
    if (clo == 0.f && which >= 3 && which < 12 && edge_tangent(P.tp, chi[0], chi[1], chi[2], h, which - 3)) return false;
    if (clo == 0.f) {
      const int r = exact32(P.tp, chi[0], chi[1], chi[2], h, which);
      if (r != kUnknown) return r == kTrue;
    }
    if (fallbacks) ++*fallbacks;
    SVDAG_FB_HOOK(which);
    return pred64(P.tp, P.c, P.k, ci, which);
  };

  // grid-plane tangency (pair_slabs): the predicates on a tangent axis pass
  const bool tx = (P.tang >> (0 + sx)) & 1u, ty = (P.tang >> (2 + sy)) & 1u, tz = (P.tang >> (4 + sz)) & 1u;
  const bool passX = ty || tz, passY = tx || tz, passZ = tx || ty;  // X-, Y-, Z-axis edge tests

  // bounding-box tests (FINDMINMAX): decided per slab in pair_setup
  if (cx == kSlabUnsure && !tx && need64(0)) return false;
  if (cy == kSlabUnsure && !ty && need64(1)) return false;
  if (cz == kSlabUnsure && !tz && need64(2)) return false;

  // nine edge-axis tests (test_triangle_box.cpp:137-156).  Per box:
  //   |p_f - p*| + |rad_f - rad*| <= (|a| + |b|)(4.1 u32 V + 3.1 u32 h + 1.02 clo)
  // so the thresholds are ab (h +- Wp) +- cd with Wp covering that and the
  // roundings of the thresholds themselves (see edge_test_box).
  const float Wp = ffma(4.7f * kU32, V, ffma(4.4f * kU32, h, 1.05f * clo));
  const float hW = fadd(h, Wp), hmW = fsub(h, Wp);
  const int X = 0, Y = 1, Z = 2;
  uint32_t rej = 0, unk = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    if ((k == 0 || k == 3 || k == 6) && passX) continue;
    if ((k == 1 || k == 4 || k == 7) && passY) continue;
    if ((k == 2 || k == 5 || k == 8) && passZ) continue;
    const int j = k / 3;
    const float e[3] = {S.e(j, 0), S.e(j, 1), S.e(j, 2)};
    int r;
    switch (k) {
      case 0: case 3:  // X01: a=e.z, b=e.y over v0, v2 on (y, z)
        r = edge_test_box(e[Z], e[Y], false, v[0][Y], v[0][Z], v[2][Y], v[2][Z], fadd(fabsf_(e[Z]), fabsf_(e[Y])), hW, hmW, cd); break;
      case 1: case 4:  // Y02: -a*v.x + b*v.z, a=e.z, b=e.x over v0, v2
        r = edge_test_box(e[Z], e[X], true, v[0][X], v[0][Z], v[2][X], v[2][Z], fadd(fabsf_(e[Z]), fabsf_(e[X])), hW, hmW, cd); break;
      case 2: case 8:  // Z12: a=e.y, b=e.x over v1, v2 on (x, y)
        r = edge_test_box(e[Y], e[X], false, v[1][X], v[1][Y], v[2][X], v[2][Y], fadd(fabsf_(e[Y]), fabsf_(e[X])), hW, hmW, cd); break;
      case 5:          // Z0: over v0, v1
        r = edge_test_box(e[Y], e[X], false, v[0][X], v[0][Y], v[1][X], v[1][Y], fadd(fabsf_(e[Y]), fabsf_(e[X])), hW, hmW, cd); break;
      case 6:          // X2: over v0, v1
        r = edge_test_box(e[Z], e[Y], false, v[0][Y], v[0][Z], v[1][Y], v[1][Z], fadd(fabsf_(e[Z]), fabsf_(e[Y])), hW, hmW, cd); break;
      default:         // 7, Y1: over v0, v1
        r = edge_test_box(e[Z], e[X], true, v[0][X], v[0][Z], v[1][X], v[1][Z], fadd(fabsf_(e[Z]), fabsf_(e[X])), hW, hmW, cd); break;
    }
    rej |= uint32_t(r == 1) << k;
    unk |= uint32_t(r == 2) << k;
  }
  if (rej) return false;  // one certain reject decides the AND of the 13 tests
  for (uint32_t m = unk; m; m &= m - 1)
    if (need64(3 + (__builtin_ctz_(m)))) return false;

  if (tx || ty || tz) return true;  // the plane test passes on a tangent grid plane
  if (P.flat) return true;          // axis-aligned triangle: implied by the bounding-box test (pair_slabs)

  // plane test with the pair's normal n = e0 x e1 (pair constants n, sn, nh):
  //   dmin* = -(|n|_1 h + n.v0),  dmax* = |n|_1 h - n.v0
  // once every component's sign is certain (the reference picks each box
  // corner by sign(n_q)).
  //   |n_f - n*| <= 4.1 u32 sn_q;  |nh_f - nh*| <= 7.2 u32 h sum sn
  //   |d_f - d*| <= 8.2 u32 h sum sn + 9.2 u32 sum sn_q |v0_q| + clo sum sn
  //   fp64 side <= 2^-42 V^2 (V + h)
  const float tn0 = ffma(kD64, fmul(V, V), kTiny);
  const float n[3] = {S.n(0), S.n(1), S.n(2)}, sn[3] = {S.sn(0), S.sn(1), S.sn(2)};
  bool sure = true;
  for (int q = 0; q < 3; ++q) sure = sure && (fabsf_(n[q]) > ffma(4.2f * kU32, sn[q], tn0));
  if (sure) {
    const float nh = S.nh();
    const float nd = fadd(fadd(fmul(n[0], v[0][0]), fmul(n[1], v[0][1])), fmul(n[2], v[0][2]));
    const float dmin = -fadd(nh, nd);
    const float dmax = fsub(nh, nd);
    const float snsum = fadd(fadd(sn[0], sn[1]), sn[2]);
    const float snv = ffma(sn[0], fabsf_(v[0][0]), ffma(sn[1], fabsf_(v[0][1]), fmul(sn[2], fabsf_(v[0][2]))));
    const float td = ffma(8.7f * kU32 * h, snsum,
                          ffma(9.7f * kU32, snv, ffma(1.06f * clo, snsum,
                                                     ffma(32.f * kD64, fmul(fmul(V, V), fadd(V, h)), kTiny))));
    if (dmin > td) return false;                 // reference: dmin > 0 -> reject
    if (dmin < -td) {
      if (dmax > td) return true;                // dmax >= 0 -> overlap
      if (dmax < -td) return false;
    }
  }
  return !need64(12);
}

SAT_HD bool child_full(const Pair32& P, int ci, unsigned* fallbacks) {
  return child_full_src(P, PairSrc{P}, ci, fallbacks);
}

// Overlap decision for child `ci` (index 4x+2y+z) of the pair: true when the
// child box overlaps the triangle exactly as the reference decides it;
// `fallbacks` counts the predicates that needed fp64.
SAT_HD bool child_overlap(const Pair32& P, int ci, unsigned* fallbacks) {
  const int f = child_fast(P, ci);
  if (f != 2) return f == 1;
  return child_full(P, ci, fallbacks);
}

}  // namespace sat
}  // namespace svdag
