// Seeded synthetic scenes for the SVDAG build: displaced icosphere, fBm
// heightfield terrain with skirts, axis-aligned boxes, and writers for the
// ASCII OBJ format the reference svbuilder reads (src/symvox/scene.cpp:51-300).
//
// Every generator is bit-reproducible across x86-64 and aarch64 hosts: only
// IEEE basic operations (+ - * / sqrt floor) are used, the file is compiled
// with -ffp-contract=off, and sine comes from a fixed Horner polynomial
// instead of libm.  Triangles are emitted as float[9] (v0 v1 v2, xyz each).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "svdag_host.h"

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

const double kPi = 3.14159265358979311599796346854;
const double kTwoPi = 6.28318530717958623199592693709;

// sin(x) by reduction to [-pi, pi] and an odd Taylor polynomial of degree 25
// evaluated in Horner form; deterministic on every IEEE-754 host.
double det_sin(double x) {
  static const double inv_fact_odd[] = {
      1.0,                                 // 1/1!
      -1.0 / 6.0,                          // -1/3!
      1.0 / 120.0,                         // 1/5!
      -1.0 / 5040.0,                       // -1/7!
      1.0 / 362880.0,                      // 1/9!
      -1.0 / 39916800.0,                   // -1/11!
      1.0 / 6227020800.0,                  // 1/13!
      -1.0 / 1307674368000.0,              // -1/15!
      1.0 / 355687428096000.0,             // 1/17!
      -1.0 / 121645100408832000.0,         // -1/19!
      1.0 / 51090942171709440000.0,        // 1/21!
      -1.0 / 25852016738884976640000.0,    // -1/23!
      1.0 / 15511210043330985984000000.0}; // 1/25!
  double k = std::floor(x / kTwoPi + 0.5);
  double r = x - k * kTwoPi;
  double r2 = r * r;
  double q = inv_fact_odd[12];
  for (int i = 11; i >= 0; --i) q = q * r2 + inv_fact_odd[i];
  return q * r;
}

inline uint32_t hash_u32(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  uint64_t h = (uint64_t(a) * 0x9E3779B97F4A7C15ull) ^ (uint64_t(b) * 0xC2B2AE3D27D4EB4Full) ^
               (uint64_t(c) * 0x165667B19E3779F9ull) ^ (uint64_t(d) * 0xD6E8FEB86659FD93ull);
  h ^= h >> 33;
  h *= 0xFF51AFD7ED558CCDull;
  h ^= h >> 33;
  h *= 0xC4CEB9FE1A85EC53ull;
  h ^= h >> 33;
  return uint32_t(h);
}

// lattice value in [0, 1) from 24 hash bits
inline double lattice(int64_t ix, int64_t iy, uint32_t octave, uint32_t seed) {
  return double(hash_u32(uint32_t(ix), uint32_t(iy), octave, seed) >> 8) * (1.0 / 16777216.0);
}

inline double smooth(double t) { return t * t * (3.0 - 2.0 * t); }

// 2-D value noise with smoothstep-weighted bilinear interpolation.
double value_noise2(double x, double y, uint32_t octave, uint32_t seed) {
  double fx = std::floor(x), fy = std::floor(y);
  int64_t ix = int64_t(fx), iy = int64_t(fy);
  double tx = smooth(x - fx), ty = smooth(y - fy);
  double v00 = lattice(ix, iy, octave, seed), v10 = lattice(ix + 1, iy, octave, seed);
  double v01 = lattice(ix, iy + 1, octave, seed), v11 = lattice(ix + 1, iy + 1, octave, seed);
  double a = v00 + (v10 - v00) * tx;
  double b = v01 + (v11 - v01) * tx;
  return a + (b - a) * ty;
}

inline void put_tri(float* t, const float a[3], const float b[3], const float c[3]) {
  std::memcpy(t, a, 12);
  std::memcpy(t + 3, b, 12);
  std::memcpy(t + 6, c, 12);
}

}  // namespace

extern "C" {

uint64_t svdag_synth_icosphere_count(uint32_t subdiv) {
  uint64_t n = 20;
  for (uint32_t i = 0; i < subdiv; ++i) n *= 4;
  return n;
}

// Icosphere of the given subdivision level, centred at (0.5,0.5,0.5), radius
// `radius`, each vertex displaced along its normal by
//   amp * sum_o w_o * sin(f_o * pi * dot(u, k_o) + phi_o),  f_o = 2,4,8,16,
// with seeded unit directions k_o, phases phi_o in [0, 2pi) and weights
// w_o = 2^-o normalised to sum 1.
int svdag_synth_icosphere(uint32_t subdiv, double radius, double amp, uint64_t seed, float* out) {
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<double> vx, vy, vz;
  auto add = [&](double x, double y, double z) {
    double n = std::sqrt(x * x + y * y + z * z);
    vx.push_back(x / n); vy.push_back(y / n); vz.push_back(z / n);
    return uint32_t(vx.size() - 1);
  };
  add(-1, phi, 0); add(1, phi, 0); add(-1, -phi, 0); add(1, -phi, 0);
  add(0, -1, phi); add(0, 1, phi); add(0, -1, -phi); add(0, 1, -phi);
  add(phi, 0, -1); add(phi, 0, 1); add(-phi, 0, -1); add(-phi, 0, 1);
  std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                             11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                             3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
  for (uint32_t s = 0; s < subdiv; ++s) {
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
    auto midpoint = [&](uint32_t a, uint32_t b) {
      std::pair<uint32_t, uint32_t> k = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
      auto it = mid.find(k);
      if (it != mid.end()) return it->second;
      uint32_t m = add((vx[a] + vx[b]) * 0.5, (vy[a] + vy[b]) * 0.5, (vz[a] + vz[b]) * 0.5);
      mid[k] = m;
      return m;
    };
    std::vector<uint32_t> g;
    g.reserve(f.size() * 4);
    for (size_t t = 0; t < f.size(); t += 3) {
      uint32_t a = f[t], b = f[t + 1], c = f[t + 2];
      uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      uint32_t q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      g.insert(g.end(), q, q + 12);
    }
    f.swap(g);
  }
  SplitMix64 rng(seed);
  double kx[4], ky[4], kz[4], ph[4], w[4];
  const double freq[4] = {2.0, 4.0, 8.0, 16.0};
  double wsum = 0.0;
  for (int o = 0; o < 4; ++o) {
    double x, y, z, n;
    do {
      x = 2.0 * rng.uniform() - 1.0;
      y = 2.0 * rng.uniform() - 1.0;
      z = 2.0 * rng.uniform() - 1.0;
      n = x * x + y * y + z * z;
    } while (n < 1e-6 || n > 1.0);
    n = std::sqrt(n);
    kx[o] = x / n; ky[o] = y / n; kz[o] = z / n;
    ph[o] = kTwoPi * rng.uniform();
    w[o] = 1.0 / double(1 << o);
    wsum += w[o];
  }
  std::vector<float> px(vx.size()), py(vx.size()), pz(vx.size());
  for (size_t i = 0; i < vx.size(); ++i) {
    double d = 0.0;
    for (int o = 0; o < 4; ++o) {
      double dp = vx[i] * kx[o] + vy[i] * ky[o] + vz[i] * kz[o];
      d += (w[o] / wsum) * det_sin(freq[o] * kPi * dp + ph[o]);
    }
    double r = radius + amp * d;
    px[i] = float(0.5 + r * vx[i]);
    py[i] = float(0.5 + r * vy[i]);
    pz[i] = float(0.5 + r * vz[i]);
  }
  for (size_t t = 0; t < f.size(); ++t) {
    out[3 * t + 0] = px[f[t]];
    out[3 * t + 1] = py[f[t]];
    out[3 * t + 2] = pz[f[t]];
  }
  return 0;
}

uint64_t svdag_synth_terrain_count(uint32_t grid) {
  uint64_t g = grid - 1;
  return 2 * g * g + 8 * g + 2;
}

// Heightfield over x,z in [0,1] on a grid x grid vertex lattice; heights from
// `octaves` octaves of value noise (base frequency 4 cells, lacunarity 2,
// gain 0.5) rescaled to [0, height].  Closed into a watertight solid by
// vertical skirts down to y = 0 on the four borders and two bottom triangles.
// Triangle order: the two triangles of each cell row-major, then skirts
// (x=0, x=1, z=0, z=1 borders), then the bottom.
int svdag_synth_terrain(uint32_t grid, uint32_t octaves, double height, uint64_t seed, float* out) {
  if (grid < 2) return -1;
  const uint32_t n = grid;
  std::vector<double> h(uint64_t(n) * n);
  const uint32_t s32 = uint32_t(seed ^ (seed >> 32));
  double hmin = 1e300, hmax = -1e300;
  for (uint32_t j = 0; j < n; ++j) {
    for (uint32_t i = 0; i < n; ++i) {
      double u = double(i) / double(n - 1), v = double(j) / double(n - 1);
      double sum = 0.0, amp = 1.0, fr = 4.0;
      for (uint32_t o = 0; o < octaves; ++o) {
        sum += amp * value_noise2(u * fr, v * fr, o, s32);
        amp *= 0.5;
        fr *= 2.0;
      }
      h[uint64_t(j) * n + i] = sum;
      if (sum < hmin) hmin = sum;
      if (sum > hmax) hmax = sum;
    }
  }
  const double span = (hmax > hmin) ? (hmax - hmin) : 1.0;
  std::vector<float> hy(h.size()), gx(n);
  for (size_t k = 0; k < h.size(); ++k) hy[k] = float(height * ((h[k] - hmin) / span));
  for (uint32_t i = 0; i < n; ++i) gx[i] = float(double(i) / double(n - 1));
  auto P = [&](uint32_t i, uint32_t j, float* p) { p[0] = gx[i]; p[1] = hy[uint64_t(j) * n + i]; p[2] = gx[j]; };
  float* t = out;
  float a[3], b[3], c[3], d[3];
  for (uint32_t j = 0; j + 1 < n; ++j) {
    for (uint32_t i = 0; i + 1 < n; ++i) {
      P(i, j, a); P(i + 1, j, b); P(i + 1, j + 1, c); P(i, j + 1, d);
      put_tri(t, a, b, c); t += 9;
      put_tri(t, a, c, d); t += 9;
    }
  }
  // skirts: border vertex pairs (top, bottom at y=0)
  auto skirt = [&](uint32_t i0, uint32_t j0, uint32_t i1, uint32_t j1) {
    float p0[3], p1[3], q0[3], q1[3];
    P(i0, j0, p0); P(i1, j1, p1);
    std::memcpy(q0, p0, 12); q0[1] = 0.0f;
    std::memcpy(q1, p1, 12); q1[1] = 0.0f;
    put_tri(t, p0, q0, q1); t += 9;
    put_tri(t, p0, q1, p1); t += 9;
  };
  for (uint32_t k = 0; k + 1 < n; ++k) skirt(0, k, 0, k + 1);
  for (uint32_t k = 0; k + 1 < n; ++k) skirt(n - 1, k, n - 1, k + 1);
  for (uint32_t k = 0; k + 1 < n; ++k) skirt(k, 0, k + 1, 0);
  for (uint32_t k = 0; k + 1 < n; ++k) skirt(k, n - 1, k + 1, n - 1);
  const float b00[3] = {0.f, 0.f, 0.f}, b10[3] = {1.f, 0.f, 0.f}, b11[3] = {1.f, 0.f, 1.f}, b01[3] = {0.f, 0.f, 1.f};
  put_tri(t, b00, b11, b10); t += 9;
  put_tri(t, b00, b01, b11); t += 9;
  return (uint64_t(t - out) == 9 * svdag_synth_terrain_count(grid)) ? 0 : -2;
}

// Axis-aligned boxes as 12 triangles each.  Box k spans
// [lo[3k..3k+2], hi[3k..3k+2]] in scene units.
int svdag_synth_boxes(const float* lo, const float* hi, uint64_t n_boxes, float* out) {
  for (uint64_t k = 0; k < n_boxes; ++k) {
    const float* l = lo + 3 * k;
    const float* h = hi + 3 * k;
    float v[8][3];
    for (int c = 0; c < 8; ++c) {
      v[c][0] = (c & 4) ? h[0] : l[0];
      v[c][1] = (c & 2) ? h[1] : l[1];
      v[c][2] = (c & 1) ? h[2] : l[2];
    }
    static const int q[6][4] = {{0, 1, 3, 2}, {4, 6, 7, 5}, {0, 4, 5, 1}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 5, 7, 3}};
    float* t = out + k * 12 * 9;
    for (int f = 0; f < 6; ++f) {
      put_tri(t, v[q[f][0]], v[q[f][1]], v[q[f][2]]); t += 9;
      put_tri(t, v[q[f][0]], v[q[f][2]], v[q[f][3]]); t += 9;
    }
  }
  return 0;
}

// Writes triangles as an ASCII OBJ the reference loader accepts: optional
// unreferenced pin vertices (0,0,0) and (1,1,1) first (they fix the scene
// bounding box to the unit cube, scene.cpp:131 merges every `v` line), then
// three `v` lines and one `f` line per triangle.  %.9g round-trips floats.
int svdag_write_obj(const char* path, const float* tris, uint64_t n_tris, int pin_unit_cube) {
  FILE* fp = std::fopen(path, "w");
  if (!fp) return -1;
  std::vector<char> buf(1 << 22);
  std::setvbuf(fp, buf.data(), _IOFBF, buf.size());
  uint64_t base = 1;
  if (pin_unit_cube) {
    std::fprintf(fp, "v 0 0 0\nv 1 1 1\n");
    base = 3;
  }
  for (uint64_t t = 0; t < n_tris; ++t) {
    const float* p = tris + 9 * t;
    for (int k = 0; k < 3; ++k)
      std::fprintf(fp, "v %.9g %.9g %.9g\n", double(p[3 * k]), double(p[3 * k + 1]), double(p[3 * k + 2]));
  }
  for (uint64_t t = 0; t < n_tris; ++t) {
    uint64_t v = base + 3 * t;
    std::fprintf(fp, "f %llu %llu %llu\n", (unsigned long long)v, (unsigned long long)(v + 1),
                 (unsigned long long)(v + 2));
  }
  std::fclose(fp);
  return 0;
}

}  // extern "C"
