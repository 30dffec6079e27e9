// Stress check of the certified fp32 SAT filter (csrc/sat.cuh, compiled as
// host code) against the oracle's fp64 restatement of the reference test
// (oracle/svdag_oracle.cpp, ora_tri_box).  Prints one summary line:
//   cases=<n> mismatches=<m> fallbacks=<f> hits=<h>
// Built and run by tests/test_sat_filter.py with -ffp-contract=off.
//
//   satcheck <n> [dump_path]
// With dump_path, every (triangle, node) case is also written there as a
// 69-byte record -- triangle float[9], node centre double[3], child half
// side double, the oracle's 8-child overlap mask u8 -- for the device-side
// check of the same filter (tests/test_sat_device.py).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "sat.cuh"
#include "svdag_oracle.h"

using namespace svdag::sat;

static uint64_t g_cases = 0, g_mis = 0, g_hits = 0;
static unsigned g_fb = 0;
static FILE* g_dump = nullptr;

static void check(const float t[9], const double pc[3], double k) {
  NodeBoxes nb;
  node_boxes(pc, k, nb);
  Pair32 P;
  pair_setup(t, t, pc, nb, k, P);
  uint8_t mask = 0;
  for (int ci = 0; ci < 8; ++ci) {
    const double c[3] = {pc[0] + ((ci & 4) ? k : -k), pc[1] + ((ci & 2) ? k : -k), pc[2] + ((ci & 1) ? k : -k)};
    const bool want = ora_tri_box(c, k, t) != 0;
    mask |= uint8_t(want) << ci;
    const bool got = child_overlap(P, ci, &g_fb);
    ++g_cases;
    g_hits += want;
    if (want != got) {
      if (g_mis < 10)
        std::printf("MISMATCH child %d k=%.17g c=(%.17g %.17g %.17g) tri=%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g want=%d\n",
                    ci, k, c[0], c[1], c[2], t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], int(want));
      ++g_mis;
    }
  }
  if (g_dump) {
    std::fwrite(t, 4, 9, g_dump);
    std::fwrite(pc, 8, 3, g_dump);
    std::fwrite(&k, 8, 1, g_dump);
    std::fwrite(&mask, 1, 1, g_dump);
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 200000;
  if (argc > 2) {
    g_dump = std::fopen(argv[2], "wb");
    if (!g_dump) { std::perror(argv[2]); return 2; }
  }
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  for (long it = 0; it < n; ++it) {
    const int level = int(U(rng) * 16);            // parent level 0..15
    const double k = 1.0 / double(1u << (level + 2));
    // parent centre on the level's dyadic grid inside the unit cube
    double pc[3];
    for (int q = 0; q < 3; ++q) {
      const double cells = double(1u << level);
      pc[q] = (std::floor(U(rng) * cells) + 0.5) / cells;
    }
    float t[9];
    const int mode = int(it % 8);
    for (int v = 0; v < 3; ++v) {
      for (int q = 0; q < 3; ++q) {
        double x;
        switch (mode) {
          case 0:  // random near the box
            x = pc[q] + (U(rng) * 6.0 - 3.0) * k;
            break;
          case 1:  // on the child grid lines (face / edge / corner contact)
            x = pc[q] + double(int(U(rng) * 5) - 2) * k;
            break;
          case 2:  // tiny triangle near a child boundary
            x = pc[q] + ((U(rng) < 0.5) ? -k : k) * (U(rng) < 0.5 ? 1.0 : 0.0) + (U(rng) - 0.5) * k * 1e-3;
            break;
          case 3:  // large triangle across the scene
            x = U(rng) * 1.2 - 0.1;
            break;
          case 4:  // dyadic coordinates (exact ties)
            x = pc[q] + std::ldexp(double(int(U(rng) * 65) - 32), -5) * k;
            break;
          case 5:  // vertices within one ulp of grid lines
            x = std::nextafter(pc[q] + double(int(U(rng) * 3) - 1) * k, U(rng) < 0.5 ? 0.0 : 2.0);
            break;
          case 6:  // degenerate: collinear / coincident vertices filled below
            x = pc[q] + (U(rng) * 4.0 - 2.0) * k;
            break;
          default:  // terrain-like small triangles
            x = pc[q] + (U(rng) - 0.5) * 2.5 * k;
            break;
        }
        t[3 * v + q] = float(x);
      }
    }
    if (mode == 6) {
      if (it % 16 == 6) {
        for (int q = 0; q < 3; ++q) t[6 + q] = t[3 + q];  // two equal vertices
      } else {
        for (int q = 0; q < 3; ++q) t[6 + q] = float(0.5 * (double(t[q]) + double(t[3 + q])));  // collinear
      }
    }
    if (mode == 7 && it % 4 == 3) {
      // axis-aligned triangle at an arbitrary (off-grid) coordinate, or on a
      // child face, as box faces are
      const int q = int(U(rng) * 3);
      const float c = (it % 16 == 3) ? float(pc[q] + (U(rng) < 0.5 ? -k : k)) : t[q];
      for (int v = 0; v < 3; ++v) t[3 * v + q] = c;
    }
    if (mode == 4 && it % 32 == 4) {
      // triangle in an axis-aligned plane through the child grid
      const int q = int(U(rng) * 3);
      for (int v = 0; v < 3; ++v) t[3 * v + q] = float(pc[q] + ((it & 64) ? k : 0.0));
    }
    check(t, pc, k);
  }
  // a few non-finite / huge inputs
  {
    const double pc[3] = {0.5, 0.5, 0.5};
    float t[9] = {0.4f, 0.4f, 0.4f, 0.6f, 0.5f, 0.5f, NAN, 0.5f, 0.6f};
    check(t, pc, 0.25);
    float u[9] = {0.4f, 0.4f, 0.4f, 0.6f, 0.5f, 0.5f, 3e30f, 0.5f, 0.6f};
    check(u, pc, 0.25);
  }
  if (g_dump) std::fclose(g_dump);
  std::printf("cases=%llu mismatches=%llu fallbacks=%u hits=%llu\n", (unsigned long long)g_cases,
              (unsigned long long)g_mis, g_fb, (unsigned long long)g_hits);
  return g_mis ? 1 : 0;
}
