// Internal state of one SVDAG build context and the phase entry points the
// C ABI (api.cu) dispatches to.
#pragma once

#include <string>
#include <vector>

#include "common.cuh"

namespace svdag {

// One octree level in HBM, structure-of-arrays.
//   hdr[n]      : mask | mirX<<8 | mirY<<16 | mirZ<<24
//   ch[8n]      : child ids (kNull when absent); empty on the leaf level
//   inv[n]      : invariant mask (SDAG only; empty otherwise)
//   clev[8n]    : child levels (CSVDAG only; empty otherwise)
//   ctr[3n]     : fp64 node centre (SVO build only)
//   nbox[8n]    : fp32 child-box centres of the node (SVO build only)
struct Level {
  uint64_t n = 0;
  DBuf<uint32_t> hdr;
  DBuf<uint32_t> ch;
  DBuf<uint8_t> inv;
  DBuf<uint8_t> clev;
  DBuf<double> ctr;
  DBuf<float> nbox;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Exec ex;
  uint64_t launches = 0;

  const float* tris = nullptr;
  uint64_t n_tris = 0;
  DBuf<float> owned_tris;

  uint32_t levels = 0;
  int state = SVDAG_S_EMPTY;
  bool child_levels_init = false;  // initChildLevels called (clev = lev+1 implicitly)
  std::vector<Level> lev;
  float bbox[6] = {0, 0, 0, 0, 0, 0};
  double root_side = 0.0;

  svdag_stats st{};
  std::string last_error;

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Profiler prof;
};

// Phases (each throws svdag::Error on failure).
// tri_list (optional, device, ascending ids): voxelize only these triangles
void phase_voxelize(Ctx& c, uint32_t levels, const double bbox[6], const uint32_t* tri_list = nullptr,
                    uint64_t n_list = 0);
// GeomOctree::buildDAG: chunked build joined and reduced to a DAG
void phase_build_dag(Ctx& c, uint32_t levels, uint32_t step_level, const double bbox[6]);
void phase_reduce_dag(Ctx& c);
void phase_reduce_sdag(Ctx& c);
void phase_cross_level_merge(Ctx& c);
// toDAG with every temporary in caller-provided device scratch (no allocation).
void phase_reduce_dag_scratch(Ctx& c, uint8_t* scratch, uint64_t capacity);

}  // namespace svdag

struct svdag_ctx {
  svdag::Ctx c;
};
