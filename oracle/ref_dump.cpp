// ref_dump: runs the REFERENCE SymVox build path (compiled from the
// reference's own src/symvox sources against oracle/sl_shim) on one OBJ and
// dumps every intermediate node pool.  Test infrastructure: it produces the
// golden vectors the restated oracle and the CUDA path are checked against.
//
//   ref_dump <scene.obj> <levels> <out_prefix> [step_levels]
//
// Writes <out_prefix>.{svo,dag,sdag,csv}.pool, the four encoded files
// <out_prefix>.{svdag,esvdag,ussvdag,ssvdag,csv.svdag} and a one-line JSON
// summary on stdout (prefixed "REFJSON ").  With step_levels > 0 the SVO is
// built by the reference's OpenMP chunked GeomOctree::buildDAG
// (geom_octree.cpp:289-435) instead of buildSVO + toDAG, and only the DAG
// and downstream pools are written.
//
// Pool file layout (little endian):
//   "SVDP" u32 version=1 u32 levels u32 state u64 nvoxels u64 nnodes
//   per level: u64 count, then count 48-byte records
//     u32 hdr = mask | mirX<<8 | mirY<<16 | mirZ<<24
//     u32 children[8]          (0xFFFFFFFE = null, as octree.cpp:22)
//     u8  childLevels[8]       (low byte of the reference's unsigned value)
//     u8  invariantBitmask, u8 pad[3]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <symvox/encoded_ssvdag.hpp>
#include <symvox/encoded_svdag.hpp>
#include <symvox/encoded_ussvdag.hpp>
#include <symvox/geom_octree.hpp>
#include <symvox/scene.hpp>

static void dump_pool(const GeomOctree& oct, const std::string& path) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { std::perror(path.c_str()); std::exit(2); }
  const GeomOctree::NodeData& d = oct.getNodeData();
  uint32_t ver = 1, levels = (uint32_t)d.size(), state = (uint32_t)oct.getState();
  uint64_t nvox = oct.getNVoxels(), nnodes = oct.getNNodes();
  std::fwrite("SVDP", 1, 4, fp);
  std::fwrite(&ver, 4, 1, fp);
  std::fwrite(&levels, 4, 1, fp);
  std::fwrite(&state, 4, 1, fp);
  std::fwrite(&nvox, 8, 1, fp);
  std::fwrite(&nnodes, 8, 1, fp);
  for (uint32_t l = 0; l < levels; ++l) {
    uint64_t n = d[l].size();
    std::fwrite(&n, 8, 1, fp);
    std::vector<unsigned char> rec(48 * n);
    for (uint64_t i = 0; i < n; ++i) {
      const GeomOctree::Node& nd = d[l][i];
      unsigned char* r = &rec[48 * i];
      uint32_t hdr = uint32_t(nd.childrenBitmask) | (uint32_t(nd.childrenMirroredBitmask[0]) << 8) |
                     (uint32_t(nd.childrenMirroredBitmask[1]) << 16) |
                     (uint32_t(nd.childrenMirroredBitmask[2]) << 24);
      std::memcpy(r, &hdr, 4);
      std::memcpy(r + 4, nd.children, 32);
      for (int c = 0; c < 8; ++c) r[36 + c] = (unsigned char)(nd.childLevels[c] & 0xFF);
      r[44] = nd.invariantBitmask;
      r[45] = r[46] = r[47] = 0;
    }
    if (n) std::fwrite(rec.data(), 1, rec.size(), fp);
  }
  std::fclose(fp);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: ref_dump scene.obj levels out_prefix [step_levels]\n");
    return 1;
  }
  std::string obj = argv[1];
  unsigned levels = (unsigned)std::atoi(argv[2]);
  std::string pre = argv[3];
  int step = argc > 4 ? std::atoi(argv[4]) : 0;

  Scene scene;
  scene.loadObj(obj, false, false, false, false, true);
  auto minF = scene.getAABB()[0], maxF = scene.getAABB()[1];
  sl::aabox3d bb(sl::point3d(minF[0], minF[1], minF[2]), sl::point3d(maxF[0], maxF[1], maxF[2]));

  GeomOctree oct(&scene);
  sl::real_time_clock ck;
  ck.restart();
  if (step == 0) {
    oct.buildSVO(levels, bb, false, NULL, false);
    dump_pool(oct, pre + ".svo.pool");
    oct.toDAG();
  } else {
    oct.buildDAG(levels, (unsigned)step, bb, false);
  }
  double t_dag = ck.elapsed().as_seconds();
  GeomOctree::Stats st_svo = oct.getStats();
  oct.initChildLevels();
  dump_pool(oct, pre + ".dag.pool");

  EncodedSVDAG svdag;
  svdag.encode(oct);
  svdag.save(pre + ".svdag");
  EncodedSSVDAG esvdag;
  esvdag.encode(oct);
  esvdag.save(pre + ".esvdag");

  GeomOctree sd(oct);
  ck.restart();
  sd.toSDAG(false, false);
  double t_sdag = ck.elapsed().as_seconds();
  dump_pool(sd, pre + ".sdag.pool");
  EncodedUSSVDAG ussvdag;
  ussvdag.encode(sd);
  ussvdag.save(pre + ".ussvdag");
  EncodedSSVDAG ssvdag;
  ssvdag.encode(sd);
  ssvdag.save(pre + ".ssvdag");

  GeomOctree cs(oct);
  ck.restart();
  unsigned merged = cs.mergeAcrossAllLevels();
  double t_csv = ck.elapsed().as_seconds();
  dump_pool(cs, pre + ".csv.pool");
  EncodedSVDAG csvdag;
  csvdag.encode(cs);
  csvdag.save(pre + ".csv.svdag");

  std::printf(
      "REFJSON {\"levels\": %u, \"nTotalVoxels\": %zu, \"nNodesSVO\": %zu, \"nNodesLastLevSVO\": %zu, "
      "\"nNodesDAG\": %zu, \"nNodesSDAG\": %zu, \"nNodesCSVDAG\": %zu, \"nCrossLevelMerged\": %u, "
      "\"t_build_dag_s\": %.6f, \"t_sdag_s\": %.6f, \"t_csv_s\": %.6f}\n",
      levels, st_svo.nTotalVoxels, st_svo.nNodesSVO, st_svo.nNodesLastLevSVO, oct.getStats().nNodesDAG,
      sd.getStats().nNodesSDAG, cs.getNNodes(), merged, t_dag, t_sdag, t_csv);
  return 0;
}
