// svbuilder: the reference CLI (src/svbuilder/main.cpp) on the GPU build path.
//
//   svbuilder input.{obj,svdag} numLevels numBuildSteps [-l [infl diff refs]] [-c] [-h]
//             [output.{svdag,ussvdag,ssvdag,esvdag}]
//
// Same argument contract, output names (<dir>/<base>_<levels>[infix].ext),
// result printout and stats.txt append as the reference.  numBuildSteps = 0
// builds the SVO and reduces it (buildSVO + toDAG); numBuildSteps > 0 runs the
// chunked buildDAG with that step level (src/svbuilder/main.cpp:158-175), so
// the node order is the reference's in both cases.  -l runs the lossy LSVDAG
// of this build (the reference's clustering is the external MCL program; see
// GeomOctree::toLossyDag) and writes the reference's lossy outputs
// (<base>_<levels>.esvdag of the DAG, then the lossy DAG's files with the
// -l_<infl>_<diff>_<refs> infix).  -h (hidden-geometry DAG, work in progress
// in the reference) is reported as unavailable.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "octree_host.hpp"
#include "scene.hpp"

using namespace svdag;

namespace {

void usage() {
  std::printf(
      "\nUsage:\n"
      "      svbuilder input_model.obj numLevels numBuildSteps [--lossy or -l] [--cross-level-merging or -c] "
      "[<output.[svo | svdag | ussvdag | ssvdag]>\n"
      "Where:\n"
      "      input_model.obj: a 3D model in ASCII OBJ format OR a pre-built SVDAG file\n"
      "      numLevels: levels of the octree to build (i.e. 10->1K^3, 13->8K^3...)\n"
      "      numBuildSteps: 0 = build the whole SVO, then reduce it; n > 0 = chunked build with step level n\n\n");
}

std::string dir_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}
std::string base_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  std::string b = k == std::string::npos ? p : p.substr(k + 1);
  size_t d = b.find_last_of('.');
  return d == std::string::npos ? b : b.substr(0, d);
}
std::string human(double v, const char* unit) {
  char b[64];
  const char* pre[] = {"", "K", "M", "G", "T"};
  int i = 0;
  while (v >= 1000.0 && i < 4) { v /= 1000.0; ++i; }
  std::snprintf(b, sizeof(b), "%.2f%s%s", v, pre[i], unit);
  return b;
}

}  // namespace

int main(int argc, char** argv) {
  std::printf(
      "\n===============================================================================\n"
      "==========   svbuilder (GB300 build path)                              =========\n"
      "===============================================================================\n");
  if (argc < 4) {
    usage();
    return 1;
  }
  const std::string input(argv[1]);
  const int nLevels = std::atoi(argv[2]);
  const int levelStep = std::atoi(argv[3]);
  std::printf(" MODEL: '%s'   [ %d levels, step %i ]   (%.0fK^3)\n", input.c_str(), nLevels, levelStep,
              std::pow(2.0, nLevels) / 1024.0);

  bool lossy = false, multiLevel = false, hidden = false;
  float infl = 2.0f, diff = 1.0f;
  int refs = 1;
  for (int i = 4; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--lossy" || a == "-l") {
      // clamps of src/svbuilder/main.cpp:121-131
      if (i + 1 < argc) infl = std::fmin(10.0f, std::fmax(1.1f, std::strtof(argv[i + 1], nullptr)));
      if (i + 2 < argc) diff = std::fmin(32.0f, std::fmax(0.01f, std::strtof(argv[i + 2], nullptr)));
      if (i + 3 < argc) refs = std::min(1000000, std::max(1, std::atoi(argv[i + 3])));
      lossy = true;
    } else if (a == "--cross-level-merging" || a == "-c") {
      multiLevel = true;
    }
    if (a == "--hidden-geometry" || a == "-h") hidden = true;
  }
  std::printf("Lossy: %d, Cross-level: %d, Hidden geom: %d\n", lossy, multiLevel, hidden);
  if (hidden) {
    // the flood fill is GeomOctree::hiddenGeometryFloodfill, but the
    // reference's hidden-geometry DAG reduction does not terminate once a
    // correspondence stays unresolved (geom_octree_extension.cpp:2059-2070)
    std::printf("--hidden-geometry is not available in this build\n");
    return 2;
  }

  Scene scene;
  GeomOctree octree(&scene);
  const bool isObj = input.find(".obj") != std::string::npos || input.find(".OBJ") != std::string::npos;
  const bool isDag = input.find(".svdag") != std::string::npos;
  if (isObj) {
    if (!scene.loadObj(input, true, true)) {
      std::printf("ERROR: Scene:loadOBJ: Can't open file %s\n", input.c_str());
      return 1;
    }
    const float* b = scene.bbox();
    const double bb[6] = {b[0], b[1], b[2], b[3], b[4], b[5]};
    if (levelStep == 0) {
      octree.buildSVO(unsigned(nLevels), bb);
      octree.toDAG();
    } else {
      octree.buildDAG(unsigned(nLevels), unsigned(levelStep), bb);
    }
    // bounding boxes outside [0.1, 1e5] are rescaled for rendering (main.cpp:178-193)
    const double dx = double(b[3]) - b[0], dy = double(b[4]) - b[1], dz = double(b[5]) - b[2];
    const float size = float(std::sqrt(dx * dx + dy * dy + dz * dz));
    if (size > 100000.f || size < 0.1f) {
      const float n = float(std::sqrt(dx * dx + dy * dy + dz * dz));
      const float nb[6] = {0, 0, 0, float(100000.0 * dx / n), float(100000.0 * dy / n), float(100000.0 * dz / n)};
      scene.setBBox(nb);
      octree.resizeSceneBbox(nb);
    }
  } else if (isDag) {
    EncodedSVDAG in;
    if (!in.load(input)) {
      std::printf("Can't read input file '%s'.\n", input.c_str());
      return 1;
    }
    octree.importDAG(in.decode(), in.bbox, in.rootSide, 0);
  } else {
    std::printf("Can't read input file '%s'. Only supported ASCII Obj files.\n", input.c_str());
    return 1;
  }

  octree.initChildLevels();
  const std::string basePath = dir_of(input) + "/" + base_of(input) + "_" + std::to_string(nLevels);

  // every encoding is built on the GPU; the SSVDAG's reference-count order
  // is the reference's std::sort, run on the host over counts from the GPU
  EncodedSVDAG svdag2;
  svdag2.encode(octree);
  svdag2.save(basePath + ".svdag");

  // the lossy run's names carry its parameters (main.cpp:213-217)
  auto trimmed = [](float v) {
    const std::string t = std::to_string(v);
    return t.substr(0, t.find('.') + 2);
  };
  const std::string paramStr = "-l_" + trimmed(infl) + "_" + trimmed(diff) + "_" + std::to_string(refs);
  uint64_t lossyMerged = 0;
  if (lossy) {
    // the DAG's own ESVDAG first (main.cpp:226-230), then the lossy DAG; the
    // clustering is the project's lossy LSVDAG (see GeomOctree::toLossyDag)
    EncodedSSVDAG esvdag2;
    esvdag2.encode(octree);
    esvdag2.save(basePath + ".esvdag");
    lossyMerged = octree.toLossyDag(infl, diff, refs);
    octree.initChildLevels();
  } else if (multiLevel) {
    octree.mergeAcrossAllLevels();
  }

  EncodedSVDAG svdag;
  svdag.encode(octree);
  EncodedSSVDAG esvdag;
  if (!multiLevel) esvdag.encode(octree);
  if (!multiLevel) octree.toSDAG();
  EncodedUSSVDAG ussvdag;
  EncodedSSVDAG ssvdag;
  if (!multiLevel) {
    ussvdag.encode(octree);
    ssvdag.encode(octree);
  }
  const std::string infix = lossy ? paramStr : (multiLevel ? "-multi" : "");
  svdag.save(basePath + infix + ".svdag");
  if (!multiLevel) {
    ussvdag.save(basePath + infix + ".ussvdag");
    ssvdag.save(basePath + infix + ".ssvdag");
    esvdag.save(basePath + infix + ".esvdag");
  }
  for (int i = 4; i < argc; ++i) {
    const std::string out = argv[i];
    if (out.find(".svo") != std::string::npos || out.find(".SVO") != std::string::npos) continue;
    if (out.find(".svdag") != std::string::npos || out.find(".SVDAG") != std::string::npos) svdag.save(out);
    else if (out.find(".ussvdag") != std::string::npos || out.find(".USSVDAG") != std::string::npos) ussvdag.save(out);
    else if (out.find(".ssvdag") != std::string::npos || out.find(".SSVDAG") != std::string::npos) ssvdag.save(out);
    else if (out.find(".esvdag") != std::string::npos || out.find(".ESVDAG") != std::string::npos) esvdag.save(out);
  }

  const Stats st = octree.getStats();
  const double nv = double(st.nTotalVoxels ? st.nTotalVoxels : 1);
  std::printf("\n========= RESULTS '%s' [%d levels] (%.0fK^3) =========\n", input.c_str(), nLevels,
              std::pow(2.0, nLevels) / 1024.0);
  std::printf("Voxels:     %s\t(%llu)\n", human(double(st.nTotalVoxels), "").c_str(), (unsigned long long)st.nTotalVoxels);
  std::printf("SVO Nodes:  %s\t(%llu)\n", human(double(st.nNodesSVO), "").c_str(), (unsigned long long)st.nNodesSVO);
  std::printf("DAG Nodes:  %s\t(%llu)\n", human(double(st.nNodesDAG), "").c_str(), (unsigned long long)st.nNodesDAG);
  std::printf("SDAG Nodes: %s\t(%llu)\n", human(double(st.nNodesSDAG), "").c_str(), (unsigned long long)st.nNodesSDAG);
  std::printf("Encoded SVDAG      : %s\t(%.3f bits/vox)\n", human(double(svdag.getDataSize()), "B").c_str(),
              8.0 * svdag.getDataSize() / nv);
  std::printf("Encoded ESVDAG     : %s\t(%.3f bits/vox)\n", human(double(esvdag.getDataSize()), "B").c_str(),
              8.0 * esvdag.getDataSize() / nv);
  std::printf("Encoded USSVDAG    : %s\t(%.3f bits/vox)\n", human(double(ussvdag.getDataSize()), "B").c_str(),
              8.0 * ussvdag.getDataSize() / nv);
  std::printf("Encoded SSVDAG     : %s\t(%.3f bits/vox)\n", human(double(ssvdag.getDataSize()), "B").c_str(),
              8.0 * ssvdag.getDataSize() / nv);
  std::printf("SVO build time     : %.3f ms (GPU)\n", st.buildSVOTime);
  std::printf("SVO->SVDAG time    : %.3f ms (GPU)\n", st.toDAGTime);
  std::printf("SVDAG->SSVDAG time : %.3f ms (GPU)\n", st.toSDAGTime);
  if (multiLevel) std::printf("Cross-level merge  : %.3f ms (GPU), %llu nodes eliminated\n", st.crossMergeTime,
                              (unsigned long long)st.nCrossLevelMerged);
  if (lossy) std::printf("Lossy LSVDAG       : %llu nodes merged (GPU)\n", (unsigned long long)lossyMerged);
  std::printf("===================================================================\n\n");

  // stats.txt append in the reference's shape (main.cpp:320-366)
  FILE* fs = std::fopen("stats.txt", "a");
  if (fs) {
    std::fprintf(fs, "%s, %d, lossy: %d, cross-level: %d\n", base_of(input).c_str(), nLevels, lossy, multiLevel);
    std::fprintf(fs, "#Voxels, %llu\n", (unsigned long long)st.nTotalVoxels);
    std::fprintf(fs, ", SVDAG, ESVDAG, SSVDAG, SVO\n");
    std::fprintf(fs, "#nodes, %llu, '', %llu, %llu\n", (unsigned long long)st.nNodesDAG,
                 (unsigned long long)st.nNodesSDAG, (unsigned long long)st.nNodesSVO);
    std::fprintf(fs, "memory (bytes), %zu, %zu, %zu, %llu\n", svdag.getDataSize(), esvdag.getDataSize(),
                 ssvdag.getDataSize(), (unsigned long long)st.nNodesSVO);
    if (lossy) {
      // the reference's hashing / similar-node / clustering times and
      // cluster statistics belong to its MCL clustering; the lossy merge
      // count stands in the cluster column
      std::fprintf(fs, "Construction times:\n,SVDAG, LSVDAG, Total, Hashing, SimNodes, Clustering\n");
      std::fprintf(fs, "time (ms), %.0f, 0, %.0f, 0, 0, 0\n", st.toDAGTime, st.buildSVOTime + st.toDAGTime + st.toSDAGTime);
      std::fprintf(fs, "Lossy stats, %.2f, %.2f, %i\n", infl, diff, refs);
      std::fprintf(fs, "TotalVoxDifference, #NodesIn, #ClustersOut, #edges, svdag mem, lsvdag mem\n");
      std::fprintf(fs, "0, 0, %llu, 0, %zu, %zu\n", (unsigned long long)lossyMerged, svdag2.getDataSize(),
                   svdag.getDataSize());
    } else if (multiLevel) {
      std::fprintf(fs, "Construction times:\n,SVDAG, Total, Cross-level\n");
      std::fprintf(fs, "time (ms), %.0f, %.0f, %.0f\n", st.toDAGTime, st.buildSVOTime + st.toDAGTime + st.crossMergeTime,
                   st.crossMergeTime);
      std::fprintf(fs, "Cross-level, nodes eliminated, svdag mem, csvdag mem\n");
      std::fprintf(fs, ", %llu, %zu, %zu\n", (unsigned long long)st.nCrossLevelMerged, svdag2.getDataSize(),
                   svdag.getDataSize());
    } else {
      std::fprintf(fs, "Construction times:\n,SVDAG, Total\n");
      std::fprintf(fs, "time (ms), %.0f, %.0f\n", st.toDAGTime, st.buildSVOTime + st.toDAGTime + st.toSDAGTime);
    }
    std::fprintf(fs, "\n\n");
    std::fclose(fs);
  }
  return 0;
}
