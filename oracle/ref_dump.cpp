// ref_dump: runs the REFERENCE SymVox build path (compiled from the
// reference's own src/symvox sources against oracle/sl_shim) on one OBJ and
// dumps every intermediate node pool.  Test infrastructure: it produces the
// golden vectors the restated oracle and the CUDA path are checked against.
//
//   ref_dump <scene.obj> <levels> <out_prefix> [step_levels] [options]
//
// Options (each adds an output; the reference code they run is named):
//   --soup            <out_prefix>.soup: the triangle soup Scene::loadObj
//                     built (scene.cpp:51-250, buildTriVector :394-416),
//                     u64 n, float bbox[6], then n float[9] triangles; with
//                     --soup-only nothing else is run
//   --flood           <out_prefix>.outside: GeomOctree::hiddenGeometryFloodfill
//                     (geom_octree_extension.cpp:1651-1891) on a copy of the
//                     SVO whose outside masks are zeroed first (the
//                     reference never initialises them), per level u64 count
//                     + one outsideMask byte per node.  Runs last: the
//                     reference exits when the start corner cell is set,
//                     after every other output is written
//   --lossy <infl> <diff> <refs>
//                     GeomOctree::toLossyDag (geom_octree_extension.cpp:
//                     797-1179) on a copy of the DAG, in the working
//                     directory: its candidate edges go to edges<lev>.txt
//                     before it runs the external MCL program as
//                     $HOME/local/bin/mcl (cluster.hpp:134-192), which the
//                     caller provides
//   --leaf-centers    <out_prefix>.leafctr: the leavesCenters list of a
//                     second GeomOctree::buildSVO(levels, bbox, true,
//                     &centers) (geom_octree.cpp:245-246): u64 n, then n
//                     double[3] (plain builds only)
//   --sdag-from-svo   <out_prefix>.sdagsvo.pool: GeomOctree::toSDAG straight
//                     on a copy of the SVO ("SVO -> SDAG", geom_octree.cpp:
//                     554-556), after initChildLevels (plain builds only)
//   --sdag-skip       <out_prefix>.sdagskip.pool: GeomOctree::toSDAG(true,
//                     true) -- skipSymmetry, pointer compression only
//                     (geom_octree.cpp:596-601); internalCall only silences
//                     its log -- on a copy of the DAG, and a REFSKIP line
//                     with its nNodesSDAG
//   --traverse <pts>  <out_prefix>.trav: EncodedSSVDAG::traverse
//                     (encoded_ssvdag.cpp:527-574) of the .ssvdag encoding
//                     for every point of <pts> (u64 n, then n float[3]); one
//                     int32 per point
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

static void dump_soup(Scene& scene, const std::string& path) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { std::perror(path.c_str()); std::exit(2); }
  const uint64_t n = scene.getNRawTriangles();
  auto lo = scene.getAABB()[0], hi = scene.getAABB()[1];
  const float bb[6] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
  std::fwrite(&n, 8, 1, fp);
  std::fwrite(bb, 4, 6, fp);
  for (uint64_t t = 0; t < n; ++t) {
    const sl::point3f* v = scene.getTrianglePtr(t);
    for (int i = 0; i < 3; ++i) {
      const float xyz[3] = {v[i][0], v[i][1], v[i][2]};
      std::fwrite(xyz, 4, 3, fp);
    }
  }
  std::fclose(fp);
}

static void dump_outside(const GeomOctree& oct, const std::string& path) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { std::perror(path.c_str()); std::exit(2); }
  const GeomOctree::NodeData& d = oct.getNodeData();
  for (size_t l = 0; l < d.size(); ++l) {
    const uint64_t n = d[l].size();
    std::fwrite(&n, 8, 1, fp);
    std::vector<unsigned char> m(n);
    for (uint64_t i = 0; i < n; ++i) m[i] = d[l][i].getOutsideMask();
    if (n) std::fwrite(m.data(), 1, n, fp);
  }
  std::fclose(fp);
}

static void dump_traverse(const EncodedSSVDAG& enc, const std::string& pts_path, const std::string& path) {
  FILE* fi = std::fopen(pts_path.c_str(), "rb");
  if (!fi) { std::perror(pts_path.c_str()); std::exit(2); }
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, fi) != 1) std::exit(2);
  std::vector<float> p(3 * n);
  if (n && std::fread(p.data(), 4, 3 * n, fi) != 3 * n) std::exit(2);
  std::fclose(fi);
  std::vector<int32_t> out(n);
  for (uint64_t i = 0; i < n; ++i) out[i] = enc.traverse(sl::point3f(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { std::perror(path.c_str()); std::exit(2); }
  if (n) std::fwrite(out.data(), 4, n, fp);
  std::fclose(fp);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: ref_dump scene.obj levels out_prefix [step_levels] [--soup|--soup-only] [--flood] "
                         "[--traverse points] [--lossy infl diff refs]\n");
    return 1;
  }
  std::string obj = argv[1];
  unsigned levels = (unsigned)std::atoi(argv[2]);
  std::string pre = argv[3];
  int step = 0;
  bool soup = false, soup_only = false, flood = false, lossy = false, sdag_skip = false, leaf_centers = false,
       sdag_from_svo = false;
  float infl = 2.f, diff_factor = 1.f;
  int refs = 1;
  std::string trav_pts;
  for (int a = 4; a < argc; ++a) {
    const std::string o = argv[a];
    if (o == "--soup") soup = true;
    else if (o == "--soup-only") soup = soup_only = true;
    else if (o == "--flood") flood = true;
    else if (o == "--sdag-skip") sdag_skip = true;
    else if (o == "--leaf-centers") leaf_centers = true;
    else if (o == "--sdag-from-svo") sdag_from_svo = true;
    else if (o == "--traverse" && a + 1 < argc) trav_pts = argv[++a];
    else if (o == "--lossy" && a + 3 < argc) {
      lossy = true;
      infl = std::strtof(argv[++a], nullptr);
      diff_factor = std::strtof(argv[++a], nullptr);
      refs = std::atoi(argv[++a]);
    }
    else step = std::atoi(argv[a]);
  }

  Scene scene;
  scene.loadObj(obj, false, false, false, false, true);
  if (soup) dump_soup(scene, pre + ".soup");
  if (soup_only) return 0;
  auto minF = scene.getAABB()[0], maxF = scene.getAABB()[1];
  sl::aabox3d bb(sl::point3d(minF[0], minF[1], minF[2]), sl::point3d(maxF[0], maxF[1], maxF[2]));

  if (leaf_centers && step == 0) {
    GeomOctree lc(&scene);
    std::vector<sl::point3d> centers;
    lc.buildSVO(levels, bb, true, &centers, false);
    FILE* f = std::fopen((pre + ".leafctr").c_str(), "wb");
    const uint64_t n = centers.size();
    std::fwrite(&n, 8, 1, f);
    for (const auto& c : centers) {
      const double v[3] = {c[0], c[1], c[2]};
      std::fwrite(v, 8, 3, f);
    }
    std::fclose(f);
  }

  GeomOctree oct(&scene);
  sl::real_time_clock ck;
  ck.restart();
  GeomOctree* svo_copy = nullptr;
  if (step == 0) {
    oct.buildSVO(levels, bb, false, NULL, false);
    dump_pool(oct, pre + ".svo.pool");
    if (sdag_from_svo) {
      GeomOctree s2(oct);
      s2.initChildLevels();
      s2.toSDAG(true, false);
      dump_pool(s2, pre + ".sdagsvo.pool");
    }
    if (flood) svo_copy = new GeomOctree(oct);
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
  if (!trav_pts.empty()) dump_traverse(ssvdag, trav_pts, pre + ".trav");

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
  std::fflush(stdout);
  if (sdag_skip) {
    GeomOctree sk(oct);
    sk.toSDAG(true, true);
    dump_pool(sk, pre + ".sdagskip.pool");
    std::printf("REFSKIP {\"nNodesSDAG\": %zu}\n", (size_t)sk.getStats().nNodesSDAG);
    std::fflush(stdout);
  }
  if (lossy) {
    GeomOctree lo(oct);
    lo.toLossyDag(infl, diff_factor, refs);
    std::printf("REFLOSSY {\"nodes_after\": %zu}\n", lo.getNNodes());
    std::fflush(stdout);
  }
  if (svo_copy) {
    // GeomOctree::Node's constructor (octree_node.cpp:22-37) leaves
    // outsideMask uninitialised (geom_octree.hpp:64) while the fill only ever
    // sets bits, so the masks start from indeterminate values; zero them
    // first, the state the fill assumes (it zeroes the root's itself, :1821)
    GeomOctree::NodeData& nd = const_cast<GeomOctree::NodeData&>(svo_copy->getNodeData());
    for (auto& lev : nd)
      for (auto& n : lev) n.outsideMask = 0;
    svo_copy->hiddenGeometryFloodfill();
    dump_outside(*svo_copy, pre + ".outside");
    delete svo_copy;
  }
  return 0;
}
