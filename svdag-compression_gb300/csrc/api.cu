// C ABI of the SVDAG construction path (include/svdag_gpu.h).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include <new>

#include "ctx.cuh"

using svdag::Ctx;
using svdag::Error;

namespace {

// Imported node records: every set mask bit has a child below `limit`, and
// no pointer sits under a clear bit (what the reductions' kernels rely on).
__global__ void k_child_range(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ ch, uint64_t n,
                              uint64_t limit, int* __restrict__ bad) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t m = hdr[i] & 0xFFu;
    for (int c = 0; c < 8; ++c) {
      const uint32_t v = ch[8 * i + c];
      const bool set = (m >> c) & 1u;
      if (set ? (v == svdag::kNull || v >= limit) : (v != svdag::kNull)) atomicExch(bad, 1);
    }
  }
}

// Checks level l's children against level l+1 once both are imported.
void check_children(Ctx& c, uint32_t l) {
  if (l + 1 >= c.lev.size()) return;
  const svdag::Level& P = c.lev[l];
  const svdag::Level& Q = c.lev[l + 1];
  if (!P.hdr.get() || !Q.hdr.get() || !P.n) return;
  svdag::DBuf<int> bad(1, c.stream);
  SVDAG_CUDA(cudaMemsetAsync(bad.get(), 0, 4, c.stream));
  SVDAG_LAUNCH(c.ex, k_child_range, svdag::grid_for(c.ex, P.n, 256), 256, 0, P.hdr.get(), P.ch.get(), P.n, Q.n,
               bad.get());
  if (svdag::read_scalar(c.ex, bad.get())) {
    c.state = SVDAG_S_EMPTY;
    throw Error(SVDAG_ERR_INVALID_ARG, "import_level: a child pointer does not match the mask or the level below");
  }
}

int fail(svdag_ctx* h, int code, const std::string& msg) {
  if (h) h->c.last_error = msg;
  return code;
}

template <class F>
int guarded(svdag_ctx* h, F&& f) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  try {
    SVDAG_CUDA(cudaSetDevice(h->c.device));
    h->c.retired.clear();
    f(h->c);
    h->c.last_error.clear();
    return SVDAG_OK;
  } catch (const Error& e) {
    return fail(h, e.code, e.what());
  } catch (const std::bad_alloc&) {
    return fail(h, SVDAG_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(h, SVDAG_ERR_CUDA, e.what());
  }
}

// Runs one build phase between two events on the context stream and returns
// its device time in milliseconds.
template <class F>
double timed(Ctx& c, F&& f) {
  SVDAG_CUDA(cudaEventRecord(c.ev0, c.stream));
  f();
  SVDAG_CUDA(cudaEventRecord(c.ev1, c.stream));
  SVDAG_CUDA(cudaEventSynchronize(c.ev1));
  float ms = 0.f;
  SVDAG_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  return double(ms);
}

// Copies the live part of a level: `per_node` elements per node (at least one
// node's worth, so that an empty level keeps a non-null buffer), not the
// buffer's capacity -- a level reduced in place keeps its SVO-sized buffers.
void copy_level(const Ctx& src, svdag::Level& dst, const svdag::Level& s, cudaStream_t st) {
  dst.n = s.n;
  const uint64_t nodes = s.n ? s.n : 1;
  auto cp = [&](auto& d, const auto& v, uint64_t per_node) {
    if (!v.get()) return;
    const uint64_t cnt = std::min<uint64_t>(v.n, per_node * nodes);
    d.alloc(cnt, st);
    SVDAG_CUDA(cudaMemcpyAsync(d.get(), v.get(), cnt * sizeof(*v.get()), cudaMemcpyDeviceToDevice, st));
  };
  cp(dst.hdr, s.hdr, 1);
  cp(dst.ch, s.ch, 8);
  cp(dst.inv, s.inv, 1);
  cp(dst.clev, s.clev, 8);
  cp(dst.outm, s.outm, 1);
  (void)src;
}

}  // namespace

extern "C" {

const char* svdag_status_string(int s) {
  switch (s) {
    case SVDAG_OK: return "ok";
    case SVDAG_ERR_INVALID_ARG: return "invalid argument";
    case SVDAG_ERR_INVALID_STATE: return "invalid octree state";
    case SVDAG_ERR_CUDA: return "CUDA error";
    case SVDAG_ERR_OOM: return "out of device memory";
    case SVDAG_ERR_OVERFLOW: return "capacity overflow";
    case SVDAG_ERR_TIMEOUT: return "bounded wait expired";
    case SVDAG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* svdag_last_error(const svdag_ctx* h) { return h ? h->c.last_error.c_str() : "null context"; }

uint64_t svdag_device_alloc_count(void) { return svdag::g_device_allocs.load(std::memory_order_relaxed); }

int svdag_create(svdag_ctx** out, int device, void* stream) {
  if (!out) return SVDAG_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SVDAG_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return SVDAG_ERR_INVALID_ARG;
  svdag_ctx* h = new (std::nothrow) svdag_ctx();
  if (!h) return SVDAG_ERR_OOM;
  Ctx& c = h->c;
  c.device = device;
  try {
    SVDAG_CUDA(cudaSetDevice(device));
    if (stream) {
      c.stream = static_cast<cudaStream_t>(stream);
    } else {
      SVDAG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
      c.own_stream = true;
    }
    int sms = 0;
    SVDAG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    // keep freed blocks of the stream-ordered allocator cached between builds
    // (a process-local attribute of this device's default pool)
    cudaMemPool_t pool;
    SVDAG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = ~0ull;
    SVDAG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    c.ex.stream = c.stream;
    c.ex.sm_count = sms;
    c.ex.launches = &c.launches;
    SVDAG_CUDA(cudaEventCreate(&c.ev0));
    SVDAG_CUDA(cudaEventCreate(&c.ev1));
  } catch (const Error& e) {
    delete h;
    return e.code;
  }
  *out = h;
  return SVDAG_OK;
}

int svdag_destroy(svdag_ctx* h) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  Ctx& c = h->c;
  cudaSetDevice(c.device);
  // every stream-ordered buffer goes back before its stream is destroyed
  c.lev.clear();
  c.retired.clear();
  c.owned_tris.release();
  c.ss_inner.clear();
  c.ss_leaves.release();
  c.leaf_ctr.release();
  cudaStreamSynchronize(c.stream);
  if (c.ev0) cudaEventDestroy(c.ev0);
  if (c.ev1) cudaEventDestroy(c.ev1);
  if (c.own_stream) cudaStreamDestroy(c.stream);
  delete h;
  return SVDAG_OK;
}

int svdag_clone(const svdag_ctx* src, svdag_ctx** out) {
  if (!src) return SVDAG_ERR_INVALID_ARG;
  return svdag_clone_on(src, src->c.own_stream ? nullptr : src->c.stream, out);
}

int svdag_clone_on(const svdag_ctx* src, void* stream, svdag_ctx** out) {
  if (!src || !out) return SVDAG_ERR_INVALID_ARG;
  const Ctx& s = src->c;
  int r = svdag_create(out, s.device, stream);
  if (r != SVDAG_OK) return r;
  return guarded(*out, [&](Ctx& c) {
    c.tris = s.owned_tris.get() ? nullptr : s.tris;
    c.n_tris = s.owned_tris.get() ? 0 : s.n_tris;
    // wait for the source stream's work before copying on the new stream
    SVDAG_CUDA(cudaStreamSynchronize(s.stream));
    c.levels = s.levels;
    c.state = s.state;
    c.child_levels_init = s.child_levels_init;
    std::memcpy(c.bbox, s.bbox, sizeof(c.bbox));
    c.root_side = s.root_side;
    c.ex.persistent_blocks = s.ex.persistent_blocks;
    c.st = s.st;
    c.lev.resize(s.lev.size());
    for (size_t l = 0; l < s.lev.size(); ++l) copy_level(s, c.lev[l], s.lev[l], c.stream);
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int svdag_set_persistent_blocks(svdag_ctx* h, unsigned blocks) {
  return guarded(h, [&](Ctx& c) { c.ex.persistent_blocks = blocks; });
}

int svdag_synchronize(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) { SVDAG_CUDA(cudaStreamSynchronize(c.stream)); });
}

int svdag_upload_triangles(svdag_ctx* h, const float* host_tris, uint64_t n_tris) {
  if (!host_tris && n_tris) return fail(h, SVDAG_ERR_INVALID_ARG, "upload: null triangle pointer");
  return guarded(h, [&](Ctx& c) {
    c.owned_tris.alloc(9 * (n_tris ? n_tris : 1), c.stream);
    if (n_tris)
      SVDAG_CUDA(cudaMemcpyAsync(c.owned_tris.get(), host_tris, 36 * n_tris, cudaMemcpyHostToDevice, c.stream));
    c.tris = c.owned_tris.get();
    c.n_tris = n_tris;
  });
}

int svdag_set_device_triangles(svdag_ctx* h, const float* device_tris, uint64_t n_tris) {
  if (!device_tris && n_tris) return fail(h, SVDAG_ERR_INVALID_ARG, "set_device_triangles: null pointer");
  return guarded(h, [&](Ctx& c) {
    c.owned_tris.release();
    c.tris = device_tris;
    c.n_tris = n_tris;
  });
}

int svdag_voxelize(svdag_ctx* h, uint32_t levels, const double bbox[6]) {
  if (!bbox) return fail(h, SVDAG_ERR_INVALID_ARG, "voxelize: null bbox");
  return guarded(h, [&](Ctx& c) { c.st.svo_ms = timed(c, [&] { svdag::phase_voxelize(c, levels, bbox); }); });
}

int svdag_voxelize_ex(svdag_ctx* h, uint32_t levels, const double bbox[6], uint32_t flags) {
  if (!bbox) return fail(h, SVDAG_ERR_INVALID_ARG, "voxelize: null bbox");
  if (flags & ~uint32_t(SVDAG_VOXELIZE_LEAF_CENTERS)) return fail(h, SVDAG_ERR_INVALID_ARG, "voxelize_ex: unknown flags");
  return guarded(h, [&](Ctx& c) {
    c.keep_leaf_centers = (flags & SVDAG_VOXELIZE_LEAF_CENTERS) != 0;
    try {
      c.st.svo_ms = timed(c, [&] { svdag::phase_voxelize(c, levels, bbox); });
    } catch (...) {
      c.keep_leaf_centers = false;
      throw;
    }
    c.keep_leaf_centers = false;
  });
}

int svdag_download_leaf_centers(svdag_ctx* h, double* xyz, uint64_t capacity, uint64_t* count) {
  return guarded(h, [&](Ctx& c) {
    const uint64_t n = c.leaf_ctr.get() ? c.leaf_ctr_n : 0;
    if (count) *count = n;
    if (!xyz || !n) return;
    if (capacity < n) throw svdag::Error(SVDAG_ERR_OVERFLOW, "download_leaf_centers: capacity below the count");
    SVDAG_CUDA(cudaMemcpyAsync(xyz, c.leaf_ctr.get(), 24 * n, cudaMemcpyDeviceToHost, c.stream));
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int svdag_build_dag(svdag_ctx* h, uint32_t levels, uint32_t step_level, const double bbox[6]) {
  if (!bbox) return fail(h, SVDAG_ERR_INVALID_ARG, "build_dag: null bbox");
  return guarded(h, [&](Ctx& c) {
    c.st.svo_ms = timed(c, [&] { svdag::phase_build_dag(c, levels, step_level, bbox); });
    c.st.dag_ms = 0.0;
  });
}

int svdag_reduce_dag(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) {
    c.st.dag_ms = timed(c, [&] { svdag::phase_reduce_dag(c); });
    for (auto& L : c.lev) L.outm.release();  // outside masks belong to the SVO
  });
}

int svdag_tri_box_children(svdag_ctx* h, const float* tris, const double* centers, const double* half_sides,
                           uint64_t n, uint8_t* masks, uint64_t* fallbacks) {
  if (n && (!tris || !centers || !half_sides || !masks))
    return fail(h, SVDAG_ERR_INVALID_ARG, "tri_box_children: null buffer");
  return guarded(h, [&](Ctx& c) { svdag::tri_box_children(c, tris, centers, half_sides, n, masks, fallbacks); });
}

int svdag_sort_by_effective_refcount(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) { svdag::phase_sort_by_effective_refcount(c); });
}

int svdag_lossy_candidates(svdag_ctx* h, uint32_t level, float diff_factor, int included_ref_count,
                           const uint8_t* reps_below, uint32_t* src, uint32_t* tgt, float* weight, uint64_t capacity,
                           uint64_t* count) {
  if (!count) return fail(h, SVDAG_ERR_INVALID_ARG, "lossy candidates: null count");
  return guarded(h, [&](Ctx& c) {
    std::vector<uint32_t> s, t;
    std::vector<float> w;
    svdag::lossy_candidate_edges(c, level, diff_factor, included_ref_count, reps_below, s, t, w);
    *count = s.size();
    if (s.size() > capacity || (!s.empty() && (!src || !tgt || !weight))) {
      if (capacity || src || tgt || weight)
        throw Error(SVDAG_ERR_OVERFLOW, "lossy candidates: " + std::to_string(s.size()) + " edges, capacity " +
                                            std::to_string(capacity));
      return;  // size query
    }
    if (!s.empty()) {
      std::memcpy(src, s.data(), 4 * s.size());
      std::memcpy(tgt, t.data(), 4 * t.size());
      std::memcpy(weight, w.data(), 4 * w.size());
    }
  });
}

int svdag_init_child_levels(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) {
    if (c.state == SVDAG_S_EMPTY) throw Error(SVDAG_ERR_INVALID_STATE, "initChildLevels: empty octree");
    for (auto& L : c.lev) L.clev.release();
    c.child_levels_init = true;
  });
}

int svdag_reduce_sdag(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) { c.st.sdag_ms = timed(c, [&] { svdag::phase_reduce_sdag(c); }); });
}

int svdag_reduce_sdag_ex(svdag_ctx* h, uint32_t flags) {
  if (flags & ~uint32_t(SVDAG_SDAG_SKIP_SYMMETRY)) return fail(h, SVDAG_ERR_INVALID_ARG, "reduce_sdag_ex: unknown flags");
  if (!(flags & SVDAG_SDAG_SKIP_SYMMETRY)) return svdag_reduce_sdag(h);
  return guarded(h, [&](Ctx& c) { c.st.sdag_ms = timed(c, [&] { svdag::phase_reduce_sdag_skip_symmetry(c); }); });
}

int svdag_cross_level_merge(svdag_ctx* h) {
  return guarded(h, [&](Ctx& c) { c.st.csv_ms = timed(c, [&] { svdag::phase_cross_level_merge(c); }); });
}

int svdag_import_begin(svdag_ctx* h, uint32_t levels, const float bbox[6], double root_side, uint64_t n_total_voxels) {
  if (!bbox) return fail(h, SVDAG_ERR_INVALID_ARG, "import_begin: null bbox");
  return guarded(h, [&](Ctx& c) {
    if (levels < 1 || levels > 21) throw Error(SVDAG_ERR_INVALID_ARG, "import_begin: levels must be in [1, 21]");
    c.lev.clear();
    c.lev.resize(levels);
    c.levels = levels;
    std::memcpy(c.bbox, bbox, sizeof(c.bbox));
    c.root_side = root_side;
    c.state = SVDAG_S_DAG;
    c.child_levels_init = false;
    c.st = svdag_stats{};
    c.st.n_total_voxels = n_total_voxels;
    c.st.levels = levels;
  });
}

int svdag_import_level(svdag_ctx* h, uint32_t level, uint64_t count, const uint32_t* hdr, const uint32_t* children) {
  return guarded(h, [&](Ctx& c) {
    if (level >= c.lev.size()) throw Error(SVDAG_ERR_INVALID_ARG, "import_level: level out of range");
    if (count && !hdr) throw Error(SVDAG_ERR_INVALID_ARG, "import_level: null hdr");
    const bool inner = level + 1 < c.lev.size();
    if (count && inner && !children) throw Error(SVDAG_ERR_INVALID_ARG, "import_level: inner level needs children");
    svdag::Level& L = c.lev[level];
    L = svdag::Level();
    L.n = count;
    L.hdr.alloc(count ? count : 1, c.stream);
    if (count) SVDAG_CUDA(cudaMemcpyAsync(L.hdr.get(), hdr, 4 * count, cudaMemcpyHostToDevice, c.stream));
    if (inner) {
      L.ch.alloc(8 * (count ? count : 1), c.stream);
      if (count) SVDAG_CUDA(cudaMemcpyAsync(L.ch.get(), children, 32 * count, cudaMemcpyHostToDevice, c.stream));
    }
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
    check_children(c, level);
    if (level > 0) check_children(c, level - 1);
    uint64_t n = 1;
    for (size_t l = 1; l < c.lev.size(); ++l) n += c.lev[l].n;
    c.st.n_nodes = n;
    c.st.n_nodes_dag = n;
  });
}

int svdag_level_count(const svdag_ctx* h, uint32_t level, uint64_t* count) {
  if (!h || !count) return SVDAG_ERR_INVALID_ARG;
  if (level >= h->c.lev.size()) return SVDAG_ERR_INVALID_ARG;
  *count = h->c.lev[level].n;
  return SVDAG_OK;
}

int svdag_download_level(svdag_ctx* h, uint32_t level, uint32_t* hdr, uint32_t* children, uint8_t* child_levels,
                         uint8_t* invariant) {
  return guarded(h, [&](Ctx& c) {
    if (level >= c.lev.size()) throw Error(SVDAG_ERR_INVALID_ARG, "download: level out of range");
    const svdag::Level& L = c.lev[level];
    const uint64_t n = L.n;
    if (hdr && n) SVDAG_CUDA(cudaMemcpyAsync(hdr, L.hdr.get(), 4 * n, cudaMemcpyDeviceToHost, c.stream));
    if (children && n) {
      if (L.ch.get())
        SVDAG_CUDA(cudaMemcpyAsync(children, L.ch.get(), 32 * n, cudaMemcpyDeviceToHost, c.stream));
      else
        for (uint64_t i = 0; i < 8 * n; ++i) children[i] = svdag::kNull;
    }
    if (invariant && n) {
      if (L.inv.get())
        SVDAG_CUDA(cudaMemcpyAsync(invariant, L.inv.get(), n, cudaMemcpyDeviceToHost, c.stream));
      else
        std::memset(invariant, 0, n);
    }
    if (child_levels && n) {
      if (L.clev.get())
        SVDAG_CUDA(cudaMemcpyAsync(child_levels, L.clev.get(), 8 * n, cudaMemcpyDeviceToHost, c.stream));
      else
        std::memset(child_levels, c.child_levels_init ? int(level + 1) : 0xFF, 8 * n);
    }
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int svdag_get_stats(const svdag_ctx* h, svdag_stats* out) {
  if (!h || !out) return SVDAG_ERR_INVALID_ARG;
  *out = h->c.st;
  out->levels = h->c.levels;
  out->state = uint32_t(h->c.state);
  out->gpu_launches = h->c.launches;
  return SVDAG_OK;
}

int svdag_profile_enable(svdag_ctx* h, int enable) {
  return guarded(h, [&](Ctx& c) { c.ex.prof = enable ? &c.prof : nullptr; });
}

int svdag_profile_report(svdag_ctx* h, char* buf, uint64_t cap) {
  if (!buf || cap == 0) return fail(h, SVDAG_ERR_INVALID_ARG, "profile_report: no buffer");
  return guarded(h, [&](Ctx& c) {
    SVDAG_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<std::string> order;
    std::vector<std::pair<uint64_t, double>> acc;
    for (auto& r : c.prof.recs) {
      float ms = 0.f;
      SVDAG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      size_t k = 0;
      while (k < order.size() && order[k] != r.name) ++k;
      if (k == order.size()) { order.push_back(r.name); acc.push_back({0, 0.0}); }
      acc[k].first += 1;
      acc[k].second += ms;
      c.prof.pool.push_back(r.a);
      c.prof.pool.push_back(r.b);
    }
    c.prof.recs.clear();
    std::string out;
    char line[512];
    for (size_t k = 0; k < order.size(); ++k) {
      std::snprintf(line, sizeof(line), "%s;%llu;%.6f\n", order[k].c_str(), (unsigned long long)acc[k].first,
                    acc[k].second);
      out += line;
    }
    if (out.size() + 1 > cap) throw Error(SVDAG_ERR_OVERFLOW, "profile_report: buffer too small");
    std::memcpy(buf, out.c_str(), out.size() + 1);
  });
}

int svdag_level_device_ptrs(const svdag_ctx* h, uint32_t level, const uint32_t** hdr, const uint32_t** children,
                            const uint8_t** child_levels, const uint8_t** invariant) {
  if (!h || level >= h->c.lev.size()) return SVDAG_ERR_INVALID_ARG;
  const svdag::Level& L = h->c.lev[level];
  if (hdr) *hdr = L.hdr.get();
  if (children) *children = L.ch.get();
  if (child_levels) *child_levels = L.clev.get();
  if (invariant) *invariant = L.inv.get();
  return SVDAG_OK;
}

}  // extern "C"
