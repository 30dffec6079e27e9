// svdag_reduce_dag_noalloc: toDAG whose temporaries live in a file-scope
// __device__ array instead of allocated memory (declared in
// include/svdag_gpu.h, which gives the size limit and the rules for callers).
//
// The array sits in its own translation unit so that, under CUDA's lazy
// module loading, its device memory is committed only when this entry point
// is first used.
#include <mutex>
#include <new>

#include "ctx.cuh"

namespace {

constexpr uint64_t kScratchBytes = SVDAG_NOALLOC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_dag_scratch[kScratchBytes];

// Device address of the array, looked up once per device (with that device
// current) and kept for the life of the process.
constexpr int kMaxDevices = 256;
std::mutex g_mu;
uint8_t* g_addr[kMaxDevices] = {};

uint8_t* static_scratch(int device) {
  if (device < 0 || device >= kMaxDevices)
    throw svdag::Error(SVDAG_ERR_INVALID_ARG, "svdag_reduce_dag_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_dag_scratch);
    if (rc != cudaSuccess || p == nullptr) {
      // loading the module commits the array; without room for it the
      // lookup fails with an allocation error
      const int code = rc == cudaErrorMemoryAllocation ? SVDAG_ERR_OOM : SVDAG_ERR_CUDA;
      if (rc != cudaSuccess) cudaGetLastError();
      throw svdag::Error(code, std::string("svdag_reduce_dag_noalloc: cudaGetSymbolAddress of the static "
                                           "scratch failed: ") + cudaGetErrorString(rc));
    }
    g_addr[device] = static_cast<uint8_t*>(p);
  }
  return g_addr[device];
}

}  // namespace

extern "C" int svdag_reduce_dag_noalloc(svdag_ctx* h) {
  if (!h) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    uint8_t* scratch = static_scratch(c.device);
    SVDAG_CUDA(cudaEventRecord(c.ev0, c.stream));
    svdag::phase_reduce_dag_scratch(c, scratch, kScratchBytes);
    SVDAG_CUDA(cudaEventRecord(c.ev1, c.stream));
    SVDAG_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    SVDAG_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.st.dag_ms = double(ms);
    // The outside masks belong to the SVO (svdag_reduce_dag drops them too).
    // Freeing is not allowed here, so they leave the levels and are released
    // by a later call on the context or by svdag_destroy.
    for (auto& L : c.lev)
      if (L.outm.get()) c.retired.push_back(std::move(L.outm));
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    c.last_error = "svdag_reduce_dag_noalloc: host allocation failed";
    return SVDAG_ERR_OOM;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return SVDAG_ERR_CUDA;
  }
}
