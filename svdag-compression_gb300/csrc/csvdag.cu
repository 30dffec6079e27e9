// GeomOctree::mergeAcrossAllLevels on the GPU (placeholder until the
// truncated-subtree formulation lands).
#include "ctx.cuh"

namespace svdag {

void phase_cross_level_merge(Ctx& c) {
  (void)c;
  throw Error(SVDAG_ERR_INVALID_STATE, "cross-level merge: not available in this build");
}

}  // namespace svdag
