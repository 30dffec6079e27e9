// Lossy LSVDAG (lossy.cu) and its learned pair proposer (mlp.cu).
#pragma once

#include "ctx.cuh"

namespace svdag {

struct LossyConfig {
  uint32_t min_above = 3;     // candidate levels L-1-max_above .. L-1-min_above
  uint32_t max_above = 5;
  double max_error = 0.01;    // allowed voxel difference per replaced subtree (fraction of its cube's voxels)
  uint32_t top_k = 384;       // learned: proposals per candidate
  uint64_t train_pairs = 2000000;
  uint32_t epochs = 1;
  uint64_t seed = 1;
  uint32_t train_batch = 8192;  // learned: pairs per training step
  float lr = 2e-3f;             // learned: Adam learning rate
};

struct LossyResult {
  uint64_t nodes_before = 0, nodes_after = 0, candidates = 0, pairs_evaluated = 0, edges = 0, merged = 0;
  double ms = 0, propose_ms = 0, train_ms = 0;
  float loss = 0;
};

// Leaf voxels of the candidates of one level: 8^k Morton-ordered bytes each
// (k = levels below the candidate), and their voxel counts.
struct LevelSubtrees {
  uint32_t n = 0, k = 0;
  uint64_t words = 0;  // u64 words per candidate
  uint32_t lim = 0;    // largest allowed voxel difference on this level
  DBuf<uint64_t> bytes;
  DBuf<uint32_t> pop;
};

struct LossyProposer {
  virtual ~LossyProposer() = default;
  // candidate pairs (indices into the level's candidates) to check exactly
  virtual uint64_t propose(Ctx& c, uint32_t lev, const LevelSubtrees& S, const LossyConfig& cfg, DBuf<uint2>& pairs) = 0;
};

LevelSubtrees lossy_subtrees(Ctx& c, uint32_t lev, const uint32_t* d_cand, uint32_t n);
uint32_t lossy_limit(const LossyConfig& cfg, uint32_t levels, uint32_t lev);
uint64_t lossy_check_pairs(Ctx& c, const LevelSubtrees& S, const uint2* d_pairs, uint64_t n_pairs, uint32_t lim,
                           DBuf<uint2>& edges);
void phase_lossy(Ctx& c, const LossyConfig& cfg, LossyProposer* proposer, LossyResult& res);

}  // namespace svdag
