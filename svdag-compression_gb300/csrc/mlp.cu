// The learned pair proposer of the lossy LSVDAG (lossy.cu).
//
// A small MLP embeds a candidate subtree's coarse occupancy -- 8^3 = 512
// cells, each the fraction of set voxels in its Morton-aligned block: one
// cell per leaf brick for candidates three levels above the leaves, 8 or 64
// bricks four or five levels above -- through two ReLU layers of 256 into 64
// dimensions.  It is trained on the GPU, by the
// kernels below, so that the squared embedding distance of two subtrees
// tracks their exact voxel Hamming distance (normalised by their voxel
// counts), on pairs sampled from the scene itself and measured exactly.
// Proposals: for every candidate, the top_k partners by embedding distance
// among those whose voxel counts allow a merge at all; lossy.cu then checks
// each proposal with the exact distance, so the network only decides which
// pairs get checked, never which merges are accepted.
//
// Kernels: a tiled fp32 GEMM (128x128 block tile, 8x8 per thread, optional
// transposes, fused bias + ReLU, split-K for the weight gradients), the
// siamese loss and its gradient, bias gradients, Adam, and a banded top-k
// selection.  The layers are small (512x256 at most); they run on the FP32
// pipes.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>

#include "ctx.cuh"
#include "lossy.cuh"

namespace svdag {
namespace {

constexpr int kIn = 512, kH = 256, kOut = 64;
constexpr int kBM = 128, kBN = 128, kBK = 8;

// C[M x N] = op(A)[M x K] * op(B)[K x N] (+ bias[N]) (ReLU); row-major.
// TA: A is stored K x M; TB: B is stored N x K.  128x128 block tile, 8x8
// outputs per thread (rows ty*4+{0..3} and 64+ty*4+{0..3}, columns likewise),
// operands staged k-major in shared memory and read as float4.  With
// gridDim.z > 1 the K range is split and partial sums are added into C
// (zeroed by the caller; no bias or ReLU then).
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm(const float* __restrict__ A, const float* __restrict__ B,
                                              float* __restrict__ C, int M, int N, int K, int k_per,
                                              const float* __restrict__ bias, int relu, int accumulate) {
  __shared__ __align__(16) float sA[kBK][kBM];
  __shared__ __align__(16) float sB[kBK][kBN];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int row0 = blockIdx.y * kBM, col0 = blockIdx.x * kBN;
  const int kb = blockIdx.z * k_per, ke = min(K, kb + k_per);
  float acc[8][8] = {};
  for (int k0 = kb; k0 < ke; k0 += kBK) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = t * 4 + e;  // 0..1023 over the 128 x 8 tile
      int r, k;
      if (TA) { k = idx / kBM; r = idx % kBM; } else { r = idx / kBK; k = idx % kBK; }
      const int gr = row0 + r, gk = k0 + k;
      float a = 0.f;
      if (gr < M && gk < ke) a = TA ? A[size_t(gk) * M + gr] : A[size_t(gr) * K + gk];
      sA[k][r] = a;
      int c, kk;
      if (TB) { c = idx / kBK; kk = idx % kBK; } else { kk = idx / kBN; c = idx % kBN; }
      const int gc = col0 + c, gk2 = k0 + kk;
      float b = 0.f;
      if (gc < N && gk2 < ke) b = TB ? B[size_t(gc) * K + gk2] : B[size_t(gk2) * N + gc];
      sB[kk][c] = b;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      const float4 a0 = *reinterpret_cast<const float4*>(&sA[k][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sA[k][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&sB[k][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sB[k][64 + tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const bool split = gridDim.z > 1;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = row0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int cidx = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (cidx >= N) continue;
      float* o = C + size_t(r) * N + cidx;
      if (split) {
        atomicAdd(o, acc[i][j]);
        continue;
      }
      float v = acc[i][j];
      if (bias) v += bias[cidx];
      if (relu) v = fmaxf(v, 0.f);
      *o = accumulate ? *o + v : v;
    }
  }
}

// Splits K when the output has too few tiles to fill the GPU (the weight
// gradients: 512x256 outputs over K = 2 x batch rows).
template <bool TA, bool TB>
void gemm(const Exec& ex, const float* A, const float* B, float* C, int M, int N, int K, const float* bias = nullptr,
          bool relu = false, bool acc = false) {
  const int tiles = ((N + kBN - 1) / kBN) * ((M + kBM - 1) / kBM);
  int splits = 1;
  if (!bias && !relu && !acc && tiles < 2 * ex.sm_count) {
    splits = std::max(1, std::min(2 * ex.sm_count / tiles, K / 256));
  }
  const int k_per = ((K + splits - 1) / splits + kBK - 1) / kBK * kBK;
  splits = (K + k_per - 1) / k_per;
  if (splits > 1) SVDAG_CUDA(cudaMemsetAsync(C, 0, sizeof(float) * size_t(M) * N, ex.stream));
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM, splits);
  SVDAG_LAUNCH(ex, (k_gemm<TA, TB>), grid, 256, 0, A, B, C, M, N, K, k_per, bias, relu ? 1 : 0, acc ? 1 : 0);
}

// Siamese loss: rows [0, n) are side a, [n, 2n) side b of the embeddings.
// pred = |e_a - e_b|^2, loss = mean (pred - t)^2; dE written for both sides.
__global__ void k_pair_loss(const float* __restrict__ E, const float* __restrict__ t, int n, float* __restrict__ dE,
                            float* __restrict__ loss) {
  for (int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); p < n; p += gridDim.x * (blockDim.x / 32)) {
    const int lane = threadIdx.x & 31;
    const float d0 = E[size_t(p) * kOut + lane] - E[size_t(p + n) * kOut + lane];
    const float d1 = E[size_t(p) * kOut + lane + 32] - E[size_t(p + n) * kOut + lane + 32];
    float s = d0 * d0 + d1 * d1;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    const float r = s - t[p];
    const float g = 2.f * r / float(n);  // d loss / d pred
    dE[size_t(p) * kOut + lane] = g * 2.f * d0;
    dE[size_t(p) * kOut + lane + 32] = g * 2.f * d1;
    dE[size_t(p + n) * kOut + lane] = -g * 2.f * d0;
    dE[size_t(p + n) * kOut + lane + 32] = -g * 2.f * d1;
    if (lane == 0) atomicAdd(loss, r * r / float(n));
  }
}

// dX *= (H > 0)
__global__ void k_relu_back(float* __restrict__ dH, const float* __restrict__ H, size_t n) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    if (H[i] <= 0.f) dH[i] = 0.f;
}

// db[j] += sum over this block's rows of dY[i][j] (db zeroed by the caller)
constexpr int kBiasRows = 128;
__global__ void k_bias_grad(const float* __restrict__ dY, int M, int N, float* __restrict__ db) {
  const int r0 = blockIdx.y * kBiasRows, r1 = min(M, r0 + kBiasRows);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int i = r0; i < r1; ++i) s += dY[size_t(i) * N + j];
    atomicAdd(&db[j], s);
  }
}
void bias_grad(const Exec& ex, const float* dY, int M, int N, float* db) {
  SVDAG_CUDA(cudaMemsetAsync(db, 0, sizeof(float) * N, ex.stream));
  SVDAG_LAUNCH(ex, k_bias_grad, dim3((N + 255) / 256, (M + kBiasRows - 1) / kBiasRows), 256, 0, dY, M, N, db);
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float c1, float c2) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
  }
}

// Candidate features: 512 cells, the fraction of set voxels in each cell's
// Morton-aligned block (8 voxels per cell three levels above the leaves).
__global__ void k_features(const uint8_t* __restrict__ bytes, uint64_t per, uint32_t n, float* __restrict__ X) {
  const uint64_t g = per / kIn;  // bytes per cell
  const float inv = 1.f / float(8 * g);
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < uint64_t(n) * kIn;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t c = i / kIn, f = i % kIn;
    const uint8_t* p = bytes + c * per + f * g;
    uint32_t cnt = 0;
    for (uint64_t k = 0; k < g; ++k) cnt += __popc(uint32_t(p[k]));
    X[i] = float(cnt) * inv;
  }
}

// Rows of X for a batch of pairs: side a then side b.
__global__ void k_gather_pairs(const float* __restrict__ X, const uint2* __restrict__ pairs, int n,
                               float* __restrict__ out) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < size_t(2 * n) * kIn;
       i += size_t(gridDim.x) * blockDim.x) {
    const size_t r = i / kIn, f = i % kIn;
    const uint2 p = pairs[r < size_t(n) ? r : r - n];
    const uint32_t c = r < size_t(n) ? p.x : p.y;
    out[i] = X[size_t(c) * kIn + f];
  }
}

// Exact normalised distance of training pairs: |a xor b| / (|a| + |b|).
__global__ void k_pair_target(const uint64_t* __restrict__ w, uint64_t words, const uint32_t* __restrict__ pop,
                              const uint2* __restrict__ pairs, uint64_t n, float* __restrict__ t) {
  const int lane = threadIdx.x & 31;
  for (uint64_t p = blockIdx.x * uint64_t(blockDim.x / 32) + (threadIdx.x >> 5); p < n;
       p += uint64_t(gridDim.x) * (blockDim.x / 32)) {
    const uint2 q = pairs[p];
    uint32_t s = 0;
    for (uint64_t i = lane; i < words; i += 32) s += __popcll(w[q.x * words + i] ^ w[q.y * words + i]);
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    if (lane == 0) t[p] = float(s) / float(max(1u, pop[q.x] + pop[q.y]));
  }
}

// Top-k partners by embedding distance within each candidate's band (block
// per candidate, sorted-position order): bitonic sort of (kept, chunk).
constexpr int kSel = 1024;
__global__ void __launch_bounds__(256) k_topk_band(const float* __restrict__ E, const uint32_t* __restrict__ order,
                                                   const uint32_t* __restrict__ band_end, uint32_t n, int k,
                                                   uint2* __restrict__ out, const uint64_t* __restrict__ out_off) {
  __shared__ float sd[2 * kSel];
  __shared__ uint32_t si[2 * kSel];
  __shared__ float ei[kOut];
  for (uint32_t p = blockIdx.x; p < n; p += gridDim.x) {
    const uint32_t i = order[p];
    const uint32_t end = band_end[p];
    for (int d = threadIdx.x; d < kOut; d += blockDim.x) ei[d] = E[size_t(i) * kOut + d];
    int kept = 0;
    __syncthreads();
    for (uint32_t q0 = p + 1; q0 < end; q0 += kSel) {
      const uint32_t cnt = min(uint32_t(kSel), end - q0);
      // slots [0, kept) hold the current best; [kept, kept+cnt) the chunk
      for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) {
        const uint32_t j = order[q0 + t];
        float s = 0.f;
        for (int d = 0; d < kOut; ++d) {
          const float x = ei[d] - E[size_t(j) * kOut + d];
          s = fmaf(x, x, s);
        }
        sd[kept + t] = s;
        si[kept + t] = j;
      }
      int total = kept + int(cnt);
      int pw = 1;
      while (pw < total) pw <<= 1;
      for (int t = total + threadIdx.x; t < pw; t += blockDim.x) { sd[t] = INFINITY; si[t] = 0xFFFFFFFFu; }
      __syncthreads();
      for (int size = 2; size <= pw; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
          for (int t = threadIdx.x; t < pw; t += blockDim.x) {
            const int u = t ^ stride;
            if (u > t) {
              const bool asc = (t & size) == 0;
              const float a = sd[t], b = sd[u];
              const uint32_t ia = si[t], ib = si[u];
              const bool gt = (a > b) || (a == b && ia > ib);
              if (gt == asc) { sd[t] = b; sd[u] = a; si[t] = ib; si[u] = ia; }
            }
          }
          __syncthreads();
        }
      }
      kept = min(k, total);
      __syncthreads();
    }
    const uint64_t o = out_off[p];
    for (int t = threadIdx.x; t < kept; t += blockDim.x) out[o + t] = make_uint2(i, si[t]);
    __syncthreads();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
struct Mlp {
  // parameters: W1 [512x256], b1, W2 [256x256], b2, W3 [256x64], b3
  static constexpr size_t kSizes[6] = {size_t(kIn) * kH, kH, size_t(kH) * kH, kH, size_t(kH) * kOut, kOut};
  static size_t total() {
    size_t s = 0;
    for (size_t v : kSizes) s += v;
    return s;
  }
  DBuf<float> w, g, m, v;
  float* p[6] = {};
  float* gp[6] = {};
  int step = 0;
  void init(uint64_t seed, cudaStream_t st) {
    const size_t n = total();
    w.alloc(n, st);
    g.alloc(n, st);
    m.alloc(n, st);
    v.alloc(n, st);
    std::vector<float> h(n, 0.f);
    std::mt19937_64 rng(seed);
    size_t o = 0;
    const int fan_in[6] = {kIn, 0, kH, 0, kH, 0};
    for (int t = 0; t < 6; ++t) {
      if (fan_in[t]) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / float(fan_in[t])));
        for (size_t i = 0; i < kSizes[t]; ++i) h[o + i] = nd(rng);
      }
      o += kSizes[t];
    }
    SVDAG_CUDA(cudaMemcpyAsync(w.get(), h.data(), 4 * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemsetAsync(m.get(), 0, 4 * n, st));
    SVDAG_CUDA(cudaMemsetAsync(v.get(), 0, 4 * n, st));
    bind();
    step = 0;
  }
  void bind() {
    size_t o = 0;
    for (int t = 0; t < 6; ++t) { p[t] = w.get() + o; gp[t] = g.get() + o; o += kSizes[t]; }
  }
};
constexpr size_t Mlp::kSizes[6];

struct MlpWork {
  DBuf<float> X, H1, H2, E, dE, dH2, dH1, t;
  DBuf<float> loss;
  int cap = 0;
  void ensure(int rows, cudaStream_t st) {
    if (rows <= cap) return;
    cap = rows;
    X.alloc(size_t(rows) * kIn, st);
    H1.alloc(size_t(rows) * kH, st);
    H2.alloc(size_t(rows) * kH, st);
    E.alloc(size_t(rows) * kOut, st);
    dE.alloc(size_t(rows) * kOut, st);
    dH2.alloc(size_t(rows) * kH, st);
    dH1.alloc(size_t(rows) * kH, st);
    t.alloc(rows, st);
    loss.alloc(1, st);
  }
};

void mlp_forward(const Exec& ex, Mlp& net, MlpWork& W, int rows) {
  gemm<false, false>(ex, W.X.get(), net.p[0], W.H1.get(), rows, kH, kIn, net.p[1], true);
  gemm<false, false>(ex, W.H1.get(), net.p[2], W.H2.get(), rows, kH, kH, net.p[3], true);
  gemm<false, false>(ex, W.H2.get(), net.p[4], W.E.get(), rows, kOut, kH, net.p[5], false);
}

// Loss and gradients of one batch of n pairs (X rows: side a, then side b; t: targets).
void mlp_loss_grad(const Exec& ex, Mlp& net, MlpWork& W, int n) {
  const int rows = 2 * n;
  mlp_forward(ex, net, W, rows);
  SVDAG_CUDA(cudaMemsetAsync(W.loss.get(), 0, 4, ex.stream));
  SVDAG_LAUNCH(ex, k_pair_loss, grid_for(ex, n, 8), 256, 0, W.E.get(), W.t.get(), n, W.dE.get(), W.loss.get());
  // layer 3
  gemm<true, false>(ex, W.H2.get(), W.dE.get(), net.gp[4], kH, kOut, rows);
  bias_grad(ex, W.dE.get(), rows, kOut, net.gp[5]);
  gemm<false, true>(ex, W.dE.get(), net.p[4], W.dH2.get(), rows, kH, kOut);
  SVDAG_LAUNCH(ex, k_relu_back, grid_for(ex, size_t(rows) * kH, 256), 256, 0, W.dH2.get(), W.H2.get(), size_t(rows) * kH);
  // layer 2
  gemm<true, false>(ex, W.H1.get(), W.dH2.get(), net.gp[2], kH, kH, rows);
  bias_grad(ex, W.dH2.get(), rows, kH, net.gp[3]);
  gemm<false, true>(ex, W.dH2.get(), net.p[2], W.dH1.get(), rows, kH, kH);
  SVDAG_LAUNCH(ex, k_relu_back, grid_for(ex, size_t(rows) * kH, 256), 256, 0, W.dH1.get(), W.H1.get(), size_t(rows) * kH);
  // layer 1
  gemm<true, false>(ex, W.X.get(), W.dH1.get(), net.gp[0], kIn, kH, rows);
  bias_grad(ex, W.dH1.get(), rows, kH, net.gp[1]);
}

void mlp_adam(const Exec& ex, Mlp& net, float lr) {
  const float b1 = 0.9f, b2 = 0.999f;
  ++net.step;
  const float c1 = 1.f - std::pow(b1, float(net.step)), c2 = 1.f - std::pow(b2, float(net.step));
  const size_t n = Mlp::total();
  SVDAG_LAUNCH(ex, k_adam, grid_for(ex, n, 256), 256, 0, net.w.get(), net.g.get(), net.m.get(), net.v.get(), n, lr, b1,
               b2, c1, c2);
}

// ---------------------------------------------------------------------------
// The proposer: trains on the first level it sees (on pairs of that level and
// the ones sampled later), embeds each level's candidates, proposes top_k.
struct LearnedProposer : LossyProposer {
  Mlp net;
  MlpWork work;
  bool trained = false;
  bool train = true;   // false: use the network as initialised (the comparison without learning)
  double train_ms = 0;
  float last_loss = 0;

  uint64_t propose(Ctx& c, uint32_t lev, const LevelSubtrees& S, const LossyConfig& cfg, DBuf<uint2>& pairs) override {
    const Exec& ex = c.ex;
    const cudaStream_t st = c.stream;
    const uint32_t n = S.n;
    if (S.k < 3) throw Error(SVDAG_ERR_INVALID_ARG, "lossy: learned proposals need candidates 3+ levels above the leaves");
    // features of all candidates
    DBuf<float> X(size_t(n) * kIn, st);
    SVDAG_LAUNCH(ex, k_features, grid_for(ex, uint64_t(n) * kIn, 256), 256, 0,
                 reinterpret_cast<const uint8_t*>(S.bytes.get()), S.words * 8, n, X.get());
    // band of each sorted position (same bound as the exact enumeration)
    std::vector<uint32_t> hp(n);
    SVDAG_CUDA(cudaMemcpyAsync(hp.data(), S.pop.get(), 4ull * n, cudaMemcpyDeviceToHost, st));
    SVDAG_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> order(n), band_end(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return hp[a] < hp[b]; });
    {
      uint32_t e = 0;
      for (uint32_t p = 0; p < n; ++p) {
        if (e < p + 1) e = p + 1;
        while (e < n && hp[order[e]] - hp[order[p]] <= S.lim) ++e;
        band_end[p] = e;
      }
    }
    if (!trained) {
      if (train) {
        const auto t0 = std::chrono::steady_clock::now();
        fit(c, S, X, order, band_end, cfg);
        train_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      }
      trained = true;
    }
    // embeddings
    DBuf<float> E(size_t(n) * kOut, st);
    const int chunk = 16384;
    work.ensure(chunk, st);
    for (uint32_t r0 = 0; r0 < n; r0 += chunk) {
      const int rows = int(std::min<uint32_t>(chunk, n - r0));
      SVDAG_CUDA(cudaMemcpyAsync(work.X.get(), X.get() + size_t(r0) * kIn, 4ull * rows * kIn, cudaMemcpyDeviceToDevice, st));
      mlp_forward(ex, net, work, rows);
      SVDAG_CUDA(cudaMemcpyAsync(E.get() + size_t(r0) * kOut, work.E.get(), 4ull * rows * kOut, cudaMemcpyDeviceToDevice, st));
    }
    // top-k per candidate within its band
    std::vector<uint64_t> off(n + 1, 0);
    for (uint32_t p = 0; p < n; ++p) off[p + 1] = off[p] + std::min<uint32_t>(cfg.top_k, band_end[p] - p - 1);
    DBuf<uint32_t> d_order(n, st), d_end(n, st);
    DBuf<uint64_t> d_off(n + 1, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_order.get(), order.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_end.get(), band_end.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), off.data(), 8ull * (n + 1), cudaMemcpyHostToDevice, st));
    pairs.alloc(off[n] ? off[n] : 1, st);
    if (off[n])
      SVDAG_LAUNCH(ex, k_topk_band, std::min<uint32_t>(n, 152u * 8), 256, 0, E.get(), d_order.get(), d_end.get(), n,
                   int(cfg.top_k), pairs.get(), d_off.get());
    (void)lev;
    return off[n];
  }

  // Training pairs: half within the bands (near pairs), half uniform.
  void fit(Ctx& c, const LevelSubtrees& S, const DBuf<float>& X, const std::vector<uint32_t>& order,
           const std::vector<uint32_t>& band_end, const LossyConfig& cfg) {
    const Exec& ex = c.ex;
    const cudaStream_t st = c.stream;
    const uint32_t n = S.n;
    const uint64_t np = std::max<uint64_t>(1024, cfg.train_pairs);
    std::vector<uint2> hp(np);
    std::mt19937_64 rng(cfg.seed * 0x9E3779B97F4A7C15ull + 7);
    for (uint64_t i = 0; i < np; ++i) {
      const uint32_t p = uint32_t(rng() % n);
      uint32_t q;
      if ((i & 1) && band_end[p] > p + 1) q = p + 1 + uint32_t(rng() % (band_end[p] - p - 1));
      else q = uint32_t(rng() % n);
      hp[i] = make_uint2(order[p], order[q]);
    }
    DBuf<uint2> pairs(np, st);
    DBuf<float> target(np, st);
    SVDAG_CUDA(cudaMemcpyAsync(pairs.get(), hp.data(), 8 * np, cudaMemcpyHostToDevice, st));
    SVDAG_LAUNCH(ex, k_pair_target, grid_for(ex, np, 8, 16), 256, 0, S.bytes.get(), S.words, S.pop.get(), pairs.get(),
                 np, target.get());
    const int B = 4096;
    work.ensure(2 * B, st);
    float loss = 0;
    for (uint32_t ep = 0; ep < std::max(1u, cfg.epochs); ++ep) {
      for (uint64_t b0 = 0; b0 < np; b0 += B) {
        const int nb = int(std::min<uint64_t>(B, np - b0));
        SVDAG_LAUNCH(ex, k_gather_pairs, grid_for(ex, size_t(2 * nb) * kIn, 256), 256, 0, X.get(), pairs.get() + b0, nb,
                     work.X.get());
        SVDAG_CUDA(cudaMemcpyAsync(work.t.get(), target.get() + b0, 4ull * nb, cudaMemcpyDeviceToDevice, st));
        mlp_loss_grad(ex, net, work, nb);
        mlp_adam(ex, net, 1e-3f);
      }
      loss = read_scalar(ex, work.loss.get());
    }
    last_loss = loss;
    (void)n;
  }
};

void lossy_run(Ctx& c, const LossyConfig& cfg, int proposer, LossyResult& res) {
  if (proposer == 0) {
    phase_lossy(c, cfg, nullptr, res);
    return;
  }
  LearnedProposer P;
  P.net.init(cfg.seed, c.stream);
  P.train = proposer == 1;
  phase_lossy(c, cfg, &P, res);
  res.train_ms = P.train_ms;
  res.loss = P.last_loss;
}

// Host-buffer access to one network (tests: gradients against a CPU model).
struct MlpHandle {
  int device = 0;
  cudaStream_t stream = nullptr;
  Exec ex;
  uint64_t launches = 0;
  Mlp net;
  MlpWork work;
};

}  // namespace svdag

struct svdag_mlp {
  svdag::MlpHandle h;
};

extern "C" {

int svdag_mlp_create(svdag_mlp** out, int device, uint64_t seed) {
  if (!out) return SVDAG_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    SVDAG_CUDA(cudaSetDevice(device));
    svdag_mlp* m = new svdag_mlp();
    m->h.device = device;
    SVDAG_CUDA(cudaStreamCreateWithFlags(&m->h.stream, cudaStreamNonBlocking));
    m->h.ex.stream = m->h.stream;
    m->h.ex.launches = &m->h.launches;
    m->h.net.init(seed, m->h.stream);
    SVDAG_CUDA(cudaStreamSynchronize(m->h.stream));
    *out = m;
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    return e.code;
  } catch (const std::exception&) {
    return SVDAG_ERR_CUDA;
  }
}

int svdag_mlp_destroy(svdag_mlp* m) {
  if (!m) return SVDAG_ERR_INVALID_ARG;
  cudaSetDevice(m->h.device);
  cudaStreamSynchronize(m->h.stream);
  cudaStream_t s = m->h.stream;
  delete m;
  cudaStreamDestroy(s);
  return SVDAG_OK;
}

uint64_t svdag_mlp_param_count(void) { return svdag::Mlp::total(); }

int svdag_mlp_get_params(svdag_mlp* m, float* host) {
  if (!m || !host) return SVDAG_ERR_INVALID_ARG;
  cudaSetDevice(m->h.device);
  if (cudaMemcpyAsync(host, m->h.net.w.get(), 4 * svdag::Mlp::total(), cudaMemcpyDeviceToHost, m->h.stream) != cudaSuccess ||
      cudaStreamSynchronize(m->h.stream) != cudaSuccess)
    return SVDAG_ERR_CUDA;
  return SVDAG_OK;
}

int svdag_mlp_set_params(svdag_mlp* m, const float* host) {
  if (!m || !host) return SVDAG_ERR_INVALID_ARG;
  cudaSetDevice(m->h.device);
  if (cudaMemcpyAsync(m->h.net.w.get(), host, 4 * svdag::Mlp::total(), cudaMemcpyHostToDevice, m->h.stream) != cudaSuccess ||
      cudaStreamSynchronize(m->h.stream) != cudaSuccess)
    return SVDAG_ERR_CUDA;
  return SVDAG_OK;
}

// Forward + backward of n pairs given as host rows (x_a, x_b: n x 512; t: n):
// writes the loss and the gradient of every parameter (same layout as the
// parameters).
int svdag_mlp_loss_grad(svdag_mlp* m, const float* x_a, const float* x_b, const float* t, uint32_t n, float* loss,
                        float* grads) {
  if (!m || !x_a || !x_b || !t || !n || !loss || !grads) return SVDAG_ERR_INVALID_ARG;
  try {
    auto& H = m->h;
    SVDAG_CUDA(cudaSetDevice(H.device));
    H.work.ensure(int(2 * n), H.stream);
    SVDAG_CUDA(cudaMemcpyAsync(H.work.X.get(), x_a, 4ull * n * svdag::kIn, cudaMemcpyHostToDevice, H.stream));
    SVDAG_CUDA(cudaMemcpyAsync(H.work.X.get() + size_t(n) * svdag::kIn, x_b, 4ull * n * svdag::kIn,
                               cudaMemcpyHostToDevice, H.stream));
    SVDAG_CUDA(cudaMemcpyAsync(H.work.t.get(), t, 4ull * n, cudaMemcpyHostToDevice, H.stream));
    svdag::mlp_loss_grad(H.ex, H.net, H.work, int(n));
    SVDAG_CUDA(cudaMemcpyAsync(loss, H.work.loss.get(), 4, cudaMemcpyDeviceToHost, H.stream));
    SVDAG_CUDA(cudaMemcpyAsync(grads, H.net.g.get(), 4 * svdag::Mlp::total(), cudaMemcpyDeviceToHost, H.stream));
    SVDAG_CUDA(cudaStreamSynchronize(H.stream));
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    return e.code;
  }
}

// Embeddings of n host rows (n x 512) into host out (n x 64).
int svdag_mlp_embed(svdag_mlp* m, const float* x, uint32_t n, float* out) {
  if (!m || !x || !n || !out) return SVDAG_ERR_INVALID_ARG;
  try {
    auto& H = m->h;
    SVDAG_CUDA(cudaSetDevice(H.device));
    H.work.ensure(int(n), H.stream);
    SVDAG_CUDA(cudaMemcpyAsync(H.work.X.get(), x, 4ull * n * svdag::kIn, cudaMemcpyHostToDevice, H.stream));
    svdag::mlp_forward(H.ex, H.net, H.work, int(n));
    SVDAG_CUDA(cudaMemcpyAsync(out, H.work.E.get(), 4ull * n * svdag::kOut, cudaMemcpyDeviceToHost, H.stream));
    SVDAG_CUDA(cudaStreamSynchronize(H.stream));
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    return e.code;
  }
}

}  // extern "C"

extern "C" int svdag_lossy_dag(svdag_ctx* h, const svdag_lossy_params* p, svdag_lossy_stats* out) {
  if (!h || !p) return SVDAG_ERR_INVALID_ARG;
  svdag::Ctx& c = h->c;
  try {
    SVDAG_CUDA(cudaSetDevice(c.device));
    if (p->proposer > SVDAG_LOSSY_UNTRAINED) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "lossy: unknown proposer");
    svdag::LossyConfig cfg;
    cfg.min_above = p->levels_above_min;
    cfg.max_above = p->levels_above_max;
    cfg.max_error = p->max_error;
    cfg.top_k = p->top_k ? p->top_k : 16;
    cfg.train_pairs = p->train_pairs ? p->train_pairs : 2000000;
    cfg.epochs = p->train_epochs ? p->train_epochs : 2;
    cfg.seed = p->seed;
    if (cfg.top_k > 512) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "lossy: top_k above 512");
    svdag::LossyResult r;
    svdag::lossy_run(c, cfg, int(p->proposer), r);
    if (out) {
      out->nodes_before = r.nodes_before;
      out->nodes_after = r.nodes_after;
      out->candidates = r.candidates;
      out->pairs_evaluated = r.pairs_evaluated;
      out->edges = r.edges;
      out->merged = r.merged;
      out->ms = r.ms;
      out->propose_ms = r.propose_ms;
      out->train_ms = r.train_ms;
      out->final_loss = r.loss;
    }
    c.last_error.clear();
    return SVDAG_OK;
  } catch (const svdag::Error& e) {
    c.last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return SVDAG_ERR_CUDA;
  }
}
