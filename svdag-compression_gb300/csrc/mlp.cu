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
// Kernels: a tensor-core GEMM (mma.sync m16n8k16 on fp16 operands, fp32
// accumulation, tiles moved by cp.async in a 3-stage pipeline) with fused
// row gather, bias, ReLU, ReLU mask and column sums (bias gradients), split-K
// for the weight gradients; the siamese loss and its gradient, Adam, the
// training-pair sampler, and a banded top-k selection.  One training step is
// captured as a CUDA graph and replayed for every batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>
#include <type_traits>

#include <cuda_fp16.h>

#include "ctx.cuh"
#include "lossy.cuh"

namespace svdag {
namespace {

constexpr int kIn = 512, kH = 256, kOut = 64;

// ---------------------------------------------------------------------------
// Tensor-core GEMM on fp16 operands.  C[M x N] = op(A)[M x K] * op(B)[K x N]
// with fp32 accumulation (mma.sync m16n8k16).  A is stored M x K (K
// contiguous) or, with A_KM, K x M; B is stored K x N or, with B_NK, N x K;
// both are fp16 in global memory.  A's stored rows may be gathered through
// `rowmap` (stored row r is row rowmap[r] of the array).  C is fp32 or fp16,
// row-major.  Epilogue, in order: x alpha, + bias[n] (fp32), ReLU, a ReLU
// mask (C[m][n] = 0 where mask[m][n] <= 0: the backward of a ReLU layer),
// column sums x colsum_scale added into colsum[N] (bias gradients); with
// gridDim.z > 1, atomic partial sums over a split K range (fp32 C zeroed by
// the caller).
//
// Block tile BM x BN x 64, 8 warps of (BM/WGM) x (BN/WGN) warp tiles built
// from m16n8 fragments loaded by ldmatrix (.trans for the K-major / K x N
// layouts).  Tiles move global -> shared memory with 16-byte cp.async in a
// 3-stage pipeline (two tiles in flight while one is multiplied); rows past
// the matrix are zero-filled by the copy itself.  Dimensions along which a
// tile is read in 8-element chunks (K for M x K / N x K storage, M and N
// otherwise) must be whole tiles (multiples of 64 along K, of the tile width
// along M and N) -- true of every layer width here.
constexpr int kBK = 64, kPad = 8, kGemmThreads = 256, kStages = 3;

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TRANS>
__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void* smem) {
  const uint32_t a = uint32_t(__cvta_generic_to_shared(smem));
  if (TRANS)
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
  else
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

// 16-byte global -> shared copy; src_bytes = 0 writes zeros.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, uint32_t src_bytes) {
  const uint32_t a = uint32_t(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(a), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Copies a ROWS x COLS tile (COLS contiguous in global memory, 8-element
// chunks) of a row-major fp16 matrix with leading dimension ld: global rows
// [r0, r0 + ROWS) below rlim (through rowmap when given), columns
// [c0, c0 + COLS); rows at or past rlim are zero.
template <int ROWS, int COLS>
__device__ __forceinline__ void tile_copy(__half* s, const __half* g, int ld, int r0, int rlim, int c0,
                                          const uint32_t* rowmap) {
  constexpr int kChunks = ROWS * COLS / 8;
  static_assert(kChunks % kGemmThreads == 0, "tile shape");
#pragma unroll
  for (int i = 0; i < kChunks / kGemmThreads; ++i) {
    const int ch = threadIdx.x + i * kGemmThreads;
    const int r = ch / (COLS / 8), c = (ch % (COLS / 8)) * 8;
    const int gr = r0 + r;
    const bool ok = gr < rlim;
    const __half* src = ok ? g + size_t(rowmap ? rowmap[gr] : uint32_t(gr)) * ld + c0 + c : g;
    cp_async16(s + r * (COLS + kPad) + c, src, ok ? 16u : 0u);
  }
}

template <class OutT>
__device__ __forceinline__ void store2(OutT* o, float a, float b);
template <>
__device__ __forceinline__ void store2<float>(float* o, float a, float b) {
  *reinterpret_cast<float2*>(o) = make_float2(a, b);
}
template <>
__device__ __forceinline__ void store2<__half>(__half* o, float a, float b) {
  *reinterpret_cast<__half2*>(o) = __floats2half2_rn(a, b);
}

template <bool A_KM, bool B_NK, int BM, int BN, int WGM>
struct GemmShape {
  static constexpr int WGN = 8 / WGM;
  static constexpr int WM = BM / WGM, WN = BN / WGN;
  static constexpr int MI = WM / 16, NI = WN / 8;
  static constexpr int AR = A_KM ? kBK : BM, AC = A_KM ? BM : kBK;
  static constexpr int BR = B_NK ? BN : kBK, BC = B_NK ? kBK : BN;
  static constexpr int kA = AR * (AC + kPad), kB = BR * (BC + kPad);
  static constexpr int kSmemBytes = kStages * (kA + kB) * 2;
};

template <bool A_KM, bool B_NK, int BM, int BN, int WGM, class OutT>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_tc(const __half* __restrict__ A, const __half* __restrict__ B,
                                                          OutT* __restrict__ C, int M, int N, int K, int k_per,
                                                          const uint32_t* __restrict__ rowmap, float alpha,
                                                          const float* __restrict__ bias, int relu,
                                                          const __half* __restrict__ mask, float* __restrict__ colsum,
                                                          float colsum_scale) {
  using S = GemmShape<A_KM, B_NK, BM, BN, WGM>;
  constexpr int WM = S::WM, WN = S::WN, MI = S::MI, NI = S::NI, AC = S::AC, BC = S::BC;
  static_assert(MI >= 1 && NI >= 2 && NI % 2 == 0, "warp tile");
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __half* sA = reinterpret_cast<__half*>(smem_raw);
  __half* sB = sA + kStages * S::kA;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp % WGM, wn = warp / WGM;
  const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
  const int kb = blockIdx.z * k_per, ke = min(K, kb + k_per);
  const int nk = ke > kb ? (ke - kb + kBK - 1) / kBK : 0;

  auto load = [&](int t, int stage) {
    const int k0 = kb + t * kBK;
    __half* a = sA + stage * S::kA;
    __half* b = sB + stage * S::kB;
    if (A_KM) tile_copy<S::AR, AC>(a, A, M, k0, ke, row0, rowmap);
    else tile_copy<S::AR, AC>(a, A, K, row0, M, k0, rowmap);
    if (B_NK) tile_copy<S::BR, BC>(b, B, K, col0, N, k0, nullptr);
    else tile_copy<S::BR, BC>(b, B, N, k0, ke, col0, nullptr);
  };
  float acc[MI][NI][4];
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NI; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

#pragma unroll
  for (int t = 0; t < kStages - 1; ++t) {
    if (t < nk) load(t, t);
    cp_async_commit();
  }
  for (int it = 0; it < nk; ++it) {
    cp_async_wait<kStages - 2>();
    __syncthreads();  // tile `it` visible to all warps; stage (it - 1) % kStages free
    if (it + kStages - 1 < nk) load(it + kStages - 1, (it + kStages - 1) % kStages);
    cp_async_commit();
    const __half* a_s = sA + (it % kStages) * S::kA;
    const __half* b_s = sB + (it % kStages) * S::kB;
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[MI][4], bf[NI][2];
#pragma unroll
      for (int mi = 0; mi < MI; ++mi) {
        const int mb = wm * WM + mi * 16;
        if (A_KM) {
          const int j = lane >> 3, r = lane & 7;
          ldsm_x4<true>(af[mi], a_s + (kk + r + (j >= 2 ? 8 : 0)) * (AC + kPad) + mb + ((j & 1) ? 8 : 0));
        } else {
          ldsm_x4<false>(af[mi], a_s + (mb + (lane & 15)) * (AC + kPad) + kk + (lane >> 4) * 8);
        }
      }
#pragma unroll
      for (int ni = 0; ni < NI; ni += 2) {
        const int nb = wn * WN + ni * 8;
        const int j = lane >> 3, r = lane & 7;
        uint32_t t[4];
        if (B_NK) ldsm_x4<false>(t, b_s + (nb + r + (j >= 2 ? 8 : 0)) * (BC + kPad) + kk + ((j & 1) ? 8 : 0));
        else ldsm_x4<true>(t, b_s + (kk + r + ((j & 1) ? 8 : 0)) * (BC + kPad) + nb + (j >= 2 ? 8 : 0));
        bf[ni][0] = t[0];
        bf[ni][1] = t[1];
        bf[ni + 1][0] = t[2];
        bf[ni + 1][1] = t[3];
      }
#pragma unroll
      for (int mi = 0; mi < MI; ++mi)
#pragma unroll
        for (int ni = 0; ni < NI; ++ni) mma16816(acc[mi][ni], af[mi], bf[ni]);
    }
  }
  cp_async_wait<0>();

  const bool split = gridDim.z > 1;
  const int g = lane >> 2, t4 = lane & 3;
  float cs[NI][2];
#pragma unroll
  for (int ni = 0; ni < NI; ++ni) cs[ni][0] = cs[ni][1] = 0.f;
#pragma unroll
  for (int mi = 0; mi < MI; ++mi)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = row0 + wm * WM + mi * 16 + g + h * 8;
      if (r >= M) continue;
#pragma unroll
      for (int ni = 0; ni < NI; ++ni) {
        const int c = col0 + wn * WN + ni * 8 + t4 * 2;  // N is a multiple of the tile width
        float v0 = alpha * acc[mi][ni][2 * h], v1 = alpha * acc[mi][ni][2 * h + 1];
        OutT* o = C + size_t(r) * N + c;
        if (split) {
          atomicAdd(reinterpret_cast<float*>(o), v0);
          atomicAdd(reinterpret_cast<float*>(o) + 1, v1);
          continue;
        }
        if (bias) { v0 += bias[c]; v1 += bias[c + 1]; }
        if (relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
        if (mask) {
          const __half2 mk = *reinterpret_cast<const __half2*>(mask + size_t(r) * N + c);
          if (!(__low2float(mk) > 0.f)) v0 = 0.f;
          if (!(__high2float(mk) > 0.f)) v1 = 0.f;
        }
        cs[ni][0] += v0;
        cs[ni][1] += v1;
        store2<OutT>(o, v0, v1);
      }
    }
  if (colsum && !split) {
    // lanes with the same t4 hold the same columns: reduce over g, then one
    // atomic per column and warp row
#pragma unroll
    for (int ni = 0; ni < NI; ++ni)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        float v = cs[ni][e];
        v += __shfl_xor_sync(0xFFFFFFFFu, v, 4);
        v += __shfl_xor_sync(0xFFFFFFFFu, v, 8);
        v += __shfl_xor_sync(0xFFFFFFFFu, v, 16);
        if (g == 0) atomicAdd(&colsum[col0 + wn * WN + ni * 8 + t4 * 2 + e], v * colsum_scale);
      }
  }
}

struct GemmOpts {
  const uint32_t* rowmap = nullptr;  // gather of A's stored rows
  float alpha = 1.f;
  const float* bias = nullptr;
  bool relu = false;
  const __half* mask = nullptr;      // ReLU backward mask (same shape as C)
  float* colsum = nullptr;           // column sums of the result (x colsum_scale), zeroed by the caller
  float colsum_scale = 1.f;
  bool zeroed = false;               // fp32 C already zero (split-K accumulates into it)
};

template <bool A_KM, bool B_NK, int BM, int BN, int WGM, class OutT>
void launch_gemm(const Exec& ex, dim3 grid, const __half* A, const __half* B, OutT* C, int M, int N, int K, int k_per,
                 const GemmOpts& o) {
  using S = GemmShape<A_KM, B_NK, BM, BN, WGM>;
  auto* kern = k_gemm_tc<A_KM, B_NK, BM, BN, WGM, OutT>;
  static bool attr = false;  // per instantiation; the attribute is a process-wide property of the function
  if (!attr) {
    SVDAG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmemBytes));
    attr = true;
  }
  SVDAG_LAUNCH(ex, (k_gemm_tc<A_KM, B_NK, BM, BN, WGM, OutT>), grid, kGemmThreads, S::kSmemBytes, A, B, C, M, N, K,
               k_per, o.rowmap, o.alpha, o.bias, o.relu ? 1 : 0, o.mask, o.colsum, o.colsum_scale);
}

// Splits K when the output has too few tiles to fill the GPU (the weight
// gradients: at most 512 x 256 outputs over K = 2 x batch rows); split
// results are atomic partial sums into C (fp32), which is zeroed here unless
// the caller already did.
// Row-major A (M = batch rows, many tiles) uses 64-row tiles: twice the
// blocks of 128-row ones, two of them resident per SM (the GEMMs are small
// and latency-bound; ncu: one 8-warp block per SM left the tensor pipe busy
// a quarter of the time) -- unless 64-row tiles would need more than one
// wave of two blocks per SM and 128-row ones would not (wide layers of
// 16,384-row batches).  K-major A (M = a layer width) keeps 128 rows and
// splits K instead.
template <bool A_KM, bool B_NK, class OutT>
void gemm_tc(const Exec& ex, const __half* A, const __half* B, OutT* C, int M, int N, int K,
             const GemmOpts& o = GemmOpts()) {
  const bool narrow = N <= 64;
  const int BN = narrow ? 64 : 128;
  const int wave = 2 * ex.sm_count;
  const bool tall = A_KM || (!narrow && (N / BN) * ((M + 63) / 64) > wave && (N / BN) * ((M + 127) / 128) <= wave);
  const int BM = tall ? 128 : 64;
  // chunked dimensions (see k_gemm_tc) must be whole tiles
  if (N % BN || (A_KM && M % BM) || (!A_KM && K % kBK) || (B_NK && K % kBK))
    throw Error(SVDAG_ERR_INVALID_ARG, "gemm: unsupported shape");
  const int tiles = (N / BN) * ((M + BM - 1) / BM);
  int splits = 1;
  const bool can_split = std::is_same<OutT, float>::value && !o.bias && !o.relu && !o.mask && !o.colsum;
  if (can_split && tiles < ex.sm_count) splits = std::max(1, std::min(2 * ex.sm_count / tiles, K / 256));
  const int k_per = ((K + splits - 1) / splits + kBK - 1) / kBK * kBK;
  splits = (K + k_per - 1) / k_per;
  if (splits > 1 && !o.zeroed) SVDAG_CUDA(cudaMemsetAsync(C, 0, sizeof(OutT) * size_t(M) * N, ex.stream));
  const dim3 grid(N / BN, (M + BM - 1) / BM, splits);
  if constexpr (A_KM) {
    if (narrow) launch_gemm<A_KM, B_NK, 128, 64, 4, OutT>(ex, grid, A, B, C, M, N, K, k_per, o);
    else launch_gemm<A_KM, B_NK, 128, 128, 2, OutT>(ex, grid, A, B, C, M, N, K, k_per, o);
  } else {
    if (narrow) launch_gemm<A_KM, B_NK, 64, 64, 2, OutT>(ex, grid, A, B, C, M, N, K, k_per, o);
    else if (tall) launch_gemm<A_KM, B_NK, 128, 128, 2, OutT>(ex, grid, A, B, C, M, N, K, k_per, o);
    else launch_gemm<A_KM, B_NK, 64, 128, 2, OutT>(ex, grid, A, B, C, M, N, K, k_per, o);
  }
}

// Static loss scale of the fp16 backward: the loss gradient is multiplied by
// it before it is rounded to fp16 (gradients of order 1e-6 stay normal fp16
// values), and the epilogues that produce the fp32 parameter gradients divide
// by it again.
constexpr float kLossScale = 1024.f;

// Siamese loss: rows [0, n) are side a, [n, 2n) side b of the embeddings.
// pred = |e_a - e_b|^2, loss = mean (pred - t)^2; dE (x kLossScale, fp16)
// written for both sides.  `counter` (training graph): the step counter,
// advanced here once the batch setup of this step has read it and before
// Adam reads it.
__global__ void k_pair_loss(const float* __restrict__ E, const float* __restrict__ t, int n, __half* __restrict__ dE,
                            float* __restrict__ loss, unsigned long long* __restrict__ counter) {
  pdl_wait();
  pdl_trigger();
  if (counter && blockIdx.x == 0 && threadIdx.x == 0) *counter += 1;
  for (int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); p < n; p += gridDim.x * (blockDim.x / 32)) {
    const int lane = threadIdx.x & 31;
    const float d0 = E[size_t(p) * kOut + lane] - E[size_t(p + n) * kOut + lane];
    const float d1 = E[size_t(p) * kOut + lane + 32] - E[size_t(p + n) * kOut + lane + 32];
    float s = d0 * d0 + d1 * d1;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    const float r = s - t[p];
    const float g = kLossScale * 2.f * r / float(n);  // d loss / d pred, scaled
    dE[size_t(p) * kOut + lane] = __float2half_rn(g * 2.f * d0);
    dE[size_t(p) * kOut + lane + 32] = __float2half_rn(g * 2.f * d1);
    dE[size_t(p + n) * kOut + lane] = __float2half_rn(-g * 2.f * d0);
    dE[size_t(p + n) * kOut + lane + 32] = __float2half_rn(-g * 2.f * d1);
    if (lane == 0) atomicAdd(loss, r * r / float(n));
  }
}

// Adam; also refreshes the fp16 copy of the parameters the GEMMs read.
__global__ void k_adam(float* __restrict__ w, __half* __restrict__ wh, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, size_t n, float lr, float b1, float b2, float c1,
                       float c2) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    w[i] = wi;
    wh[i] = __float2half_rn(wi);
  }
}

// Adam with the step number read from the device (training replays one
// captured step graph; the loss kernel has already advanced the counter):
// step = *counter.  The gradients are zeroed for the next step's
// accumulation once read.
__global__ void k_adam_dev(float* __restrict__ w, __half* __restrict__ wh, float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, size_t n, float lr, float b1, float b2,
                           const unsigned long long* __restrict__ counter) {
  const float t = float(*counter);
  const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    g[i] = 0.f;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    w[i] = wi;
    wh[i] = __float2half_rn(wi);
  }
}

// Training pairs drawn on the device from a counter-based generator
// (splitmix64 of seed and pair index): pair i takes a candidate p at a
// uniform sorted position and, for odd i when p's band has partners, a
// partner inside the band (near pairs), otherwise a uniform one.  Written as
// the pair (for the exact targets) and as input-row indices laid out per
// batch of B pairs (the a sides, then the b sides).
__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_sample_pairs(const uint32_t* __restrict__ order, const uint32_t* __restrict__ band_end, uint32_t n,
                               uint64_t np, int B, uint64_t seed, uint2* __restrict__ pairs,
                               uint32_t* __restrict__ rows) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < np; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t r0 = splitmix(seed ^ (2 * i)), r1 = splitmix(seed ^ (2 * i + 1));
    const uint32_t p = uint32_t(r0 % n);
    const uint32_t e = band_end[p];
    const uint32_t q = ((i & 1) && e > p + 1) ? p + 1 + uint32_t(r1 % (e - p - 1)) : uint32_t(r1 % n);
    const uint2 pr = make_uint2(order[p], order[q]);
    pairs[i] = pr;
    const uint64_t b0 = i / B * B, j = i - b0;
    rows[2 * b0 + j] = pr.x;
    rows[2 * b0 + B + j] = pr.y;
  }
}

// Start of a replayed training step: batch (*counter mod batches) of the
// epoch's rows and targets into the step's fixed buffers, and the loss
// accumulator zeroed.
__global__ void k_batch_setup(const unsigned long long* __restrict__ counter, uint32_t batches, int B,
                              const uint32_t* __restrict__ rows_all, const float* __restrict__ t_all,
                              uint32_t* __restrict__ rows, float* __restrict__ t, float* __restrict__ loss) {
  const uint64_t b = *counter % batches;
  if (blockIdx.x == 0 && threadIdx.x == 0) *loss = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * B; i += gridDim.x * blockDim.x) {
    rows[i] = rows_all[2 * b * B + i];
    if (i < B) t[i] = t_all[b * B + i];
  }
}

// Candidate features: 512 cells, the fraction of set voxels in each cell's
// Morton-aligned block (8 voxels per cell three levels above the leaves).
// (The fractions k / (8 g) are exact in fp16 for the 1, 8 and 64 bytes per
// cell of candidates 3-5 levels above the leaves.)
__global__ void k_features(const uint8_t* __restrict__ bytes, uint64_t per, uint32_t n, __half* __restrict__ X) {
  const uint64_t g = per / kIn;  // bytes per cell
  const float inv = 1.f / float(8 * g);
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < uint64_t(n) * kIn;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t c = i / kIn, f = i % kIn;
    const uint8_t* p = bytes + c * per + f * g;
    uint32_t cnt = 0;
    for (uint64_t k = 0; k < g; ++k) cnt += __popc(uint32_t(p[k]));
    X[i] = __float2half_rn(float(cnt) * inv);
  }
}

// fp32 rows -> fp16 (network input of the C ABI's test entry points, and the
// fp16 copy of the parameters)
__global__ void k_to_half(const float* __restrict__ x, size_t n, __half* __restrict__ out) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    out[i] = __float2half_rn(x[i]);
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
  DBuf<__half> wh;  // fp16 copy of w, the GEMMs' operand (refreshed by Adam and set_params)
  float* p[6] = {};
  float* gp[6] = {};
  __half* h[6] = {};
  int step = 0;
  void init(uint64_t seed, cudaStream_t st) {
    const size_t n = total();
    w.alloc(n, st);
    wh.alloc(n, st);
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
    refresh_half(st);
    step = 0;
  }
  void bind() {
    size_t o = 0;
    for (int t = 0; t < 6; ++t) { p[t] = w.get() + o; gp[t] = g.get() + o; h[t] = wh.get() + o; o += kSizes[t]; }
  }
  void refresh_half(cudaStream_t st);
};
constexpr size_t Mlp::kSizes[6];
void Mlp::refresh_half(cudaStream_t st) {
  k_to_half<<<unsigned(std::min<size_t>((total() + 255) / 256, 4096)), 256, 0, st>>>(w.get(), total(), wh.get());
  SVDAG_CUDA(cudaGetLastError());
}

// Activations and gradients of one batch (rows = 2 x pairs: side a, then
// side b); inputs, hidden activations and hidden gradients are fp16.
struct MlpWork {
  DBuf<__half> X, H1, H2, dE, dH2, dH1;
  DBuf<float> E, t, loss, xin;
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

// Forward of `rows` input rows (row r = X row rowmap[r] when given): fp16
// operands (the inputs are exact in fp16) and hidden activations, fp32
// accumulation, fp32 embeddings.
void mlp_forward(const Exec& ex, Mlp& net, MlpWork& W, const __half* X, const uint32_t* rowmap, int rows) {
  GemmOpts o1;
  o1.rowmap = rowmap;
  o1.bias = net.p[1];
  o1.relu = true;
  gemm_tc<false, false, __half>(ex, X, net.h[0], W.H1.get(), rows, kH, kIn, o1);
  GemmOpts o2;
  o2.bias = net.p[3];
  o2.relu = true;
  gemm_tc<false, false, __half>(ex, W.H1.get(), net.h[2], W.H2.get(), rows, kH, kH, o2);
  GemmOpts o3;
  o3.bias = net.p[5];
  gemm_tc<false, false, float>(ex, W.H2.get(), net.h[4], W.E.get(), rows, kOut, kH, o3);
}

// A second stream and fork / join events for the weight-gradient GEMMs,
// which run beside the hidden-gradient GEMMs of the same layer inside a
// captured training step (graph branches).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork[2] = {nullptr, nullptr}, join = nullptr;
  void create() {
    SVDAG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto& e : fork) SVDAG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    SVDAG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  }
  ~SideStream() {
    for (auto e : fork)
      if (e) cudaEventDestroy(e);
    if (join) cudaEventDestroy(join);
    if (stream) cudaStreamDestroy(stream);
  }
};

// Loss and gradients of one batch of n pairs (X rows through rowmap: side a,
// then side b; W.t: targets).  The backward runs on fp16 operands scaled by
// kLossScale (dE, dH2, dH1), fp32 accumulation; the ReLU backward and the
// bias gradients are fused into the GEMMs that produce dH2 and dH1 (the
// output bias's gradient is an exact zero: the two sides of every pair
// contribute opposite terms), and the weight-gradient epilogues undo the
// scale.  Every gradient is zeroed by one memset -- or, inside the captured
// training step (`counter` given), already zero (Adam zeroes them once read)
// with the loss zeroed by the batch setup, and the loss kernel advances the
// step counter.  With `side`, the weight gradients of layers 3 and 2 run on
// the side stream, beside dH2 and dH1 (ordinary launches there: the
// programmatic launches of ex.pdl chain kernels of one stream).
void mlp_loss_grad(const Exec& ex, Mlp& net, MlpWork& W, const __half* X, const uint32_t* rowmap, int n,
                   SideStream* side = nullptr, unsigned long long* counter = nullptr) {
  const int rows = 2 * n;
  const float inv = 1.f / kLossScale;
  mlp_forward(ex, net, W, X, rowmap, rows);
  if (!counter) {
    SVDAG_CUDA(cudaMemsetAsync(W.loss.get(), 0, 4, ex.stream));
    SVDAG_CUDA(cudaMemsetAsync(net.g.get(), 0, 4 * Mlp::total(), ex.stream));
  }
  SVDAG_LAUNCH(ex, k_pair_loss, grid_for(ex, n, 8), 256, 0, W.E.get(), W.t.get(), n, W.dE.get(), W.loss.get(),
               counter);
  Exec sx = ex;
  if (side) {
    sx.stream = side->stream;
    sx.pdl = false;
  }
  GemmOpts wg;  // weight gradients: split-K partial sums into the zeroed gradients, unscaled
  wg.alpha = inv;
  wg.zeroed = true;
  GemmOpts hg;  // hidden gradients: ReLU mask, bias gradient as column sums
  hg.colsum_scale = inv;
  // layer 3: dW3 (side) beside dH2
  if (side) {
    SVDAG_CUDA(cudaEventRecord(side->fork[0], ex.stream));
    SVDAG_CUDA(cudaStreamWaitEvent(side->stream, side->fork[0], 0));
  }
  gemm_tc<true, false, float>(sx, W.H2.get(), W.dE.get(), net.gp[4], kH, kOut, rows, wg);
  hg.mask = W.H2.get();
  hg.colsum = net.gp[3];
  gemm_tc<false, true, __half>(ex, W.dE.get(), net.h[4], W.dH2.get(), rows, kH, kOut, hg);
  // layer 2: dW2 (side) beside dH1
  if (side) {
    SVDAG_CUDA(cudaEventRecord(side->fork[1], ex.stream));
    SVDAG_CUDA(cudaStreamWaitEvent(side->stream, side->fork[1], 0));
  }
  gemm_tc<true, false, float>(sx, W.H1.get(), W.dH2.get(), net.gp[2], kH, kH, rows, wg);
  hg.mask = W.H1.get();
  hg.colsum = net.gp[1];
  gemm_tc<false, true, __half>(ex, W.dH2.get(), net.h[2], W.dH1.get(), rows, kH, kH, hg);
  // layer 1
  wg.rowmap = rowmap;
  gemm_tc<true, false, float>(ex, X, W.dH1.get(), net.gp[0], kIn, kH, rows, wg);
  if (side) {
    SVDAG_CUDA(cudaEventRecord(side->join, side->stream));
    SVDAG_CUDA(cudaStreamWaitEvent(ex.stream, side->join, 0));
  }
}

void mlp_adam(const Exec& ex, Mlp& net, float lr) {
  const float b1 = 0.9f, b2 = 0.999f;
  ++net.step;
  const float c1 = 1.f - std::pow(b1, float(net.step)), c2 = 1.f - std::pow(b2, float(net.step));
  const size_t n = Mlp::total();
  SVDAG_LAUNCH(ex, k_adam, grid_for(ex, n, 256), 256, 0, net.w.get(), net.wh.get(), net.g.get(), net.m.get(),
               net.v.get(), n, lr, b1, b2, c1, c2);
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
    // features of all candidates (fp16)
    DBuf<__half> X(size_t(n) * kIn, st);
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
    DBuf<uint32_t> d_order(n, st), d_end(n, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_order.get(), order.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    SVDAG_CUDA(cudaMemcpyAsync(d_end.get(), band_end.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    if (!trained) {
      if (train) {
        const auto t0 = std::chrono::steady_clock::now();
        fit(c, S, X, d_order, d_end, cfg);
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
      mlp_forward(ex, net, work, X.get() + size_t(r0) * kIn, nullptr, rows);
      SVDAG_CUDA(cudaMemcpyAsync(E.get() + size_t(r0) * kOut, work.E.get(), 4ull * rows * kOut, cudaMemcpyDeviceToDevice, st));
    }
    // top-k per candidate within its band
    std::vector<uint64_t> off(n + 1, 0);
    for (uint32_t p = 0; p < n; ++p) off[p + 1] = off[p] + std::min<uint32_t>(cfg.top_k, band_end[p] - p - 1);
    DBuf<uint64_t> d_off(n + 1, st);
    SVDAG_CUDA(cudaMemcpyAsync(d_off.get(), off.data(), 8ull * (n + 1), cudaMemcpyHostToDevice, st));
    pairs.alloc(off[n] ? off[n] : 1, st);
    if (off[n])
      SVDAG_LAUNCH(ex, k_topk_band, std::min<uint32_t>(n, 152u * 8), 256, 0, E.get(), d_order.get(), d_end.get(), n,
                   int(cfg.top_k), pairs.get(), d_off.get());
    (void)lev;
    return off[n];
  }

  // Training pairs: half within the bands (near pairs), half uniform, drawn
  // on the device (k_sample_pairs), rounded up to whole batches of
  // cfg.train_batch pairs; their exact targets (k_pair_target).  One training
  // step -- batch setup, forward, loss, backward with the fused bias and
  // ReLU gradients (the weight gradients on a parallel branch), Adam, step
  // counter -- is captured once as a CUDA graph and replayed for every batch
  // of every epoch (the batch and the Adam step come from a device counter),
  // without host synchronisation.
  void fit(Ctx& c, const LevelSubtrees& S, const DBuf<__half>& X, const DBuf<uint32_t>& d_order,
           const DBuf<uint32_t>& d_end, const LossyConfig& cfg) {
    const Exec& ex = c.ex;
    const cudaStream_t st = c.stream;
    const uint32_t n = S.n;
    const int B = int(cfg.train_batch);
    const uint64_t batches = std::max<uint64_t>(1, (std::max<uint64_t>(1024, cfg.train_pairs) + B - 1) / B);
    const uint64_t np = batches * B;
    DBuf<uint2> pairs(np, st);
    DBuf<uint32_t> rows_all(2 * np, st), rows(2 * B, st);
    DBuf<float> target(np, st);
    DBuf<unsigned long long> counter(1, st);
    SVDAG_LAUNCH(ex, k_sample_pairs, grid_for(ex, np, 256), 256, 0, d_order.get(), d_end.get(), n, np, B,
                 cfg.seed * 0x9E3779B97F4A7C15ull + 7, pairs.get(), rows_all.get());
    SVDAG_LAUNCH(ex, k_pair_target, grid_for(ex, np, 8, 16), 256, 0, S.bytes.get(), S.words, S.pop.get(), pairs.get(),
                 np, target.get());
    SVDAG_CUDA(cudaMemsetAsync(counter.get(), 0, 8, st));
    SVDAG_CUDA(cudaMemsetAsync(net.g.get(), 0, 4 * Mlp::total(), st));  // then zeroed by Adam every step
    work.ensure(2 * B, st);
    Exec gx = ex;
    gx.prof = nullptr;  // no per-launch timing events inside a captured graph
    // programmatic launches between the step's consecutive kernels on the
    // stream (each waits for its predecessor with pdl_wait); the batch setup
    // (the graph's first node) and Adam (after the side stream's join) launch
    // ordinarily
    Exec gp = gx;
    gp.pdl = true;
    SideStream side;
    side.create();
    const uint64_t l0 = gx.launches ? *gx.launches : 0;
    cudaGraph_t graph = nullptr;
    SVDAG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      SVDAG_LAUNCH(gx, k_batch_setup, 32, 256, 0, counter.get(), uint32_t(batches), B, rows_all.get(), target.get(),
                   rows.get(), work.t.get(), work.loss.get());
      mlp_loss_grad(gp, net, work, X.get(), rows.get(), B, &side, counter.get());
      SVDAG_LAUNCH(gx, k_adam_dev, grid_for(gx, Mlp::total(), 256), 256, 0, net.w.get(), net.wh.get(), net.g.get(),
                   net.m.get(), net.v.get(), Mlp::total(), cfg.lr, 0.9f, 0.999f, counter.get());
    } catch (...) {
      cudaStreamEndCapture(st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    SVDAG_CUDA(cudaStreamEndCapture(st, &graph));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ri = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    SVDAG_CUDA(ri);
    const uint64_t steps = batches * std::max(1u, cfg.epochs);
    cudaError_t rl = cudaSuccess;
    for (uint64_t i = 0; i < steps && rl == cudaSuccess; ++i) rl = cudaGraphLaunch(exec, st);
    // the replays run the step's kernels again (counted once at capture)
    if (gx.launches) *gx.launches += (steps - 1) * (*gx.launches - l0);
    const float loss = rl == cudaSuccess ? read_scalar(ex, work.loss.get()) : 0.f;
    cudaGraphExecDestroy(exec);
    SVDAG_CUDA(rl);
    last_loss = loss;
    net.step += int(steps);
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
  if (cudaMemcpyAsync(m->h.net.w.get(), host, 4 * svdag::Mlp::total(), cudaMemcpyHostToDevice, m->h.stream) != cudaSuccess)
    return SVDAG_ERR_CUDA;
  try {
    m->h.net.refresh_half(m->h.stream);
  } catch (const svdag::Error& e) {
    return e.code;
  }
  if (cudaStreamSynchronize(m->h.stream) != cudaSuccess) return SVDAG_ERR_CUDA;
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
    const size_t cnt = size_t(n) * svdag::kIn;
    H.work.xin.alloc(2 * cnt, H.stream);
    SVDAG_CUDA(cudaMemcpyAsync(H.work.xin.get(), x_a, 4 * cnt, cudaMemcpyHostToDevice, H.stream));
    SVDAG_CUDA(cudaMemcpyAsync(H.work.xin.get() + cnt, x_b, 4 * cnt, cudaMemcpyHostToDevice, H.stream));
    SVDAG_LAUNCH(H.ex, svdag::k_to_half, svdag::grid_for(H.ex, 2 * cnt, 256), 256, 0, H.work.xin.get(), 2 * cnt,
                 H.work.X.get());
    SVDAG_CUDA(cudaMemcpyAsync(H.work.t.get(), t, 4ull * n, cudaMemcpyHostToDevice, H.stream));
    svdag::mlp_loss_grad(H.ex, H.net, H.work, H.work.X.get(), nullptr, int(n));
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
    const size_t cnt = size_t(n) * svdag::kIn;
    H.work.xin.alloc(cnt, H.stream);
    SVDAG_CUDA(cudaMemcpyAsync(H.work.xin.get(), x, 4 * cnt, cudaMemcpyHostToDevice, H.stream));
    SVDAG_LAUNCH(H.ex, svdag::k_to_half, svdag::grid_for(H.ex, cnt, 256), 256, 0, H.work.xin.get(), cnt,
                 H.work.X.get());
    svdag::mlp_forward(H.ex, H.net, H.work, H.work.X.get(), nullptr, int(n));
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
    cfg.top_k = p->top_k ? p->top_k : 384;
    cfg.train_pairs = p->train_pairs ? p->train_pairs : 2000000;
    cfg.epochs = p->train_epochs ? p->train_epochs : 1;
    cfg.seed = p->seed;
    cfg.train_batch = p->train_batch ? p->train_batch : 8192;
    cfg.lr = p->train_lr > 0.f ? p->train_lr : 2e-3f;
    if (cfg.top_k > 512) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "lossy: top_k above 512");
    if (cfg.train_batch % 64 || cfg.train_batch < 256 || cfg.train_batch > 65536)
      throw svdag::Error(SVDAG_ERR_INVALID_ARG, "lossy: train_batch must be a multiple of 64 in [256, 65536]");
    if (!(cfg.lr < 1.f)) throw svdag::Error(SVDAG_ERR_INVALID_ARG, "lossy: train_lr must be below 1");
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
