// wotg_onthefly.cu — cost tiles recomputed on the tensor cores (tcgen05), sm_103a.
//
// The squared-Euclidean cost of the reference (wot/ot/ot_model.py:249-252) is
//   C_ij = |x_i|^2 + |y_j|^2 - 2 x_i . y_j,
// whose only dense contraction, the cross term x_i . y_j over the 30-50 PCA
// dimensions, runs here as an FP16 split-precision MMA (x = hi + lo, three
// products hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM).
#include <algorithm>

#include "wotg_common.cuh"
#include "wotg_onthefly.cuh"
#include "wotg_tc.cuh"

namespace wotg {

constexpr uint32_t kTcWaitTries = 1u << 22;

// ---------------------------------------------------------------------------
// Self-test of the MMA path: D (128 x 128, FP32) = A (128 x 32) B (128 x 32)^T
// with `terms` = 1 (hi.hi) or 3 (hi.hi + hi.lo + lo.hi). One CTA of 128 threads.
// The descriptor strides are parameters so that a test can check the layout
// convention; any (lbo, sbo) <= 512 keeps every operand read inside the 32 KB
// of staged tiles. A timed-out wait sets *err = 1 and skips the TMEM reads.
// ---------------------------------------------------------------------------
constexpr int kSelfM = 128, kSelfN = 128, kSelfK = 32;

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A,
                                                          const float* __restrict__ B, float* __restrict__ D,
                                                          uint32_t lbo, uint32_t sbo, int terms, int* err) {
  __shared__ __align__(1024) __half sA[2][kSelfM * kSelfK];
  __shared__ __align__(1024) __half sB[2][kSelfN * kSelfK];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < kSelfM * kSelfK; idx += 128) {
    const int r = idx / kSelfK, k = idx % kSelfK;
    const uint32_t off = tc::core_offset(r, k, kSelfK) >> 1;
    __half h, l;
    tc::split_f16(A[idx], h, l);
    sA[0][off] = h;
    sA[1][off] = l;
    tc::split_f16(B[idx], h, l);
    sB[0][off] = h;
    sB[1][off] = l;
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, 128);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_f16_f32(kSelfM, kSelfN);
    const uint32_t a0 = tc::smem_u32(sA[0]), a1 = tc::smem_u32(sA[1]);
    const uint32_t b0 = tc::smem_u32(sB[0]), b1 = tc::smem_u32(sB[1]);
    uint32_t acc = 0;
    for (int s = 0; s < kSelfK / 16; ++s) {
      const uint32_t ko = s * 2 * tc::kCoreLbo;
      tc::mma_f16(tmem, tc::smem_desc(a0 + ko, lbo, sbo), tc::smem_desc(b0 + ko, lbo, sbo), idesc, acc);
      acc = 1;
      if (terms == 3) {
        tc::mma_f16(tmem, tc::smem_desc(a0 + ko, lbo, sbo), tc::smem_desc(b1 + ko, lbo, sbo), idesc, 1);
        tc::mma_f16(tmem, tc::smem_desc(a1 + ko, lbo, sbo), tc::smem_desc(b0 + ko, lbo, sbo), idesc, 1);
      }
    }
    tc::mma_commit(&bar);
  }
  const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(&bar, 0, kTcWaitTries));
  if (!ok && lane == 0) atomicExch(err, 1);
  tc::fence_after_sync();
  if (ok) {
    for (int c = 0; c < kSelfN; c += 32) {
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      tc::tmem_wait_ld();
#pragma unroll
      for (int t = 0; t < 32; ++t) D[(warp * 32 + lane) * kSelfN + c + t] = v[t];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}


// ---------------------------------------------------------------------------
// Point packing (once per solve): each 128-point tile is stored as its FP16 hi
// block then its lo block, K-major core-matrix layout with KP halfs per row
// (dimensions beyond d and points beyond n are zero), plus FP64 |x|^2.
// ---------------------------------------------------------------------------
__global__ void tc_pack_kernel(const float* __restrict__ X, int64_t n, int64_t ldx, int d, int kp,
                               __half* __restrict__ tiles, double* __restrict__ norm) {
  const int64_t ntiles = (n + 127) / 128;
  const int64_t total = ntiles * 128 * kp;
  const int64_t tile_halfs = (int64_t)2 * 128 * kp;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / kp;
    const int k = (int)(idx % kp);
    const float x = (i < n && k < d) ? X[i * ldx + k] : 0.f;
    __half h, l;
    tc::split_f16(x, h, l);
    __half* tile = tiles + (i / 128) * tile_halfs;
    const uint32_t off = tc::core_offset((int)(i % 128), k, kp) >> 1;
    tile[off] = h;
    tile[128 * kp + off] = l;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < d; ++k) {
      const double x = X[i * ldx + k];
      s += x * x;
    }
    norm[i] = s;
  }
}

// ---------------------------------------------------------------------------
// On-the-fly half-step: for each point p_i of a 128-point row tile and the
// column tiles [q0, q1) of the other set, the base-2 log-sum-exp partial
//   (m_i, s_i):  s_i 2^m_i = sum_j 2^(bias_j + gamma (p_i . q_j))
// where p . q comes from the FP16 split-precision MMA (hi.hi + hi.lo + lo.hi,
// FP32 accumulation in TMEM). The row term of the exponent (-kappa |p_i|^2)
// and the FP64 merge of the partials are applied by the caller.
//
// CTA: 256 threads = 2 warpgroups; TMEM accumulator 128 lanes x 128 columns;
// warpgroup g reads columns [64 g, 64 g + 64) of every row. The A tile is loaded
// once; B tiles and their 128 biases are double-buffered through bulk
// asynchronous copies so that the copy of tile k+1 overlaps tile k. Every wait
// is bounded: on a timeout the CTA sets *err, stops, waits (bounded) for what it
// issued and frees its TMEM.
// ---------------------------------------------------------------------------
template <int KP>
struct TcSmem {
  static constexpr uint32_t kHalfBytes = 128u * KP * 2u;      // one of hi / lo
  static constexpr uint32_t kTileBytes = 2u * kHalfBytes;      // hi + lo
  static constexpr uint32_t kA = 0;
  static constexpr uint32_t kB = kTileBytes;                   // 2 buffers
  static constexpr uint32_t kBias = kB + 2 * kTileBytes;       // 2 x 128 floats
  static constexpr uint32_t kBar = kBias + 2 * 512;            // 3 mbarriers + TMEM slot
  static constexpr uint32_t kMerge = kBar + 64;                // 128 float2
  static constexpr uint32_t kBytes = kMerge + 128 * 8;
  static constexpr uint32_t kAlloc = kBytes + 1024;            // slack for 1024-byte alignment
};

template <int KP>
__global__ void __launch_bounds__(256, 3) lse_tc_kernel(const __half* __restrict__ Pt, const __half* __restrict__ Qt,
                                                        const float* __restrict__ bias, int nqt, int nsplit,
                                                        float gamma, float2* __restrict__ part, int64_t n_pad,
                                                        int* __restrict__ err) {
  using L = TcSmem<KP>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~uintptr_t(1023));
  uint64_t* bar_ld = reinterpret_cast<uint64_t*>(smem + L::kBar);  // [2]
  uint64_t* bar_mma = bar_ld + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_ld + 3);
  float2* merge = reinterpret_cast<float2*>(smem + L::kMerge);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = warp >> 2, wq = warp & 3;
  const int t = blockIdx.y, sp = blockIdx.x;
  const int q0 = (int)((int64_t)sp * nqt / nsplit);
  const int q1 = (int)((int64_t)(sp + 1) * nqt / nsplit);
  const int ntiles = q1 - q0;
  const int64_t tile_halfs = (int64_t)2 * 128 * KP;

  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, 128);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar_ld[0], 1);
    tc::mbar_init(&bar_ld[1], 1);
    tc::mbar_init(bar_mma, 1);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sA = tc::smem_u32(smem + L::kA);
  const uint32_t sB = tc::smem_u32(smem + L::kB);
  const uint32_t sBias = tc::smem_u32(smem + L::kBias);
  if (tid == 0 && ntiles > 0) {
    tc::mbar_expect_tx(&bar_ld[0], 2 * L::kTileBytes + 512);
    tc::bulk_g2s(sA, Pt + (int64_t)t * tile_halfs, L::kTileBytes, &bar_ld[0]);
    tc::bulk_g2s(sB, Qt + (int64_t)q0 * tile_halfs, L::kTileBytes, &bar_ld[0]);
    tc::bulk_g2s(sBias, bias + (int64_t)q0 * 128, 512, &bar_ld[0]);
  }
  constexpr uint32_t idesc = tc::idesc_f16_f32(128, 128);
  constexpr uint32_t sbo = KP * 16;
  float m = kNegBig, s = 0.f;
  bool ok = true;
  bool next_issued = false;
  int k = 0;
  for (; k < ntiles; ++k) {
    const int buf = k & 1;
    bool good = tc::mbar_wait(&bar_ld[buf], (uint32_t)((k >> 1) & 1), kTcWaitTries);
    next_issued = false;
    if (tid == 0) {
      if (k + 1 < ntiles) {
        const uint32_t nb = (uint32_t)(buf ^ 1);
        tc::mbar_expect_tx(&bar_ld[nb], L::kTileBytes + 512);
        tc::bulk_g2s(sB + nb * L::kTileBytes, Qt + (int64_t)(q0 + k + 1) * tile_halfs, L::kTileBytes, &bar_ld[nb]);
        tc::bulk_g2s(sBias + nb * 512, bias + (int64_t)(q0 + k + 1) * 128, 512, &bar_ld[nb]);
      }
      tc::fence_after_sync();
      const uint32_t b0 = sB + (uint32_t)buf * L::kTileBytes;
#pragma unroll
      for (int st = 0; st < KP / 16; ++st) {
        const uint32_t ko = (uint32_t)st * 2u * tc::kCoreLbo;
        const uint64_t ahi = tc::smem_desc(sA + ko, tc::kCoreLbo, sbo);
        const uint64_t alo = tc::smem_desc(sA + L::kHalfBytes + ko, tc::kCoreLbo, sbo);
        const uint64_t bhi = tc::smem_desc(b0 + ko, tc::kCoreLbo, sbo);
        const uint64_t blo = tc::smem_desc(b0 + L::kHalfBytes + ko, tc::kCoreLbo, sbo);
        tc::mma_f16(tmem, ahi, bhi, idesc, st > 0 ? 1u : 0u);
        tc::mma_f16(tmem, ahi, blo, idesc, 1u);
        tc::mma_f16(tmem, alo, bhi, idesc, 1u);
      }
      tc::mma_commit(bar_mma);
    }
    next_issued = k + 1 < ntiles;
    good = tc::mbar_wait(bar_mma, (uint32_t)(k & 1), kTcWaitTries) && good;
    good = __all_sync(0xffffffffu, good);
    tc::fence_after_sync();
    if (good) {
      const float* bt = reinterpret_cast<const float*>(smem + L::kBias + buf * 512) + 64 * wg;
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(64 * wg + 32 * h), v);
        tc::tmem_wait_ld();
        float mx = kNegBig;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          v[c] = fmaf(gamma, v[c], bt[32 * h + c]);
          mx = fmaxf(mx, v[c]);
        }
        const float mn = fmaxf(m, mx);
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 32; ++c) acc += ex2(v[c] - mn);
        s = s * ex2(m - mn) + acc;
        m = mn;
      }
    }
    tc::fence_before_sync();
    ok = __syncthreads_and(good) != 0;
    if (!ok) break;
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    // bounded waits for the copies / MMAs this CTA issued, then release TMEM
    tc::mbar_wait(&bar_ld[k & 1], (uint32_t)((k >> 1) & 1), kTcWaitTries);
    if (next_issued) tc::mbar_wait(&bar_ld[(k & 1) ^ 1], (uint32_t)(((k + 1) >> 1) & 1), kTcWaitTries);
    tc::mbar_wait(bar_mma, (uint32_t)(k & 1), kTcWaitTries);
  } else {
    const int row = 32 * wq + lane;
    if (wg == 1) merge[row] = make_float2(m, s);
    __syncthreads();
    if (wg == 0) {
      const float2 o = merge[row];
      lse_merge(m, s, o.x, o.y);
      part[(int64_t)sp * n_pad + (int64_t)t * 128 + row] = make_float2(m, s);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

int tc_pack_points(const float* X, int64_t n, int64_t ldx, int d, int kp, __half* tiles, double* norm,
                   cudaStream_t st) {
  const int64_t total = (n + 127) / 128 * 128 * kp;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 8);
  tc_pack_kernel<<<grid, 256, 0, st>>>(X, n, ldx, d, kp, tiles, norm);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

template <int KP>
static cudaError_t tc_set_smem_attr() {
  static cudaError_t once = cudaFuncSetAttribute(lse_tc_kernel<KP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)TcSmem<KP>::kAlloc);
  return once;
}

int tc_ctas_per_sm(int kp) {
  int n = 0;
  if (kp == 32) {
    if (tc_set_smem_attr<32>() != cudaSuccess) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lse_tc_kernel<32>, 256, TcSmem<32>::kAlloc) != cudaSuccess)
      return 1;
  } else {
    if (tc_set_smem_attr<64>() != cudaSuccess) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lse_tc_kernel<64>, 256, TcSmem<64>::kAlloc) != cudaSuccess)
      return 1;
  }
  return n > 0 ? n : 1;
}

int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nqt, const float* bias, int kp,
                  float gamma, int nsplit, float2* part, int64_t n_pad, int* err, cudaStream_t st) {
  dim3 grid((unsigned)nsplit, (unsigned)n_ptiles);
  if (kp == 32) {
    WOTG_CUDA(tc_set_smem_attr<32>());
    lse_tc_kernel<32><<<grid, 256, TcSmem<32>::kAlloc, st>>>(Pt, Qt, bias, nqt, nsplit, gamma, part, n_pad, err);
  } else if (kp == 64) {
    WOTG_CUDA(tc_set_smem_attr<64>());
    lse_tc_kernel<64><<<grid, 256, TcSmem<64>::kAlloc, st>>>(Pt, Qt, bias, nqt, nsplit, gamma, part, n_pad, err);
  } else {
    return WOTG_BADARG;
  }
  WOTG_LAUNCHED();
  return WOTG_OK;
}

}  // namespace wotg

using namespace wotg;

extern "C" int wotg_tc_selftest(const float* A, const float* B, float* D, uint32_t lbo, uint32_t sbo,
                                int32_t terms, int32_t* err, void* stream) {
  if (!A || !B || !D || !err || lbo > 512 || sbo > 512 || (lbo & 15) || (sbo & 15) || (terms != 1 && terms != 3))
    return WOTG_BADARG;
  tc_selftest_kernel<<<1, 128, 0, (cudaStream_t)stream>>>(A, B, D, lbo, sbo, terms, err);
  WOTG_LAUNCHED();
  return WOTG_OK;
}
