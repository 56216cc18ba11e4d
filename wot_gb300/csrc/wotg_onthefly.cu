// wotg_onthefly.cu — cost tiles recomputed on the tensor cores (tcgen05), sm_103a.
//
// The squared-Euclidean cost of the reference (wot/ot/ot_model.py:249-252) is
//   C_ij = |x_i|^2 + |y_j|^2 - 2 x_i . y_j,
// whose only dense contraction, the cross term x_i . y_j over the 30-50 PCA
// dimensions, runs here as an FP16 split-precision MMA (x = hi + lo, three
// products hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM).
#include <algorithm>
#include <cmath>

#include "wotg_common.cuh"
#include "wotg_onthefly.cuh"
#include "wotg_tc.cuh"

namespace wotg {

constexpr uint32_t kTcWaitTries = kTcDefaultWaitTries;  // x up to 1 us per try: about 4 s

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
// Point packing. Each 128-point tile is stored as its FP16 hi block then its
// lo block, K-major core-matrix layout with KP halfs per row (x = hi + lo).
// The MMA computes, per (row point p, column point q), the base-2 exponent
//   sum_k a_k b_k = gamma (p . q) + bias_q
// from two packings of the points:
//   row form     a = [gamma x_1 .. gamma x_d, 1, 1, 0 ...]   (repacked per epsilon)
//   column form  b = [x_1 .. x_d, beta1_q, beta2_q, 0 ...]   (bias columns per half-step)
// where beta1 + beta2 carries the FP64 bias to ~44 bits (beta1 = fp32(bias),
// beta2 = the remainder after beta1's hi/lo split). Points beyond n are zero,
// and in the column form carry the bias of weight 0 (beta1 = -60000) from the
// start: the bias columns of real points are rewritten per half-step, those of
// the padding never.
// ---------------------------------------------------------------------------
__global__ void tc_pack_kernel(const float* __restrict__ X, int64_t n, int64_t ldx, int d, int kp, float scale,
                               int row_form, __half* __restrict__ tiles, double* __restrict__ norm) {
  const int64_t ntiles = (n + 127) / 128;
  const int64_t total = ntiles * 128 * kp;
  const int64_t tile_halfs = (int64_t)2 * 128 * kp;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / kp;
    const int k = (int)(idx % kp);
    float x = 0.f;
    if (k < d) x = i < n ? scale * X[i * ldx + k] : 0.f;
    else if (row_form && k < d + 2) x = 1.f;
    else if (!row_form && i >= n && k == d) x = -60000.f;
    __half h, l;
    tc::split_f16(x, h, l);
    __half* tile = tiles + (i / 128) * tile_halfs;
    const uint32_t off = tc::core_offset((int)(i % 128), k, kp) >> 1;
    tile[off] = h;
    tile[128 * kp + off] = l;
  }
  if (norm) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) {
        const double x = X[i * ldx + k];
        s += x * x;
      }
      norm[i] = s;
    }
  }
}

// Column-form bias columns of every point (and of the padding points):
//   bias_q = (pot_q / eps + lsc_q) log2 e - kappa2 |q|^2      (lsc may be null: 0)
// (-inf -> a large negative finite value, i.e. weight 0; NaN / +inf -> NaN so
// that non-finite potentials propagate like in the materialised form).
__global__ void tc_bias_pack_kernel(int64_t n, int64_t n_pad, const double* __restrict__ pot,
                                    const double* __restrict__ lsc, const double* __restrict__ norm,
                                    double inv_eps, double kappa2d, int d, int kp, __half* __restrict__ tiles) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += (int64_t)gridDim.x * blockDim.x) {
    const double beta = i < n ? (pot[i] * inv_eps + (lsc ? lsc[i] : 0.0)) * kLog2e - kappa2d * norm[i] : -INFINITY;
    tc_write_bias(i, beta, d, kp, tiles);
  }
}

// ---------------------------------------------------------------------------
// On-the-fly half-step: base-2 log-sum-exp partials
//   (m, s):  s 2^m = sum_j 2^(bias_j + gamma (p_i . q_j))
// over 128-point tiles of the other set. The whole exponent comes out of the
// FP16 split-precision MMA (hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM)
// of the row-form and column-form packings. The row term of the exponent
// (-kappa |p_i|^2) and the FP64 merge of the partials are applied by the caller.
//
// Persistent schedule: the n_pt x nq (row tile, column tile) pairs are walked
// row-major and cut into gridDim.x contiguous, equal stretches, one per CTA. A
// stretch covers one or more row tiles ("segments"); at the end of each
// segment the CTA writes, for every row of that row tile and each of the four
// 32-column quarters, one partial at part[((cta + tile) * 128 + row) * 4 + quarter].
// Along the walk (cta, tile) only ever steps up, so cta + tile indexes every
// (CTA, row tile) segment uniquely.
//
// Warp roles (10 warps, two CTAs per SM):
//   warp 0      producer: bulk asynchronous copies of A tiles (one per segment,
//               kABuf buffers) and B tiles (a kStages-deep ring);
//   warp 1      MMA issuer: 3 split-precision MMAs per 16-column step into one
//               of two 128 x 128 FP32 TMEM accumulators; owns the TMEM allocation;
//   warps 2-9   epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 and the
//               64 columns of half (w - 2) / 4 and folds them into a running
//               (max, sum).
// mbarriers hand buffers between roles (full / empty per B stage, per A buffer
// and per accumulator). Every wait is bounded (wait_tries tries of up to 1 us):
// a role that times out sets *err and a shared abort flag and stops; the
// producer also stops at its next wait once the flag is set, and the other
// roles' waits run out in turn (the hot waits of the MMA issuer and the
// epilogue do not poll the flag). Before the CTA frees TMEM and exits,
// whether it completed or gave up, the producer waits (with the full budget)
// for every bulk copy it issued to land, and the MMA issuer commits once more
// and waits until every MMA it issued has completed, so that no asynchronous
// copy or product is still writing shared memory or TMEM when they are freed.
// ---------------------------------------------------------------------------
constexpr int kTcStages = 4;
constexpr int kTcAcc = 2;            // TMEM accumulators (128 columns each)
constexpr int kTcEpiWarps = 8;       // 4 x kTcParts: each reads one lane quarter x 128 / kTcParts columns
constexpr int kTcParts = kTcEpiWarps / 4;
constexpr int kTcColsPerWarp = 128 / kTcParts;
constexpr int kTcCtasPerSm = 2;
constexpr int kTcThreads = 32 * (2 + kTcEpiWarps);

template <int KP>
struct TcSmem {
  static constexpr uint32_t kHalfBytes = 128u * KP * 2u;      // one of hi / lo
  static constexpr uint32_t kTileBytes = 2u * kHalfBytes;      // packed 128-point tile (hi + lo)
  // Two CTAs per SM in 96 KB each: 32 columns double-buffer the row tile (A) and
  // keep a 4-deep ring of column tiles (B); 64 columns single-buffer A (it
  // changes only at the few row-tile boundaries of a CTA's stretch) and keep 2 B stages.
  static constexpr int kStages = KP == 32 ? kTcStages : 2;     // B ring depth
  static constexpr int kABuf = KP == 32 ? 2 : 1;               // A buffers
  static constexpr uint32_t kA = 0;                            // kABuf buffers
  static constexpr uint32_t kB = kABuf * kTileBytes;           // kStages buffers
  static constexpr uint32_t kBar = kB + kStages * kTileBytes;
  // barriers: full[S], empty[S], a_full[kABuf], a_empty[kABuf], acc_full[kTcAcc], acc_empty[kTcAcc],
  // drain; then the TMEM slot and the abort flag
  static constexpr uint32_t kBytes = kBar + 8 * (2 * kStages + 2 * kABuf + 2 * kTcAcc + 1) + 16;
  static constexpr uint32_t kAlloc = kBytes + 1024;            // slack for 1024-byte alignment
  static constexpr uint32_t kTmemCols = 128 * kTcAcc;
};

template <int KP>
__device__ __forceinline__ void tc_issue_mma(uint32_t tmem_d, uint32_t sAt, uint32_t sBt) {
  using L = TcSmem<KP>;
  constexpr uint32_t idesc = tc::idesc_f16_f32(128, 128);
  constexpr uint32_t sbo = KP * 16;
#pragma unroll
  for (int st = 0; st < KP / 16; ++st) {
    const uint32_t ko = (uint32_t)st * 2u * tc::kCoreLbo;
    const uint64_t ahi = tc::smem_desc(sAt + ko, tc::kCoreLbo, sbo);
    const uint64_t alo = tc::smem_desc(sAt + L::kHalfBytes + ko, tc::kCoreLbo, sbo);
    const uint64_t bhi = tc::smem_desc(sBt + ko, tc::kCoreLbo, sbo);
    const uint64_t blo = tc::smem_desc(sBt + L::kHalfBytes + ko, tc::kCoreLbo, sbo);
    tc::mma_f16(tmem_d, ahi, bhi, idesc, st > 0 ? 1u : 0u);
    tc::mma_f16(tmem_d, ahi, blo, idesc, 1u);
    tc::mma_f16(tmem_d, alo, bhi, idesc, 1u);
  }
}

// Online LSE of 32 exponents d[c] into (m, s): packed FP32x2 arithmetic and
// tree reductions.
__device__ __forceinline__ void lse32(const float (&d)[32], float& m, float& s) {
  float2 x[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) x[c] = make_float2(d[2 * c], d[2 * c + 1]);
  float mx[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) mx[c] = fmaxf(fmaxf(x[2 * c].x, x[2 * c].y), fmaxf(x[2 * c + 1].x, x[2 * c + 1].y));
#pragma unroll
  for (int w = 4; w >= 1; w >>= 1)
#pragma unroll
    for (int c = 0; c < w; ++c) mx[c] = fmaxf(mx[c], mx[c + w]);
  const float mn = fmaxf(m, mx[0]);
  const float2 neg = make_float2(-mn, -mn);
  float2 e[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float2 z = __fadd2_rn(x[c], neg);
    e[c] = make_float2(ex2(z.x), ex2(z.y));
  }
#pragma unroll
  for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
    for (int c = 0; c < w; ++c) e[c] = __fadd2_rn(e[c], e[c + w]);
  s = s * ex2(m - mn) + (e[0].x + e[0].y);
  m = mn;
}

// Sums of 2^(d[c] - o) of 32 exponents into four FP32x2 accumulators
// (speculative form: o is the row's log-sum-exp from the previous half-step, so
// no running maximum is needed). kFmaPairs of the 16 pairs take their 2^z on
// the FMA pipe (ex2_fma2), the rest on the SFU: the epilogue's SFU, TMEM-load
// and tensor work then overlap better (4 of 32 measured best; more moves the
// bound to instruction issue).
constexpr int kFmaPairs = 2;
__device__ __forceinline__ void sum32_off(const float (&d)[32], float o, float2 (&acc)[4]) {
  const float2 neg = make_float2(-o, -o);
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float2 z = __fadd2_rn(make_float2(d[2 * c], d[2 * c + 1]), neg);
    const float2 e = c < kFmaPairs ? ex2_fma2(z) : make_float2(ex2(z.x), ex2(z.y));
    acc[c & 3] = __fadd2_rn(acc[c & 3], e);
  }
}

// Weighted sums of 32 exponents for up to NPOP populations at once (the
// population form of the epilogue): one exp2 per element against the running
// maximum m, then s[k] += 2^(d - m) w[k][col] for every population k, the
// weights w (npop rows of ldw floats, 16-byte aligned) read as warp-uniform
// 128-bit loads. The sums are rescaled when the maximum moves.
template <int NPOP>
__device__ __forceinline__ void multi32(const float (&d)[32], const float* __restrict__ w, int npop, int ldw,
                                        int col0, float& m, float (&s)[NPOP]) {
  float mx = d[0];
#pragma unroll
  for (int c = 1; c < 32; ++c) mx = fmaxf(mx, d[c]);
  const float mn = fmaxf(m, mx);
  const float r = ex2(m - mn);
#pragma unroll
  for (int k = 0; k < NPOP; ++k) s[k] *= r;
  m = mn;
#pragma unroll
  for (int c = 0; c < 32; c += 4) {
    const float e0 = ex2(d[c] - mn), e1 = ex2(d[c + 1] - mn), e2 = ex2(d[c + 2] - mn), e3 = ex2(d[c + 3] - mn);
#pragma unroll
    for (int k = 0; k < NPOP; ++k) {
      if (k < npop) {
        const float4 pw = __ldg(reinterpret_cast<const float4*>(w + (int64_t)k * ldw + col0 + c));
        s[k] = fmaf(e0, pw.x, fmaf(e1, pw.y, fmaf(e2, pw.z, fmaf(e3, pw.w, s[k]))));
      }
    }
  }
}

// NPOP = 0: the log-sum-exp half-step (partials (m, s) in part). NPOP > 0: the
// population form, npop <= NPOP weighted sums per row (maxima in part[].x,
// sums in psum[slot * NPOP + k]) with the population weights popw.
template <int KP, int NPOP>
__global__ void __launch_bounds__(kTcThreads, kTcCtasPerSm) lse_tc_kernel(const __half* __restrict__ Pt,
                                                               const __half* __restrict__ Qt,
                                                               int n_pt, int nq, float2* __restrict__ part,
                                                               const float* __restrict__ off,
                                                               int* __restrict__ err, uint32_t wait_tries,
                                                               const float* __restrict__ popw, int npop,
                                                               int ldpw, float* __restrict__ psum) {
  using L = TcSmem<KP>;
  constexpr int S = L::kStages;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::kBar);
  uint64_t* empty = full + S;
  constexpr int NA = L::kABuf;
  uint64_t* a_full = empty + S;
  uint64_t* a_empty = a_full + NA;
  uint64_t* acc_full = a_empty + NA;
  uint64_t* acc_empty = acc_full + kTcAcc;
  uint64_t* drain = acc_empty + kTcAcc;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t total = (int64_t)n_pt * nq;
  const int64_t f0 = tc_stretch_begin(blockIdx.x, total, gridDim.x);
  const int64_t f1 = tc_stretch_begin(blockIdx.x + 1, total, gridDim.x);
  const int n = (int)(f1 - f0);
  const int64_t tile_halfs = (int64_t)2 * 128 * KP;
  const int t_first = (int)(f0 / nq);
  const int q_first = (int)(f0 % nq);

  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, L::kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < S; ++b) {
      tc::mbar_init(&full[b], 1);
      tc::mbar_init(&empty[b], 1);
    }
    for (int b = 0; b < NA; ++b) {
      tc::mbar_init(&a_full[b], 1);
      tc::mbar_init(&a_empty[b], 1);
    }
    for (int b = 0; b < kTcAcc; ++b) {
      tc::mbar_init(&acc_full[b], 1);
      tc::mbar_init(&acc_empty[b], kTcEpiWarps);
    }
    tc::mbar_init(drain, 1);
    *abort_flag = 0;
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // launched as a dependent of the previous half-step's combine: everything
  // above is this CTA's own set-up; global memory only from here on
  pdl_wait();
  pdl_trigger();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sA = tc::smem_u32(smem + L::kA);
  const uint32_t sB = tc::smem_u32(smem + L::kB);

  if (warp == 0) {
    if (lane == 0) {
      // producer
      int t = t_first, q = q_first, seg = 0;
      int j_last = -1, seg_last = -1;  // last column tile / row tile whose copy was issued
      for (int j = 0; j < n; ++j) {
        const int stage = j % S;
        if (j >= S && !tc::mbar_wait_or_abort(&empty[stage], (uint32_t)((j / S - 1) & 1), wait_tries, abort_flag)) {
          *abort_flag = 1;
          atomicExch(err, 1);
          break;
        }
        if (j == 0 || q == 0) {
          if (j > 0) ++seg;
          if (seg >= NA && !tc::mbar_wait_or_abort(&a_empty[seg % NA], (uint32_t)((seg / NA - 1) & 1), wait_tries,
                                                    abort_flag)) {
            *abort_flag = 1;
            atomicExch(err, 1);
            break;
          }
          tc::mbar_expect_tx(&a_full[seg % NA], L::kTileBytes);
          tc::bulk_g2s(sA + (uint32_t)(seg % NA) * L::kTileBytes, Pt + (int64_t)t * tile_halfs, L::kTileBytes,
                       &a_full[seg % NA]);
          seg_last = seg;
        }
        tc::mbar_expect_tx(&full[stage], L::kTileBytes);
        tc::bulk_g2s(sB + (uint32_t)stage * L::kTileBytes, Qt + (int64_t)q * tile_halfs, L::kTileBytes,
                     &full[stage]);
        j_last = j;
        if (++q == nq) {
          q = 0;
          ++t;
        }
      }
      // Drain: the last copy issued into each buffer has landed. Copies into one
      // buffer complete its full barrier's phases in order and no later phase is
      // armed, so these waits return at once for copies that the MMA issuer
      // already consumed.
      for (int b = 0; b < S && b <= j_last; ++b) {
        const int jb = j_last - (j_last - b) % S;
        if (!tc::mbar_wait(&full[b], (uint32_t)((jb / S) & 1), kTcWaitTries)) atomicExch(err, 2);
      }
      for (int b = 0; b < NA && b <= seg_last; ++b) {
        const int sb = seg_last - (seg_last - b) % NA;
        if (!tc::mbar_wait(&a_full[b], (uint32_t)((sb / NA) & 1), kTcWaitTries)) atomicExch(err, 2);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer. The 6 MMAs of a tile accumulate into one TMEM accumulator and
      // so run one after another; tiles are therefore issued in pairs with their
      // MMAs interleaved, giving the tensor core two independent chains.
      int q = q_first, seg = 0;
      bool issued = false;
      constexpr int kGroup = kTcAcc >= 4 ? 2 : 1;
      for (int j0 = 0; j0 < n; j0 += kGroup) {
        const int cnt = j0 + 1 < n ? kGroup : 1;
        uint32_t a_addr[kGroup], b_addr[kGroup], d_addr[kGroup];
        bool seg_end[kGroup];
        int seg_of[kGroup];
        bool good = true;
        for (int u = 0; u < cnt; ++u) {
          const int j = j0 + u;
          const int stage = j % S, b = j % kTcAcc;
          const bool new_seg = j == 0 || q == 0;
          if (new_seg && j > 0) ++seg;
          if (new_seg)
            good = good &&
                   tc::mbar_wait(&a_full[seg % NA], (uint32_t)((seg / NA) & 1), wait_tries);
          good = good && tc::mbar_wait(&full[stage], (uint32_t)((j / S) & 1), wait_tries);
          if (j >= kTcAcc)
            good = good && tc::mbar_wait(&acc_empty[b], (uint32_t)((j / kTcAcc - 1) & 1), wait_tries);
          a_addr[u] = sA + (uint32_t)(seg % NA) * L::kTileBytes;
          b_addr[u] = sB + (uint32_t)stage * L::kTileBytes;
          d_addr[u] = tmem + (uint32_t)(128 * b);
          seg_of[u] = seg;
          if (++q == nq) q = 0;
          seg_end[u] = j == n - 1 || q == 0;
        }
        if (!good) {
          *abort_flag = 1;
          atomicExch(err, 1);
          break;
        }
        tc::fence_after_sync();
        issued = true;
        constexpr uint32_t idesc = tc::idesc_f16_f32(128, 128);
        constexpr uint32_t sbo = KP * 16;
#pragma unroll
        for (int st = 0; st < KP / 16; ++st) {
          const uint32_t ko = (uint32_t)st * 2u * tc::kCoreLbo;
#pragma unroll
          for (int pr = 0; pr < 3; ++pr) {
            for (int u = 0; u < cnt; ++u) {
              const uint32_t a_off = pr == 2 ? L::kHalfBytes : 0u;   // lo.hi uses A lo
              const uint32_t b_off = pr == 1 ? L::kHalfBytes : 0u;   // hi.lo uses B lo
              tc::mma_f16(d_addr[u], tc::smem_desc(a_addr[u] + a_off + ko, tc::kCoreLbo, sbo),
                          tc::smem_desc(b_addr[u] + b_off + ko, tc::kCoreLbo, sbo), idesc,
                          (st > 0 || pr > 0) ? 1u : 0u);
            }
          }
        }
        for (int u = 0; u < cnt; ++u) {
          const int j = j0 + u;
          tc::mma_commit(&empty[j % S]);
          tc::mma_commit(&acc_full[j % kTcAcc]);
          if (seg_end[u]) tc::mma_commit(&a_empty[seg_of[u] % NA]);
        }
      }
      // Drain: a last commit arrives once every MMA issued above has completed
      // (and after the arrivals of the commits before it).
      if (issued) {
        tc::mma_commit(drain);
        if (!tc::mbar_wait(drain, 0, kTcWaitTries)) atomicExch(err, 2);
      }
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31, columns of group (w - 2) / 4
    const int wq = warp & 3, cq = (warp - 2) >> 2;
    const int row = 32 * wq + lane;
    float m = kNegBig, s = 0.f;
    float2 acc[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    float sp[NPOP > 0 ? NPOP : 1];
#pragma unroll
    for (int k = 0; k < (NPOP > 0 ? NPOP : 1); ++k) sp[k] = 0.f;
    int t = t_first, q = q_first;
    // speculative form: the row's offset for the current row tile
    if (off) m = off[(int64_t)t * 128 + row];
    for (int j = 0; j < n; ++j) {
      const int b = j % kTcAcc;
      const bool good = __all_sync(
          0xffffffffu, tc::mbar_wait(&acc_full[b], (uint32_t)((j / kTcAcc) & 1), wait_tries));
      if (!good) {
        if (lane == 0) {
          *abort_flag = 1;
          atomicExch(err, 1);
        }
        break;
      }
      tc::fence_after_sync();
      static_assert(kTcColsPerWarp == 64, "two 32-column TMEM blocks per warp and tile");
      const uint32_t taddr = tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(128 * b + kTcColsPerWarp * cq);
      float d0[32], d1[32];
      const int col0 = q * 128 + kTcColsPerWarp * cq;   // first column of d0 within the column set
      if constexpr (NPOP > 0) {
        // first block, then the second block's load runs under the first
        // block's sums (fewer live registers beside the population sums)
        tc::tmem_ld32(taddr, d0);
        tc::tmem_wait_ld();
        tc::tmem_hold(d0);
        tc::tmem_ld32(taddr + 32, d1);
        multi32<NPOP>(d0, popw, npop, ldpw, col0, m, sp);
        tc::tmem_wait_ld();
        tc::tmem_hold(d1);
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        multi32<NPOP>(d1, popw, npop, ldpw, col0 + 32, m, sp);
      } else {
        // both 32-column blocks loaded at once and the accumulator handed back
        // to the MMA issuer before any sums (measured 3 % faster than
        // overlapping the second load with the first block's sums)
        tc::tmem_ld32(taddr, d0);
        tc::tmem_ld32(taddr + 32, d1);
        tc::tmem_wait_ld();
        tc::tmem_hold(d0);
        tc::tmem_hold(d1);
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        if (off) {
          sum32_off(d0, m, acc);
          sum32_off(d1, m, acc);
        } else {
          lse32(d0, m, s);
          lse32(d1, m, s);
        }
      }
      if (++q == nq || j == n - 1) {
        const int64_t slot = (((int64_t)blockIdx.x + t) * 128 + row) * kTcParts + cq;
        if (NPOP == 0 && off) {
          const float2 a = __fadd2_rn(__fadd2_rn(acc[0], acc[1]), __fadd2_rn(acc[2], acc[3]));
          s = a.x + a.y;
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[k] = make_float2(0.f, 0.f);
        }
        part[slot] = make_float2(m, s);
        if constexpr (NPOP > 0) {
#pragma unroll
          for (int k = 0; k < NPOP; ++k) {
            psum[slot * NPOP + k] = sp[k];
            sp[k] = 0.f;
          }
        }
        m = kNegBig;
        s = 0.f;
        if (q == nq) {
          q = 0;
          ++t;
        }
        if (off && j < n - 1) m = off[(int64_t)t * 128 + row];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, L::kTmemCols);
}

int tc_pack_points(const float* X, int64_t n, int64_t ldx, int d, int kp, float scale, int row_form,
                   __half* tiles, double* norm, cudaStream_t st) {
  const int64_t total = (n + 127) / 128 * 128 * kp;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 8);
  tc_pack_kernel<<<grid, 256, 0, st>>>(X, n, ldx, d, kp, scale, row_form, tiles, norm);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

int tc_pack_bias(int64_t n, const double* pot, const double* lsc, const double* norm, double inv_eps,
                 double kappa2d, int d, int kp, __half* tiles, cudaStream_t st) {
  const int64_t n_pad = (n + 127) / 128 * 128;
  const int grid = (int)std::min<int64_t>((n_pad + 255) / 256, (int64_t)sm_count() * 8);
  tc_bias_pack_kernel<<<grid, 256, 0, st>>>(n, n_pad, pot, lsc, norm, inv_eps, kappa2d, d, kp, tiles);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

template <int KP, int NPOP = 0>
static cudaError_t tc_set_smem_attr() {
  static cudaError_t once = cudaFuncSetAttribute(lse_tc_kernel<KP, NPOP>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcSmem<KP>::kAlloc);
  return once;
}

// Resident CTAs per SM of the half-step kernel.
int tc_ctas_per_sm(int kp) {
  (void)kp;
  return kTcCtasPerSm;
}
int tc_parts() { return kTcParts; }

int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nq, int kp, int ctas, float2* part,
                  const float* off, int* err, cudaStream_t st, uint32_t wait_tries, bool dependent) {
  const float* no_w = nullptr;
  float* no_s = nullptr;
  if (kp == 32) {
    WOTG_CUDA(tc_set_smem_attr<32>());
    if (dependent)
      WOTG_CUDA(launch_dependent(lse_tc_kernel<32, 0>, dim3(ctas), dim3(kTcThreads), TcSmem<32>::kAlloc, st, Pt, Qt,
                                 n_ptiles, nq, part, off, err, wait_tries, no_w, 0, 0, no_s));
    else
      lse_tc_kernel<32, 0><<<ctas, kTcThreads, TcSmem<32>::kAlloc, st>>>(Pt, Qt, n_ptiles, nq, part, off, err,
                                                                          wait_tries, nullptr, 0, 0, nullptr);
  } else if (kp == 64) {
    WOTG_CUDA(tc_set_smem_attr<64>());
    if (dependent)
      WOTG_CUDA(launch_dependent(lse_tc_kernel<64, 0>, dim3(ctas), dim3(kTcThreads), TcSmem<64>::kAlloc, st, Pt, Qt,
                                 n_ptiles, nq, part, off, err, wait_tries, no_w, 0, 0, no_s));
    else
      lse_tc_kernel<64, 0><<<ctas, kTcThreads, TcSmem<64>::kAlloc, st>>>(Pt, Qt, n_ptiles, nq, part, off, err,
                                                                          wait_tries, nullptr, 0, 0, nullptr);
  } else {
    return WOTG_BADARG;
  }
  WOTG_LAUNCHED();
  return WOTG_OK;
}


// Finish of the standalone half-step: L_i = ln2 (m + log2 s) - scale |x_i|^2; with
// `off`, also the base-2 offset m + log2 s that the speculative form reads.
__global__ void lse_points_finish_kernel(int64_t n, int nq, int ctas, int nparts, const float2* __restrict__ part,
                                         const double* __restrict__ norm, double scale, double* __restrict__ L,
                                         float* __restrict__ off) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t t = i >> 7;
  const int64_t total = ((n + 127) >> 7) * (int64_t)nq;
  const int64_t c_lo = tc_cta_of(t * nq, total, ctas);
  const int64_t c_hi = tc_cta_of((t + 1) * nq - 1, total, ctas);
  float m = kNegBig, s = 0.f;
  for (int64_t cc = c_lo; cc <= c_hi; ++cc) {
    const float2* pp = part + ((cc + t) * 128 + (i & 127)) * nparts;
    for (int k = 0; k < nparts; ++k) lse_merge(m, s, pp[k].x, pp[k].y);
  }
  const double D = lse2(m, s);
  if (L) L[i] = D * kLn2 - scale * norm[i];
  if (off) off[i] = (float)D;
}

// Population weights of columns [0, J) of k populations (FP64, row stride ldp),
// from population k0 on, as FP32 rows of jpad entries (zero past J).
__global__ void pop_pack_kernel(const double* __restrict__ P, int64_t ldp, int k0, int k, int64_t J, int64_t jpad,
                                int npop_max, float* __restrict__ popw) {
  const int64_t total = (int64_t)npop_max * jpad;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kk = (int)(idx / jpad);
    const int64_t j = idx % jpad;
    popw[idx] = (kk < k && j < J) ? (float)P[(int64_t)(k0 + kk) * ldp + j] : 0.f;
  }
}

// Finish of the population form: per row, the partials of every CTA range
// merged in FP64 against their largest maximum, then
// out[(k0 + kk) * n + i] = exp(b_i - scale |x_i|^2) 2^M S_kk.
__global__ void pop_finish_kernel(int64_t n, int nq, int ctas, int nparts, const float2* __restrict__ part,
                                  const float* __restrict__ psum, int npop_max, int k0, int k,
                                  const double* __restrict__ norm, double scale, const double* __restrict__ b,
                                  double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t t = i >> 7;
  const int64_t total = ((n + 127) >> 7) * (int64_t)nq;
  const int64_t c_lo = tc_cta_of(t * nq, total, ctas);
  const int64_t c_hi = tc_cta_of((t + 1) * nq - 1, total, ctas);
  float M = kNegBig;
  for (int64_t cc = c_lo; cc <= c_hi; ++cc)
    for (int q = 0; q < nparts; ++q) M = fmaxf(M, part[((cc + t) * 128 + (i & 127)) * nparts + q].x);
  const double base = (double)M * kLn2 - scale * norm[i] + (b ? b[i] : 0.0);
  for (int kk = 0; kk < k; ++kk) {
    double S = 0.0;
    for (int64_t cc = c_lo; cc <= c_hi; ++cc)
      for (int q = 0; q < nparts; ++q) {
        const int64_t slot = ((cc + t) * 128 + (i & 127)) * nparts + q;
        S += (double)psum[slot * npop_max + kk] * (double)ex2(part[slot].x - M);
      }
    out[(int64_t)(k0 + kk) * n + i] = S > 0.0 ? exp(base + log(S)) : 0.0;
  }
}

struct PointsLayout {
  int kp, n_xt, n_yt, ctas;
  __half* Xa;
  __half* Yb;
  double* normX;
  double* normY;
  float2* part;
  float* off;
  int* err;
};

static size_t points_layout(Bump& b, int64_t I, int64_t J, int d, PointsLayout& P) {
  P.kp = tc_kp(d);
  P.n_xt = (int)((I + 127) / 128);
  P.n_yt = (int)((J + 127) / 128);
  P.ctas = (int)std::min<int64_t>((int64_t)sm_count() * tc_ctas_per_sm(P.kp), (int64_t)P.n_xt * P.n_yt);
  const size_t tb = tc_tile_bytes(P.kp);
  P.Xa = reinterpret_cast<__half*>(b.take<unsigned char>(tb * P.n_xt));
  P.Yb = reinterpret_cast<__half*>(b.take<unsigned char>(tb * P.n_yt));
  P.normX = b.take<double>(I);
  P.normY = b.take<double>(J);
  P.part = b.take<float2>((size_t)(P.ctas + P.n_xt) * 128 * kTcParts);
  P.off = b.take<float>((size_t)P.n_xt * 128);
  P.err = b.take<int>(4);
  return b.off + 256;
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

extern "C" size_t wotg_lse_points_workspace_bytes(int64_t I, int64_t J, int32_t d) {
  if (I <= 0 || J <= 0 || d < 1 || d > tc_max_dim()) return 0;
  Bump b{nullptr, 0};
  PointsLayout P{};
  return points_layout(b, I, J, d, P);
}

static int lse_points_run(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy, int32_t d,
                          double scale, const double* w, double* L, void* workspace, size_t workspace_bytes,
                          cudaStream_t st, uint32_t wait_tries, int** err_out) {
  if (!X || !Y || !w || !L || I <= 0 || J <= 0 || d < 1 || d > tc_max_dim() || ldx < d || ldy < d ||
      !(scale > 0))
    return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_lse_points_workspace_bytes(I, J, d)) return WOTG_WORKSPACE;
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  PointsLayout P{};
  points_layout(b, I, J, d, P);
  if (err_out) *err_out = P.err;
  const double sigma = std::sqrt(scale);
  WOTG_CUDA(cudaMemsetAsync(P.err, 0, sizeof(int), st));
  int s = tc_pack_points(X, I, ldx, d, P.kp, (float)(2.0 * kLog2e * sigma), 1, P.Xa, P.normX, st);
  if (s) return s;
  s = tc_pack_points(Y, J, ldy, d, P.kp, (float)sigma, 0, P.Yb, P.normY, st);
  if (s) return s;
  s = tc_pack_bias(J, w, nullptr, P.normY, 1.0, scale * kLog2e, d, P.kp, P.Yb, st);
  if (s) return s;
  s = tc_lse_launch(P.Xa, P.n_xt, P.Yb, P.n_yt, P.kp, P.ctas, P.part, nullptr, P.err, st, wait_tries);
  if (s) return s;
  lse_points_finish_kernel<<<(unsigned)((I + 255) / 256), 256, 0, st>>>(I, P.n_yt, P.ctas, kTcParts, P.part,
                                                                        P.normX, scale, L, nullptr);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

extern "C" int wotg_lse_points(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy,
                               int32_t d, double scale, const double* w, double* L, void* workspace,
                               size_t workspace_bytes, void* stream) {
  return lse_points_run(X, I, ldx, Y, J, ldy, d, scale, w, L, workspace, workspace_bytes, (cudaStream_t)stream,
                        kTcWaitTries, nullptr);
}

extern "C" int wotg_lse_points_bounded(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J,
                                       int64_t ldy, int32_t d, double scale, const double* w, double* L,
                                       uint32_t wait_tries, void* workspace, size_t workspace_bytes, void* stream) {
  if (wait_tries > kTcWaitTries) return WOTG_BADARG;
  cudaStream_t st = (cudaStream_t)stream;
  int* err_dev = nullptr;
  int s = lse_points_run(X, I, ldx, Y, J, ldy, d, scale, w, L, workspace, workspace_bytes, st, wait_tries, &err_dev);
  if (s) return s;
  int err = 0;
  WOTG_CUDA(cudaMemcpyAsync(&err, err_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  WOTG_CUDA(cudaStreamSynchronize(st));
  if (err) {
    set_last_message(err == 1 ? "tensor-core half-step: a bounded wait ran out; the kernel stopped and drained"
                              : "tensor-core half-step: a drain wait ran out");
    return WOTG_CUDA_ERROR;
  }
  return WOTG_OK;
}

extern "C" int wotg_lse_points_timing(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J,
                                      int64_t ldy, int32_t d, double scale, const double* w, int32_t speculative,
                                      int32_t n_launch, float* ms_per_launch, void* workspace,
                                      size_t workspace_bytes, void* stream) {
  if (!X || !Y || !w || !ms_per_launch || I <= 0 || J <= 0 || d < 1 || d > tc_max_dim() || ldx < d ||
      ldy < d || !(scale > 0) || n_launch < 1 || n_launch > 10000)
    return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_lse_points_workspace_bytes(I, J, d)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  PointsLayout P{};
  points_layout(b, I, J, d, P);
  const double sigma = std::sqrt(scale);
  WOTG_CUDA(cudaMemsetAsync(P.err, 0, sizeof(int), st));
  WOTG_CUDA(cudaMemsetAsync(P.off, 0, sizeof(float) * (size_t)P.n_xt * 128, st));
  int s = tc_pack_points(X, I, ldx, d, P.kp, (float)(2.0 * kLog2e * sigma), 1, P.Xa, P.normX, st);
  if (s) return s;
  s = tc_pack_points(Y, J, ldy, d, P.kp, (float)sigma, 0, P.Yb, P.normY, st);
  if (s) return s;
  s = tc_pack_bias(J, w, nullptr, P.normY, 1.0, scale * kLog2e, d, P.kp, P.Yb, st);
  if (s) return s;
  // one exact launch gives every row's offset (the previous LSE, as in the solve's steady state)
  s = tc_lse_launch(P.Xa, P.n_xt, P.Yb, P.n_yt, P.kp, P.ctas, P.part, nullptr, P.err, st);
  if (s) return s;
  lse_points_finish_kernel<<<(unsigned)((I + 255) / 256), 256, 0, st>>>(I, P.n_yt, P.ctas, kTcParts, P.part,
                                                                        P.normX, scale, nullptr, P.off);
  WOTG_LAUNCHED();
  cudaEvent_t e0, e1;
  WOTG_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    set_last_error("cudaEventCreate", cudaGetLastError());
    return WOTG_CUDA_ERROR;
  }
  cudaError_t e = cudaEventRecord(e0, st);
  for (int k = 0; k < n_launch && e == cudaSuccess && s == WOTG_OK; ++k)
    s = tc_lse_launch(P.Xa, P.n_xt, P.Yb, P.n_yt, P.kp, P.ctas, P.part, speculative ? P.off : nullptr, P.err, st);
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s) return s;
  if (e != cudaSuccess) {
    set_last_error("lse_points timing", e);
    return WOTG_CUDA_ERROR;
  }
  int err = 0;
  WOTG_CUDA(cudaMemcpy(&err, P.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    set_last_message("tensor-core half-step: a bounded wait timed out");
    return WOTG_CUDA_ERROR;
  }
  *ms_per_launch = ms / (float)n_launch;
  return WOTG_OK;
}

// ---------------------------------------------------------------------------
// The population form: out[k, i] = exp(b_i) sum_j exp(w_j - scale |x_i - y_j|^2) P[k, j]
// with one exp per (i, j) for up to kTcPops populations per launch.
// ---------------------------------------------------------------------------
namespace wotg {
constexpr int kTcPops = 8;

static size_t apply_layout(Bump& b, int64_t I, int64_t J, int d, PointsLayout& P, float** popw, float** psum) {
  points_layout(b, I, J, d, P);
  *popw = b.take<float>((size_t)kTcPops * P.n_yt * 128);
  *psum = b.take<float>((size_t)(P.ctas + P.n_xt) * 128 * kTcParts * kTcPops);
  return b.off + 256;
}
}  // namespace wotg

extern "C" size_t wotg_apply_points_workspace_bytes(int64_t I, int64_t J, int32_t d) {
  if (I <= 0 || J <= 0 || d < 1 || d > tc_max_dim()) return 0;
  Bump b{nullptr, 0};
  PointsLayout P{};
  float *popw, *psum;
  return apply_layout(b, I, J, d, P, &popw, &psum);
}

extern "C" int wotg_apply_points(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy,
                                 int32_t d, double scale, const double* w, const double* bias, const double* Pw,
                                 int64_t ldp, int32_t k, double* out, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  if (!X || !Y || !w || !Pw || !out || I <= 0 || J <= 0 || d < 1 || d > tc_max_dim() || ldx < d || ldy < d ||
      !(scale > 0) || k < 1 || ldp < J)
    return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_apply_points_workspace_bytes(I, J, d)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  PointsLayout P{};
  float *popw, *psum;
  apply_layout(b, I, J, d, P, &popw, &psum);
  const double sigma = std::sqrt(scale);
  const int64_t jpad = (int64_t)P.n_yt * 128;
  WOTG_CUDA(cudaMemsetAsync(P.err, 0, sizeof(int), st));
  int s = tc_pack_points(X, I, ldx, d, P.kp, (float)(2.0 * kLog2e * sigma), 1, P.Xa, P.normX, st);
  if (s) return s;
  s = tc_pack_points(Y, J, ldy, d, P.kp, (float)sigma, 0, P.Yb, P.normY, st);
  if (s) return s;
  s = tc_pack_bias(J, w, nullptr, P.normY, 1.0, scale * kLog2e, d, P.kp, P.Yb, st);
  if (s) return s;
  for (int k0 = 0; k0 < k; k0 += kTcPops) {
    const int kc = std::min(kTcPops, k - k0);
    const int pgrid = (int)std::min<int64_t>((kTcPops * jpad + 255) / 256, (int64_t)sm_count() * 8);
    pop_pack_kernel<<<pgrid, 256, 0, st>>>(Pw, ldp, k0, kc, J, jpad, kTcPops, popw);
    WOTG_LAUNCHED();
    if (P.kp == 32) {
      WOTG_CUDA((tc_set_smem_attr<32, kTcPops>()));
      lse_tc_kernel<32, kTcPops><<<P.ctas, kTcThreads, TcSmem<32>::kAlloc, st>>>(
          P.Xa, P.Yb, P.n_xt, P.n_yt, P.part, nullptr, P.err, kTcWaitTries, popw, kc, (int)jpad, psum);
    } else {
      WOTG_CUDA((tc_set_smem_attr<64, kTcPops>()));
      lse_tc_kernel<64, kTcPops><<<P.ctas, kTcThreads, TcSmem<64>::kAlloc, st>>>(
          P.Xa, P.Yb, P.n_xt, P.n_yt, P.part, nullptr, P.err, kTcWaitTries, popw, kc, (int)jpad, psum);
    }
    WOTG_LAUNCHED();
    pop_finish_kernel<<<(unsigned)((I + 255) / 256), 256, 0, st>>>(I, P.n_yt, P.ctas, kTcParts, P.part, psum,
                                                                  kTcPops, k0, kc, P.normX, scale, bias, out);
    WOTG_LAUNCHED();
  }
  return WOTG_OK;
}
