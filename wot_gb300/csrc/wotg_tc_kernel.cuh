// wotg_tc_kernel.cuh — the tensor-core half-step kernel (tcgen05 cost tiles,
// log-sum-exp epilogue from TMEM), shared by the standalone entry points and
// the solvers. Its `Fin` policy lets a solver finish each row tile inside the
// kernel (merge of the partials and the FP64 update, see lse_tc_kernel);
// NoFin leaves the partials to a separate pass.
#pragma once

#include <stdint.h>

#include "wotg_common.cuh"
#include "wotg_onthefly.cuh"
#include "wotg_tc.cuh"

namespace wotg {

constexpr uint32_t kTcWaitTries = kTcDefaultWaitTries;  // x up to 1 us per try: about 4 s

// The partials stay in `part` for a separate merge.
struct NoFin {
  static constexpr bool kActive = false;
  __device__ __forceinline__ void start() const {}
  __device__ __forceinline__ void quarter_done(const float2* part, int t, int wq, int lane) const {}
};

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
// Fin (a solver's policy): once a warp has written its partial of a segment,
// fin.quarter_done() counts it for its row tile and lane quarter; the warp
// that brings the count to 2 x (CTAs covering the tile) merges those 32 rows'
// partials and applies the solver's update (no barrier, no wait: per-warp
// counters in global memory, reset by that warp for the next launch).
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
template <int KP, int NPOP, class Fin = NoFin>
__global__ void __launch_bounds__(kTcThreads, kTcCtasPerSm) lse_tc_kernel(const __half* __restrict__ Pt,
                                                               const __half* __restrict__ Qt,
                                                               int n_pt, int nq, float2* __restrict__ part,
                                                               const float* off,
                                                               int* __restrict__ err, uint32_t wait_tries,
                                                               const float* __restrict__ popw, int npop,
                                                               int ldpw, float* __restrict__ psum, Fin fin) {
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
  if (Fin::kActive && blockIdx.x == 0 && tid == 0) fin.start();
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
        // the warp that writes the last partial of rows [t 128 + 32 wq, + 32)
        // (over the CTAs and column halves covering the row tile) finishes them
        if constexpr (Fin::kActive) fin.quarter_done(part, t, wq, lane);
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


template <int KP, int NPOP = 0, class Fin = NoFin>
static cudaError_t tc_set_smem_attr() {
  static cudaError_t once = cudaFuncSetAttribute(lse_tc_kernel<KP, NPOP, Fin>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcSmem<KP>::kAlloc);
  return once;
}

}  // namespace wotg
