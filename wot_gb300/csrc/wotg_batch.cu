// wotg_batch.cu — batched transport solves on a materialised cost (sm_103a).
//
// A batch is a set of day pairs (FP32 cost C and its transpose CT) and a set of
// items, each one transport problem on one pair with its own parameters (a
// 40-pair time course x a 5 x 5 epsilon x lambda1 sweep is 1000 items on 40
// pairs). The reference solves them one by one (wot/ot/ot_model.py:124-201,
// optimal_transport.py:67-164); here they advance together:
//
//  * A half-step is one persistent launch over tiles of (pair, 8 x RW rows of C
//    or CT). A tile reads its rows of the cost once and evaluates the base-2
//    log-sum-exp of every active item of the pair against them (KG items per
//    register group), so the HBM traffic of a pair is paid once per half-step
//    however many parameter sets it carries and the exp rate becomes the bound.
//  * The sum is speculative: each (row, item) keeps the previous half-step's
//    log-sum-exp as an offset o, so sum_j 2^(t_j - o) needs no running maximum;
//    a sum outside [2^-80, 2^100] (stage start, first iteration) is recomputed
//    exactly with a running maximum by the warp that owns the row.
//  * The reference's control flow runs per item on the device: after the two
//    half-steps, `item_kernel` applies tau-absorption and counts iterations and
//    batches; a check pass recomputes the row sums of items whose batch ended
//    in the final stage (and sum exp(-C/eps) for items entering it);
//    `test_kernel` evaluates the stage-exit test or the duality gap and decides
//    each item's next step (next batch, next stage, next growth iteration,
//    done), whose O(I + J) work `apply_kernel` does. Each item's O(I + J) loops
//    are split over several CTAs (FP64 is 1/64 of the FP32 rate on this part,
//    so one CTA per item would serialise them), with fixed-order sums. The last
//    CTA of each of those kernels rebuilds the per-pair lists of items the next
//    pass will see.
//  * Six launches per iteration of the whole batch, captured B iterations at a
//    time in a CUDA graph and replayed until no item is active.
//
// Item state and iteration counts follow the single-problem driver
// (wotg_sinkhorn.cu) step for step, so every item gives the reference's
// sequence of stages, checks and absorptions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "wotg_coef.cuh"
#include "wotg_common.cuh"

namespace wotg {
namespace batch {

enum Mode : int { kRowA = 0, kColB = 1, kFresh = 2, kSumK = 3, kOut = 4, kNone = 5 };
enum Status : int { kActive = 0, kMaxIterPending = 1, kDone = 2, kDoneMaxIter = 3, kNonfinite = 4 };
constexpr int kScalings = 5;   // n_scalings of the duality-gap solver (optimal_transport.py:105)
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 128;    // columns per staged chunk: one float4 per lane
constexpr float kSpecLo = 0x1p-80f;
constexpr float kSpecHi = 0x1p100f;

// One right-hand side of a pass over a pair's rows.
struct Entry {
  const float* w;  // base-2 column weights, >= roundup(cols, 4) floats, 16-byte aligned
  float* o;        // base-2 row offsets (speculative sum), in/out; NULL = 0
  double* out;     // kOut: natural-log LSE per row
  float nk2;       // -kappa2 (< 0)
  int item;
  int mode;
  int pad_;
};

struct Seg {
  const float* C;  // rows x ldc
  int64_t ldc;
  int rows, cols;
};

struct Tile {
  int pair;
  int row0;
};

// One transport problem and its solver state.
struct Item {
  int pair, I, J, pad0;
  double cost_scale;
  // parameters
  double epsilon, lambda1, lambda2, epsilon0, tau, tolerance, max_iter;
  int batch_size, growth_iters;
  // state vectors
  double *u, *la, *la_old, *logp, *p, *Lrow, *rsum;
  double *v, *lb, *lb_old, *Lcol;
  float *wrow, *orow, *wcol, *ocol;
  // outputs
  double *ubar, *vbar, *row_sums, *learned;
  // control
  Coef c;
  double scale_factor, eps_i, gap, sumK, threshold, q;
  long long it, it_total, checks, absorptions;
  int status, stage, batch_cnt, parity, skip_row, due, need_sumk, gi, hit_max_iter, action;
  int first_blk, nblk;  // this item's CTAs in the per-item kernels
  double eps_prev, q_next;
  unsigned long long maxslot[2];
};

// CTA b of a per-item kernel works on item blk[b].item, slice blk[b].rank.
struct ItemBlock {
  int item, rank;
};

struct PassArgs {
  const Seg* segs;  // 2 per pair: [2p] = C rows, [2p + 1] = CT rows
  int dir;
  const Tile* tiles;
  int ntiles;
  const int* list_n;    // entries per pair
  const Entry* list;    // entries of pair p at list + list_off[p]
  const int* list_off;
  Item* items;
  int* counter;         // tile ticket
};

struct BatchArgs {
  Item* items;
  int n_items, n_pairs;
  const int* pair_items;      // items of pair p: pair_items[pair_off[p] .. pair_off[p + 1])
  const int* pair_off;
  int* row_n;
  Entry* row_list;            // capacity K_p per pair at pair_off[p]
  int* col_n;
  Entry* col_list;
  int* chk_n;
  Entry* chk_list;            // capacity 2 K_p per pair at 2 pair_off[p]
  int* counters;              // [0] row, [1] col, [2] check tickets; [3..7] grid-wide last-block counters
  int* active;
  const float* zeros;
  const ItemBlock* blk;       // per-item kernels: one entry per CTA
  int* item_ctr;              // per item: CTAs of the current per-item kernel that finished
  double* part;               // per CTA: kNq partial sums
};

constexpr int kNq = 10;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* g, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(saddr), "l"(g), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Packed FP32 pairs (sm_100 family): one instruction for two elements.
__device__ __forceinline__ uint64_t pk(float x, float y) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float2 upk(uint64_t r) {
  float2 v;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
  return v;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// 2^(t - o) for a packed pair t and packed offset (-o, -o).
__device__ __forceinline__ uint64_t ex2_off(uint64_t t, uint64_t mo) {
  const float2 v = upk(add2(t, mo));
  return pk(ex2(v.x), ex2(v.y));
}

__device__ __forceinline__ float warp_sumf(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// ---------------------------------------------------------------------------
// Per-(row, item) epilogues: the single-problem driver's a- and b-updates
// (optimal_transport.py:131-135) on the item's vectors.
// ---------------------------------------------------------------------------
// Both return the new log-scaling (the absorption test takes exp of its maximum).
__device__ __forceinline__ double item_a_update(Item& it, int64_t i, double L) {
  const Coef& c = it.c;
  const double ui = it.u[i];
  const double logs = ui * c.inv_eps + L - c.logJ;
  const double la_new = c.alpha1 * (it.logp[i] - logs) - ui * c.inv_l1e;
  it.la_old[i] = it.la[i];
  it.la[i] = la_new;
  it.wrow[i] = (float)((ui * c.inv_eps + la_new) * kLog2e);
  return la_new;
}

__device__ __forceinline__ double item_b_update(Item& it, int64_t j, double L) {
  const Coef& c = it.c;
  const double vj = it.v[j];
  const double logt = vj * c.inv_eps + L - c.logI;
  const double lb_new = c.alpha2 * (c.logq - logt) - vj * c.inv_l2e;
  it.lb_old[j] = it.lb[j];
  it.lb[j] = lb_new;
  it.wcol[j] = (float)((vj * c.inv_eps + lb_new) * kLog2e);
  return lb_new;
}

// L2 = base-2 log-sum-exp of row r for entry e; returns the log-scaling whose
// maximum over rows feeds the absorption test (log a_i or log b_j), else -inf.
__device__ __forceinline__ double entry_epilogue(Item* items, const Entry& e, int64_t r, double L2) {
  const double L = L2 * kLn2;
  switch (e.mode) {
    case kOut:
      e.out[r] = L;
      if (e.o) e.o[r] = (float)L2;
      return -INFINITY;
    case kFresh: {
      Item& it = items[e.item];
      it.Lrow[r] = L;
      it.orow[r] = (float)L2;
      return -INFINITY;
    }
    case kSumK:
      items[e.item].rsum[r] = exp(L);
      return -INFINITY;
    case kRowA: {
      Item& it = items[e.item];
      it.Lrow[r] = L;
      it.orow[r] = (float)L2;
      return item_a_update(it, r, L);
    }
    case kColB: {
      Item& it = items[e.item];
      it.Lcol[r] = L;
      it.ocol[r] = (float)L2;
      return item_b_update(it, r, L);
    }
    default:
      return -INFINITY;
  }
}

// Exact base-2 LSE of one row for one entry, by a whole warp from global memory
// (running maximum; entries past `cols` masked). Returns (m, s): value s 2^m.
__device__ float2 exact_row(const float* crow, int64_t ldc, const float* w, float nk2, int cols, int lane) {
  float m = kNegBig, s = 0.f;
  const float4* c4 = reinterpret_cast<const float4*>(crow);
  const float4* w4 = reinterpret_cast<const float4*>(w);
  const int64_t nq = ((int64_t)cols + 3) >> 2;
  for (int64_t q = lane; q < nq; q += 32) {
    const float4 cc = c4[q];
    const float4 ww = w4[q];
    const int64_t col = q * 4;
    const float t0 = fmaf(nk2, cc.x, ww.x);
    const float t1 = col + 1 < cols ? fmaf(nk2, cc.y, ww.y) : -INFINITY;
    const float t2 = col + 2 < cols ? fmaf(nk2, cc.z, ww.z) : -INFINITY;
    const float t3 = col + 3 < cols ? fmaf(nk2, cc.w, ww.w) : -INFINITY;
    const float mn = fmaxf(m, fmaxf(fmaxf(t0, t1), fmaxf(t2, t3)));
    s = s * ex2(m - mn) + ((ex2(t0 - mn) + ex2(t1 - mn)) + (ex2(t2 - mn) + ex2(t3 - mn)));
    m = mn;
  }
  (void)ldc;
  warp_lse(m, s);
  return make_float2(m, s);
}

// Stage the weights of columns [col0, col0 + 128) of the group's entries into
// shared memory (zero past `cols`), one 16-byte cp.async per thread and float4.
template <int KG>
__device__ __forceinline__ void stage_weights(float (*dst)[kChunk], const Entry* gp, int ng, int64_t col0,
                                              int cols) {
  for (int idx = threadIdx.x; idx < ng * 32; idx += kThreads) {
    const int k = idx >> 5, q = idx & 31;
    const int64_t col = col0 + q * 4;
    const int64_t left = (int64_t)cols - col;
    const uint32_t bytes = left >= 4 ? 16u : (left > 0 ? (uint32_t)left * 4u : 0u);
    const float* src = bytes ? gp[k].w + col : gp[k].w;
    cp_async16(smem_addr(&dst[k][q * 4]), src, bytes);
  }
}

__device__ __forceinline__ float4 load_cost(const float4* crow, int64_t q, int64_t nv, bool valid) {
  if (valid && q < nv) return ld_stream(crow + q);
  return make_float4(INFINITY, INFINITY, INFINITY, INFINITY);
}

// One group of up to KG entries over the tile's rows (warp w owns rows
// row0 + w * RW + [0, RW)). SPEC: offset sums with exact fallback; else running max.
template <int KG, int RW, bool SPEC>
__device__ __forceinline__ void run_group(const PassArgs& A, const Seg& sg, int row0, int ng, const Entry* gp,
                                          float (*sW)[KG][kChunk], double (*s_vmax)[KG], int warp, int lane) {
  float nk2[KG];
  float acc[RW][KG], off[RW][KG];
  bool valid[RW];
  int64_t row[RW];
  const float4* crow[RW];
#pragma unroll
  for (int rr = 0; rr < RW; ++rr) {
    row[rr] = (int64_t)row0 + warp * RW + rr;
    valid[rr] = row[rr] < sg.rows;
    crow[rr] = reinterpret_cast<const float4*>(sg.C + (valid[rr] ? row[rr] : 0) * sg.ldc);
  }
#pragma unroll
  for (int k = 0; k < KG; ++k) {
    nk2[k] = k < ng ? gp[k].nk2 : -1.f;
#pragma unroll
    for (int rr = 0; rr < RW; ++rr) {
      acc[rr][k] = 0.f;
      if (SPEC)
        off[rr][k] = (k < ng && valid[rr] && gp[k].o) ? gp[k].o[row[rr]] : 0.f;
      else
        off[rr][k] = kNegBig;
    }
  }
  const int nch = (sg.cols + kChunk - 1) / kChunk;
  const int64_t nv = sg.ldc >> 2;
  stage_weights<KG>(sW[0], gp, ng, 0, sg.cols);
  cp_async_commit();
  float4 nxt[RW];
#pragma unroll
  for (int rr = 0; rr < RW; ++rr) nxt[rr] = load_cost(crow[rr], lane, nv, valid[rr]);
  for (int ch = 0; ch < nch; ++ch) {
    if (ch + 1 < nch) stage_weights<KG>(sW[(ch + 1) & 1], gp, ng, (int64_t)(ch + 1) * kChunk, sg.cols);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    float4 cc[RW];
#pragma unroll
    for (int rr = 0; rr < RW; ++rr) {
      cc[rr] = nxt[rr];
      if (ch + 1 < nch) nxt[rr] = load_cost(crow[rr], (int64_t)(ch + 1) * 32 + lane, nv, valid[rr]);
    }
    const float* wb = &sW[ch & 1][0][lane * 4];
    if (SPEC) {
      uint64_t c01[RW], c23[RW];
#pragma unroll
      for (int rr = 0; rr < RW; ++rr) {
        c01[rr] = pk(cc[rr].x, cc[rr].y);
        c23[rr] = pk(cc[rr].z, cc[rr].w);
      }
#pragma unroll
      for (int k = 0; k < KG; ++k) {
        if (k < ng) {
          const float4 w = *reinterpret_cast<const float4*>(wb + k * kChunk);
          const uint64_t w01 = pk(w.x, w.y), w23 = pk(w.z, w.w), kk = pk(nk2[k], nk2[k]);
#pragma unroll
          for (int rr = 0; rr < RW; ++rr) {
            const uint64_t mo = pk(-off[rr][k], -off[rr][k]);
            const uint64_t e01 = ex2_off(fma2(kk, c01[rr], w01), mo);
            const uint64_t e23 = ex2_off(fma2(kk, c23[rr], w23), mo);
            const float2 e = upk(add2(e01, e23));
            acc[rr][k] += e.x + e.y;
          }
        }
      }
    } else {
#pragma unroll
    for (int k = 0; k < KG; ++k) {
      if (k < ng) {
        const float4 w = *reinterpret_cast<const float4*>(wb + k * kChunk);
#pragma unroll
        for (int rr = 0; rr < RW; ++rr) {
          const float t0 = fmaf(nk2[k], cc[rr].x, w.x);
          const float t1 = fmaf(nk2[k], cc[rr].y, w.y);
          const float t2 = fmaf(nk2[k], cc[rr].z, w.z);
          const float t3 = fmaf(nk2[k], cc[rr].w, w.w);
          {
            const float m = off[rr][k];
            const float mn = fmaxf(m, fmaxf(fmaxf(t0, t1), fmaxf(t2, t3)));
            acc[rr][k] = acc[rr][k] * ex2(m - mn) + ((ex2(t0 - mn) + ex2(t1 - mn)) + (ex2(t2 - mn) + ex2(t3 - mn)));
            off[rr][k] = mn;
          }
        }
      }
    }
    }
    __syncthreads();
  }
  // Warp totals (every lane ends with every (row, entry) total).
#pragma unroll
  for (int rr = 0; rr < RW; ++rr)
#pragma unroll
    for (int k = 0; k < KG; ++k) {
      if (k < ng) {
        if (SPEC)
          acc[rr][k] = warp_sumf(acc[rr][k]);
        else
          warp_lse(off[rr][k], acc[rr][k]);
      }
    }
  // Lane k finishes entry k.
  double vmax = -INFINITY;
#pragma unroll
  for (int rr = 0; rr < RW; ++rr) {
    float s = 0.f, o = 0.f;
#pragma unroll
    for (int k = 0; k < KG; ++k)
      if (k == lane) {
        s = acc[rr][k];
        o = off[rr][k];
      }
    bool mine = lane < ng && valid[rr];
    if (SPEC) {
      const bool bad = mine && !(s >= kSpecLo && s <= kSpecHi);
      unsigned redo = __ballot_sync(0xffffffffu, bad);
      while (redo) {
        const int k = __ffs(redo) - 1;
        redo &= redo - 1;
        const float2 ms = exact_row(sg.C + row[rr] * sg.ldc, sg.ldc, gp[k].w, gp[k].nk2, sg.cols, lane);
        if (lane == k) {
          o = ms.x;
          s = ms.y;
        }
      }
    }
    if (mine) {
      vmax = fmax(vmax, entry_epilogue(A.items, gp[lane], row[rr], lse2(o, s)));
    }
  }
  if (lane < KG) s_vmax[warp][lane] = vmax;
}

// One entry over the tile's rows (a pair with a single active item, as in the
// tail of a batch): each warp streams its rows with 128-bit loads of the cost
// and the weights (L1/L2-resident), no shared-memory staging and no barrier.
// Columns past `cols` in the last float4 meet the cost's +inf padding.
template <int RW, int KG>
__device__ __forceinline__ void run_single(const PassArgs& A, const Seg& sg, int row0, const Entry* gp,
                                           double (*s_vmax)[KG], int warp, int lane) {
  const Entry e = gp[0];
  const float nk2 = e.nk2;
  const float4* __restrict__ w4 = reinterpret_cast<const float4*>(e.w);
  const int64_t nq = ((int64_t)sg.cols + 3) >> 2;
  double vmax = -INFINITY;
#pragma unroll 1
  for (int rr = 0; rr < RW; ++rr) {
    const int64_t row = (int64_t)row0 + warp * RW + rr;
    if (row >= sg.rows) break;
    const float4* __restrict__ crow = reinterpret_cast<const float4*>(sg.C + row * sg.ldc);
    const float o = e.o ? e.o[row] : 0.f;
    const uint64_t kk = pk(nk2, nk2), mo = pk(-o, -o);
    float s0 = 0.f, s1 = 0.f;
    int64_t q = lane;
    for (; q + 96 < nq; q += 128) {
      float4 cc[4], ww[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) cc[t] = ld_stream(crow + q + 32 * t);
#pragma unroll
      for (int t = 0; t < 4; ++t) ww[t] = __ldg(w4 + q + 32 * t);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const uint64_t e01 = ex2_off(fma2(kk, pk(cc[t].x, cc[t].y), pk(ww[t].x, ww[t].y)), mo);
        const uint64_t e23 = ex2_off(fma2(kk, pk(cc[t].z, cc[t].w), pk(ww[t].z, ww[t].w)), mo);
        const float2 e = upk(add2(e01, e23));
        s0 += e.x;
        s1 += e.y;
      }
    }
    for (; q < nq; q += 32) {
      const float4 cc = ld_stream(crow + q);
      const float4 ww = __ldg(w4 + q);
      s0 += ex2(fmaf(nk2, cc.x, ww.x) - o) + ex2(fmaf(nk2, cc.y, ww.y) - o);
      s1 += ex2(fmaf(nk2, cc.z, ww.z) - o) + ex2(fmaf(nk2, cc.w, ww.w) - o);
    }
    float s = warp_sumf(s0 + s1);
    float oo = o;
    if (!(s >= kSpecLo && s <= kSpecHi)) {
      const float2 ms = exact_row(sg.C + row * sg.ldc, sg.ldc, e.w, nk2, sg.cols, lane);
      oo = ms.x;
      s = ms.y;
    }
    if (lane == 0) vmax = fmax(vmax, entry_epilogue(A.items, e, row, lse2(oo, s)));
  }
  if (lane == 0) s_vmax[warp][0] = vmax;
}

template <int KG, int RW, bool SPEC>
__global__ void __launch_bounds__(kThreads) pass_kernel(PassArgs A) {
  __shared__ __align__(16) float sW[2][KG][kChunk];
  __shared__ Entry gp[KG];
  __shared__ double s_vmax[kWarps][KG];
  __shared__ int s_tile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(A.counter, 1);
    __syncthreads();
    const int t = s_tile;
    __syncthreads();
    if (t >= A.ntiles) break;
    const Tile tile = A.tiles[t];
    const Seg sg = A.segs[2 * tile.pair + A.dir];
    const int nk = A.list_n[tile.pair];
    const Entry* lst = A.list + A.list_off[tile.pair];
    for (int g0 = 0; g0 < nk; g0 += KG) {
      const int ng = min(KG, nk - g0);
      if (threadIdx.x < ng) gp[threadIdx.x] = lst[g0 + threadIdx.x];
      __syncthreads();
      if (SPEC && ng == 1)
        run_single<RW, KG>(A, sg, tile.row0, gp, s_vmax, warp, lane);
      else
        run_group<KG, RW, SPEC>(A, sg, tile.row0, ng, gp, sW, s_vmax, warp, lane);
      __syncthreads();
      // absorption maxima of this group: one atomic per item
      if (threadIdx.x < ng) {
        const Entry& e = gp[threadIdx.x];
        if (e.mode == kRowA || e.mode == kColB) {
          double v = -INFINITY;
#pragma unroll
          for (int w = 0; w < kWarps; ++w) v = fmax(v, s_vmax[w][threadIdx.x]);
          Item& it = A.items[e.item];
          atomic_max_nonneg(&it.maxslot[it.parity], exp(v));
        }
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Per-item kernels. Item k owns CTAs [first_blk, first_blk + nblk) of each
// launch; its O(I + J) loops are split over them (ITEM_LOOP), its sums are
// per-CTA partials reduced in a fixed order by the item's last CTA, which also
// takes the item's scalar decisions. The grid's last CTA rebuilds the lists.
// ---------------------------------------------------------------------------
enum Action : int { kActNone = 0, kActCont = 1, kActStage = 2, kActFinish = 3, kActFinishMax = 4 };

#define ITEM_LOOP(var, n) \
  for (int var = rank * kThreads + (int)threadIdx.x; var < (n); var += nblk * kThreads)

template <int NQ>
__device__ void block_sum(double (&acc)[NQ]) {
  __shared__ double sh[kWarps][NQ];
  __shared__ double tot[NQ];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = warp_sum(acc[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) sh[wid][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < NQ) {
    double t = 0.0;
    for (int w = 0; w < kWarps; ++w) t += sh[w][threadIdx.x];
    tot[threadIdx.x] = t;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = tot[q];
  __syncthreads();
}

__device__ double block_max(double v) {
  __shared__ double sh[kWarps];
  __shared__ double tot;
  v = warp_maxd(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = -INFINITY;
    for (int w = 0; w < kWarps; ++w) t = fmax(t, sh[w]);
    tot = t;
  }
  __syncthreads();
  v = tot;
  __syncthreads();
  return v;
}

// True in every thread of the last CTA (of `expected`) to arrive at *ctr; all
// other arrivals' writes are visible to it. The counter is reset for reuse.
__device__ bool arrive_last(int* ctr, int expected) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const int t = atomicAdd(ctr, 1);
    last = (t == expected - 1);
    if (last) *ctr = 0;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__device__ __forceinline__ Entry make_entry(Item* items, int idx, int mode, const float* zeros) {
  Item& it = items[idx];
  Entry e;
  e.item = idx;
  e.mode = mode;
  e.out = nullptr;
  e.pad_ = 0;
  e.nk2 = -__ldcg(&it.c.kappa2);
  switch (mode) {
    case kColB:
      e.w = it.wrow;
      e.o = it.ocol;
      break;
    case kSumK:
      e.w = zeros;
      e.o = nullptr;
      break;
    default:  // kRowA, kFresh
      e.w = it.wcol;
      e.o = it.orow;
      break;
  }
  return e;
}

// Lists of the two iteration passes (run by one CTA): active items, minus the
// row pass of items whose a-update the last gap check already applied.
__device__ void build_iter_lists(const BatchArgs& B) {
  for (int p = threadIdx.x; p < B.n_pairs; p += blockDim.x) {
    const int off = B.pair_off[p], end = B.pair_off[p + 1];
    int nr = 0, nc = 0;
    for (int k = off; k < end; ++k) {
      const int idx = B.pair_items[k];
      Item& it = B.items[idx];
      if (__ldcg(&it.status) != kActive) continue;
      if (!__ldcg(&it.skip_row)) B.row_list[off + nr++] = make_entry(B.items, idx, kRowA, B.zeros);
      B.col_list[off + nc++] = make_entry(B.items, idx, kColB, B.zeros);
    }
    B.row_n[p] = nr;
    B.col_n[p] = nc;
  }
}

// List of the check pass: fresh row sums for final-stage checks and max_iter
// exits, sum exp(-C/eps) for items that entered the final stage.
__device__ void build_check_lists(const BatchArgs& B) {
  for (int p = threadIdx.x; p < B.n_pairs; p += blockDim.x) {
    const int off = B.pair_off[p], end = B.pair_off[p + 1];
    int n = 0;
    for (int k = off; k < end; ++k) {
      const int idx = B.pair_items[k];
      Item& it = B.items[idx];
      const int st = __ldcg(&it.status);
      if (st == kMaxIterPending || (st == kActive && __ldcg(&it.due) && __ldcg(&it.stage) == kScalings))
        B.chk_list[2 * off + n++] = make_entry(B.items, idx, kFresh, B.zeros);
      if (st == kActive && __ldcg(&it.need_sumk) == 1)
        B.chk_list[2 * off + n++] = make_entry(B.items, idx, kSumK, B.zeros);
    }
    B.chk_n[p] = n;
  }
}

// Active-item count for the host, tickets of the next iteration passes.
__device__ void finish_body(const BatchArgs& B) {
  build_iter_lists(B);
  __shared__ int cnt[kWarps];
  int n = 0;
  for (int k = threadIdx.x; k < B.n_items; k += blockDim.x) {
    const int s = __ldcg(&B.items[k].status);
    n += (s == kActive || s == kMaxIterPending) ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) cnt[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kWarps; ++w) t += cnt[w];
    B.active[0] = t;
    B.counters[0] = 0;
    B.counters[1] = 0;
  }
}

// Start of a solve (growth iteration) with p, logp, q in place: stage 0 with
// the single-problem driver's epsilon arithmetic (eps0 * sf / sf). Scalars only.
__device__ void start_solve(Item& it) {
  it.scale_factor = exp(-log(it.epsilon) / kScalings);
  double eps = it.epsilon0 * it.scale_factor;
  eps = eps / it.scale_factor;
  it.eps_i = eps;
  it.c = make_coef(eps, it.lambda1, it.lambda2, it.cost_scale, it.I, it.J, it.q);
  it.maxslot[0] = 0ull;
  it.maxslot[1] = 0ull;
  it.parity = 0;
  it.skip_row = 0;
  it.stage = 0;
  it.batch_cnt = 0;
  it.due = 0;
  it.gap = INFINITY;
  it.threshold = kScalings == 0 ? it.tolerance : 1e-6;
  it.need_sumk = kScalings == 0 ? 1 : 0;
  it.it = 0;
  it.action = kActNone;
  it.status = kActive;
}

// Zero the item's slice of the state with p = G; returns the slice's sum of G.
__device__ double reset_slice(Item& it, const double* G, int rank, int nblk) {
  double sum = 0.0;
  ITEM_LOOP(i, it.I) {
    const double pi = G[i];
    it.u[i] = 0.0;
    it.la[i] = 0.0;
    it.la_old[i] = 0.0;
    it.p[i] = pi;
    it.logp[i] = log(pi);
    it.wrow[i] = 0.f;
    it.orow[i] = 0.f;
    sum += pi;
  }
  ITEM_LOOP(j, it.J) {
    it.v[j] = 0.0;
    it.lb[j] = 0.0;
    it.lb_old[j] = 0.0;
    it.wcol[j] = 0.f;
    it.ocol[j] = 0.f;
  }
  return sum;
}

// Deterministic total of the item's per-CTA partials (fixed order).
__device__ __forceinline__ double item_total(const BatchArgs& B, const Item& it, int q) {
  double t = 0.0;
  for (int b = 0; b < it.nblk; ++b) t += __ldcg(&B.part[(int64_t)(it.first_blk + b) * kNq + q]);
  return t;
}

__global__ void __launch_bounds__(kThreads) init_kernel(BatchArgs B, const double* const* G) {
  const ItemBlock ib = B.blk[blockIdx.x];
  Item& it = B.items[ib.item];
  const int rank = ib.rank, nblk = it.nblk;
  const double* g = G[ib.item];
  if (it.learned) ITEM_LOOP(i, it.I) it.learned[i] = g[i];
  if (rank == 0) {
    // padding of the weight vectors stays 0 (read by the staged passes)
    const int wr = (it.I + 3) & ~3, wc = (it.J + 3) & ~3;
    for (int i = it.I + threadIdx.x; i < wr; i += blockDim.x) it.wrow[i] = 0.f;
    for (int j = it.J + threadIdx.x; j < wc; j += blockDim.x) it.wcol[j] = 0.f;
  }
  double acc[1] = {reset_slice(it, g, rank, nblk)};
  block_sum<1>(acc);
  if (threadIdx.x == 0) B.part[(int64_t)blockIdx.x * kNq] = acc[0];
  if (arrive_last(B.item_ctr + ib.item, nblk) && threadIdx.x == 0) {
    it.q = item_total(B, it, 0) / (double)it.I;
    it.gi = 0;
    it.it_total = 0;
    it.checks = 0;
    it.absorptions = 0;
    it.hit_max_iter = 0;
    start_solve(it);
  }
  if (arrive_last(B.counters + 5, gridDim.x)) {
    finish_body(B);
    if (threadIdx.x == 0) B.counters[2] = 0;
  }
}

// After the two half-steps: tau-absorption (optimal_transport.py:137-141),
// iteration / batch counting, max_iter (:143-145).
__global__ void __launch_bounds__(kThreads) item_kernel(BatchArgs B) {
  const ItemBlock ib = B.blk[blockIdx.x];
  Item& it = B.items[ib.item];
  const int rank = ib.rank, nblk = it.nblk;
  if (it.status == kActive) {
    const int par = it.parity;
    const double mx = __longlong_as_double((long long)it.maxslot[par]);
    const bool absorb = mx > it.tau;
    if (absorb) {
      const double eps = it.c.eps, inv_eps = it.c.inv_eps;
      ITEM_LOOP(i, it.I) {
        const double un = it.u[i] + eps * it.la[i];
        it.u[i] = un;
        it.la[i] = 0.0;
        it.wrow[i] = (float)(un * inv_eps * kLog2e);
      }
      ITEM_LOOP(j, it.J) {
        const double vn = it.v[j] + eps * it.lb[j];
        it.v[j] = vn;
        it.lb[j] = 0.0;
        it.wcol[j] = (float)(vn * inv_eps * kLog2e);
      }
    }
    if (arrive_last(B.item_ctr + ib.item, nblk) && threadIdx.x == 0) {
      it.maxslot[par ^ 1] = 0ull;
      if (absorb) it.absorptions += 1;
      it.skip_row = 0;
      it.it += 1;
      it.parity = par ^ 1;
      it.batch_cnt += 1;
      const int nb = it.stage == kScalings ? it.batch_size : 5;
      if ((double)it.it >= it.max_iter) {
        it.status = kMaxIterPending;
        it.hit_max_iter = 1;
      } else if (it.batch_cnt >= nb) {
        it.due = 1;
      }
    }
  }
  if (arrive_last(B.counters + 3, gridDim.x)) {
    build_check_lists(B);
    if (threadIdx.x == 0) B.counters[2] = 0;
  }
}

// Python's max(x, y): x unless y > x.
__device__ __forceinline__ double py_max(double x, double y) { return (y > x) ? y : x; }

// Stage-exit test / duality gap (optimal_transport.py:146-164), sum exp(-C/eps)
// of a new final stage, and the decision that follows (applied by apply_kernel).
// Partials: [0..6] gap terms or [0..3] stage-test terms, [7] sum of the row
// sums of the current coupling (next growth), [8] sum exp(-C/eps).
__global__ void __launch_bounds__(kThreads) test_kernel(BatchArgs B) {
  const ItemBlock ib = B.blk[blockIdx.x];
  Item& it = B.items[ib.item];
  const int rank = ib.rank, nblk = it.nblk;
  const int st = it.status;
  const bool sumk = st == kActive && it.need_sumk == 1;
  const bool due = st == kActive && it.due;
  if (sumk || due || st == kMaxIterPending) {
    const Coef c = it.c;
    const bool final = it.stage == kScalings;
    double acc[kNq];
#pragma unroll
    for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
    if (sumk) ITEM_LOOP(i, it.I) acc[8] += it.rsum[i];
    if (st == kMaxIterPending) {
      ITEM_LOOP(i, it.I) acc[7] += exp(it.la[i] + it.u[i] * c.inv_eps + it.Lrow[i]);
    } else if (due && final) {
      ITEM_LOOP(i, it.I) {
        const double ui = it.u[i], lai = it.la[i], pi = it.p[i];
        const double x = exp(lai + ui * c.inv_eps + it.Lrow[i] - c.logJ);
        const double ub = ui + c.eps * lai;
        const double at = exp(lai) * exp(ui * c.inv_eps);
        const double f = x * log(x / pi) - x + pi;
        const double conj = c.lambda1 * pi * (exp(-c.eps * log(at) / c.lambda1) - 1.0);
        acc[0] += c.lambda1 * f + conj + ub * x;
        acc[2] += f;
        acc[4] += ub * x;
        acc[6] += x;
      }
      ITEM_LOOP(j, it.J) {
        const double vj = it.v[j], lbj = it.lb[j];
        const double y = exp(lbj + vj * c.inv_eps + it.Lcol[j] - c.logI);
        const double vb = vj + c.eps * lbj;
        const double bt = exp(lbj) * exp(vj * c.inv_eps);
        const double f = y * log(y / c.q) - y + c.q;
        const double conj = c.lambda2 * c.q * (exp(-c.eps * log(bt) / c.lambda2) - 1.0);
        acc[1] += c.lambda2 * f + conj + vb * y;
        acc[3] += f;
        acc[5] += vb * y;
      }
      acc[7] = acc[6];
    } else if (due) {
      ITEM_LOOP(i, it.I) {
        const double e = exp(it.u[i] * c.inv_eps);
        const double ta = exp(it.la[i]) * e;
        const double d = ta - exp(it.la_old[i]) * e;
        acc[0] += d * d;
        acc[1] += ta * ta;
      }
      ITEM_LOOP(j, it.J) {
        const double e = exp(it.v[j] * c.inv_eps);
        const double tb = exp(it.lb[j]) * e;
        const double d = tb - exp(it.lb_old[j]) * e;
        acc[2] += d * d;
        acc[3] += tb * tb;
      }
    }
    block_sum<kNq>(acc);
    if (threadIdx.x < kNq) B.part[(int64_t)blockIdx.x * kNq + threadIdx.x] = acc[threadIdx.x];
    if (arrive_last(B.item_ctr + ib.item, nblk) && threadIdx.x == 0) {
      double t[kNq];
      for (int q = 0; q < kNq; ++q) t[q] = item_total(B, it, q);
      if (sumk) {
        it.sumK = t[8];
        it.need_sumk = 0;
      }
      if (st == kMaxIterPending) {
        it.action = kActFinishMax;
        it.q_next = t[7] / (double)it.I;
      } else if (due) {
        double gap;
        if (final) {
          const double I = (double)it.I, J = (double)it.J;
          const double dx = 1.0 / I, dy = 1.0 / J;
          const double gap_abs = dx * t[0] + dy * t[1];
          const double pri = c.lambda1 * dx * t[2] + c.lambda2 * dy * t[3] + dx * t[4] + dy * t[5] +
                             it.eps_i * (it.sumK / (I * J) - dx * t[6]);
          gap = gap_abs / fabs(pri);
        } else {
          gap = py_max(sqrt(t[0]) / (1.0 + sqrt(t[1])), sqrt(t[2]) / (1.0 + sqrt(t[3])));
        }
        it.checks += 1;
        it.due = 0;
        it.batch_cnt = 0;
        it.gap = gap;
        if (gap > it.threshold) {
          if (final) {
            // The check's row sums are the next iteration's first half-step:
            // apply_kernel applies its a-update and the row pass is skipped.
            it.action = kActCont;
            it.skip_row = 1;
          }
        } else if (!final) {
          // Next epsilon stage (optimal_transport.py:118-125); vectors in apply_kernel.
          it.eps_prev = it.eps_i;
          it.eps_i = it.eps_i / it.scale_factor;
          it.c = make_coef(it.eps_i, it.lambda1, it.lambda2, it.cost_scale, it.I, it.J, it.q);
          it.maxslot[0] = 0ull;
          it.maxslot[1] = 0ull;
          it.parity = 0;
          it.skip_row = 0;
          it.stage += 1;
          it.gap = INFINITY;
          it.threshold = it.stage == kScalings ? it.tolerance : 1e-6;
          if (it.stage == kScalings) it.need_sumk = 1;
          it.action = kActStage;
        } else if (isnan(gap)) {
          it.it_total += it.it;
          it.status = kNonfinite;
        } else {
          it.action = kActFinish;
          it.q_next = t[7] / (double)it.I;
        }
      }
    }
  }
}

// The vector work of test_kernel's decisions, then the next iteration's lists.
__global__ void __launch_bounds__(kThreads) apply_kernel(BatchArgs B) {
  const ItemBlock ib = B.blk[blockIdx.x];
  Item& it = B.items[ib.item];
  const int rank = ib.rank, nblk = it.nblk;
  const int act = it.action;
  if (act != kActNone) {
    const Coef c = it.c;
    if (act == kActCont) {
      double lmax = -INFINITY;
      ITEM_LOOP(i, it.I) lmax = fmax(lmax, item_a_update(it, i, it.Lrow[i]));
      lmax = block_max(lmax);
      if (threadIdx.x == 0) atomic_max_nonneg(&it.maxslot[it.parity], exp(lmax));
    } else if (act == kActStage) {
      // absorb with the old epsilon, a = b = 1; offsets scale with 1/eps
      const double eps_old = it.eps_prev;
      const double inv_new = 1.0 / it.eps_i;
      const float ratio = (float)(eps_old / it.eps_i);
      ITEM_LOOP(i, it.I) {
        const double un = it.u[i] + eps_old * it.la[i];
        it.u[i] = un;
        it.la[i] = 0.0;
        it.la_old[i] = 0.0;
        it.wrow[i] = (float)(un * inv_new * kLog2e);
        it.orow[i] *= ratio;
      }
      ITEM_LOOP(j, it.J) {
        const double vn = it.v[j] + eps_old * it.lb[j];
        it.v[j] = vn;
        it.lb[j] = 0.0;
        it.lb_old[j] = 0.0;
        it.wcol[j] = (float)(vn * inv_new * kLog2e);
        it.ocol[j] *= ratio;
      }
    } else {
      // End of a solve: the reference returns R / J, or R at max_iter.
      const double log_scale = act == kActFinishMax ? 0.0 : -c.logJ;
      if (it.gi + 1 < it.growth_iters) {
        // next growth iteration: G = row sums of this coupling, fresh state
        double* nextG = it.learned ? it.learned + (int64_t)(it.gi + 1) * it.I : it.rsum;
        ITEM_LOOP(i, it.I) nextG[i] = exp(it.la[i] + it.u[i] * c.inv_eps + it.Lrow[i] + log_scale);
        reset_slice(it, nextG, rank, nblk);
      } else {
        ITEM_LOOP(i, it.I) {
          it.row_sums[i] = exp(it.la[i] + it.u[i] * c.inv_eps + it.Lrow[i] + log_scale);
          it.ubar[i] = it.u[i] + c.eps * it.la[i];
        }
        ITEM_LOOP(j, it.J) it.vbar[j] = it.v[j] + c.eps * it.lb[j];
      }
    }
    if (arrive_last(B.item_ctr + ib.item, nblk) && threadIdx.x == 0) {
      if (act == kActFinish || act == kActFinishMax) {
        it.it_total += it.it;
        if (it.gi + 1 < it.growth_iters) {
          it.gi += 1;
          it.q = it.q_next;
          start_solve(it);
        } else {
          it.status = act == kActFinishMax ? kDoneMaxIter : kDone;
        }
      }
      it.action = kActNone;
    }
  }
  if (arrive_last(B.counters + 7, gridDim.x)) finish_body(B);
}

// ---------------------------------------------------------------------------
// Cost transpose, dense coupling from potentials.
// ---------------------------------------------------------------------------
__global__ void transpose_kernel(const float* __restrict__ C, int64_t I, int64_t J, int64_t ldc,
                                 float* __restrict__ CT, int64_t ldct) {
  __shared__ float tile[32][33];
  const int64_t j0 = (int64_t)blockIdx.x * 32, i0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = i0 + r, j = j0 + threadIdx.x;
    tile[r][threadIdx.x] = (i < I && j < J) ? C[i * ldc + j] : INFINITY;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t j = j0 + r, i = i0 + threadIdx.x;
    if (j < J && i < ldct) CT[j * ldct + i] = (i < I) ? tile[threadIdx.x][r] : INFINITY;
  }
}

__global__ void coupling_potentials_kernel(const float* __restrict__ C, int64_t I, int64_t J, int64_t ldc,
                                           double kappa, double inv_eps, const double* __restrict__ ubar,
                                           const double* __restrict__ vbar, double log_scale,
                                           double* __restrict__ out) {
  for (int64_t i = blockIdx.y; i < I; i += gridDim.y) {
    const double wr = ubar[i] * inv_eps + log_scale;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < J; j += (int64_t)gridDim.x * blockDim.x)
      out[i * J + j] = exp(wr + vbar[j] * inv_eps - kappa * (double)C[i * ldc + j]);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using PassFn = void (*)(PassArgs);

struct PassCfg {
  int kg, rw;
  PassFn spec, exact;
};

static const PassCfg kCfgs[] = {
    {8, 1, pass_kernel<8, 1, true>, pass_kernel<8, 1, false>},
    {8, 2, pass_kernel<8, 2, true>, pass_kernel<8, 2, false>},
    {16, 1, pass_kernel<16, 1, true>, pass_kernel<16, 1, false>},
    {16, 2, pass_kernel<16, 2, true>, pass_kernel<16, 2, false>},
    {8, 4, pass_kernel<8, 4, true>, pass_kernel<8, 4, false>},
    {13, 2, pass_kernel<13, 2, true>, pass_kernel<13, 2, false>},
};
constexpr int kNumCfgs = sizeof(kCfgs) / sizeof(kCfgs[0]);

static int pass_grid(PassFn fn) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreads, 0) != cudaSuccess || occ <= 0) occ = 2;
  return sm_count() * occ;
}

// Tiles of one direction for rows_per_tile rows, largest work first.
static std::vector<Tile> make_tiles(const std::vector<int>& rows, const std::vector<int>& cols,
                                    const std::vector<int>& kp, int rows_per_tile) {
  std::vector<std::pair<double, Tile>> t;
  for (size_t p = 0; p < rows.size(); ++p)
    for (int r = 0; r < rows[p]; r += rows_per_tile)
      t.push_back({(double)cols[p] * std::max(1, kp[p]), Tile{(int)p, r}});
  std::stable_sort(t.begin(), t.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  std::vector<Tile> out(t.size());
  for (size_t i = 0; i < t.size(); ++i) out[i] = t[i].second;
  return out;
}

// CTAs of the per-item kernels for an item of I + J points.
static inline int item_blocks(int64_t I, int64_t J) {
  return (int)std::min<int64_t>(32, std::max<int64_t>(1, (I + J + 2047) / 2048));
}

struct Layout {
  ItemBlock* blk;
  int nblk;
  int* item_ctr;
  double* part;
  Item* items;
  Seg* segs;
  Tile* tiles[2][3];  // [dir][rw_slot(rw)]
  int ntiles[2][3];
  int *pair_items, *pair_off, *list_off, *row_n, *col_n, *chk_n, *counters, *active;
  Entry *row_list, *col_list, *chk_list;
  float* zeros;
  const double** G;
  size_t bytes;
};

static inline int64_t round4(int64_t n) { return (n + 3) & ~int64_t(3); }

// Rows per warp of a pass configuration (1, 2 or 4) -> its tile table.
constexpr int kRowsPerWarp[3] = {1, 2, 4};
static inline int rw_slot(int rw) { return rw == 4 ? 2 : rw - 1; }

// Workspace layout; with base == nullptr only sizes. Fills host-side item
// pointers when `host_items` is given.
static size_t layout(char* base, const wotg_pair* pairs, int np, const wotg_item* items, int ni, Layout& L,
                     std::vector<Item>* host_items) {
  Bump b{base, 0};
  L.items = b.take<Item>(ni);
  L.nblk = 0;
  for (int k = 0; k < ni; ++k) L.nblk += item_blocks(pairs[items[k].pair].I, pairs[items[k].pair].J);
  L.blk = b.take<ItemBlock>(L.nblk);
  L.item_ctr = b.take<int>(ni);
  L.part = b.take<double>((size_t)L.nblk * kNq);
  L.segs = b.take<Seg>(2 * (size_t)np);
  int64_t maxcols = 4;
  std::vector<int> rows0(np), cols0(np), kp(np, 0);
  for (int p = 0; p < np; ++p) {
    rows0[p] = (int)pairs[p].I;
    cols0[p] = (int)pairs[p].J;
    maxcols = std::max(maxcols, round4(std::max(pairs[p].J, pairs[p].I)));
  }
  for (int k = 0; k < ni; ++k) kp[items[k].pair] += 1;
  for (int d = 0; d < 2; ++d)
    for (int sl = 0; sl < 3; ++sl) {
      const int rw = kRowsPerWarp[sl];
      size_t n = 0;
      for (int p = 0; p < np; ++p) {
        const int rows = d == 0 ? rows0[p] : cols0[p];
        n += (size_t)((rows + 8 * rw - 1) / (8 * rw));
      }
      L.ntiles[d][sl] = (int)n;
      L.tiles[d][sl] = b.take<Tile>(n);
    }
  L.pair_items = b.take<int>(ni);
  L.pair_off = b.take<int>(np + 1);
  L.list_off = L.pair_off;
  L.row_n = b.take<int>(np);
  L.col_n = b.take<int>(np);
  L.chk_n = b.take<int>(np);
  L.row_list = b.take<Entry>(ni);
  L.col_list = b.take<Entry>(ni);
  L.chk_list = b.take<Entry>(2 * (size_t)ni);
  L.counters = b.take<int>(8);
  L.active = b.take<int>(4);
  L.zeros = b.take<float>(maxcols);
  L.G = b.take<const double*>(ni);
  for (int k = 0; k < ni; ++k) {
    const wotg_pair& pr = pairs[items[k].pair];
    const int64_t I = pr.I, J = pr.J;
    Item it;
    std::memset(&it, 0, sizeof(it));
    it.u = b.take<double>(I);
    it.la = b.take<double>(I);
    it.la_old = b.take<double>(I);
    it.logp = b.take<double>(I);
    it.p = b.take<double>(I);
    it.Lrow = b.take<double>(I);
    it.rsum = b.take<double>(I);
    it.v = b.take<double>(J);
    it.lb = b.take<double>(J);
    it.lb_old = b.take<double>(J);
    it.Lcol = b.take<double>(J);
    it.wrow = b.take<float>(round4(I));
    it.orow = b.take<float>(I);
    it.wcol = b.take<float>(round4(J));
    it.ocol = b.take<float>(J);
    if (host_items) (*host_items)[k] = it;
  }
  L.bytes = b.off + 256;
  return L.bytes;
}

static int validate(const wotg_pair* pairs, int np, const wotg_item* items, int ni) {
  if (!pairs || !items || np <= 0 || ni <= 0) return WOTG_BADARG;
  for (int p = 0; p < np; ++p) {
    const wotg_pair& q = pairs[p];
    if (q.I <= 0 || q.J <= 0 || q.I > (1 << 30) || q.J > (1 << 30)) return WOTG_BADARG;
    if (!q.C || !q.CT || !q.G || q.ldc < q.J || q.ldct < q.I || (q.ldc & 3) || (q.ldct & 3)) return WOTG_BADARG;
    if ((reinterpret_cast<uintptr_t>(q.C) & 15) || (reinterpret_cast<uintptr_t>(q.CT) & 15)) return WOTG_BADARG;
    if (!(q.cost_scale > 0)) return WOTG_BADARG;
  }
  for (int k = 0; k < ni; ++k) {
    const wotg_item& it = items[k];
    const wotg_params& P = it.params;
    if (it.pair < 0 || it.pair >= np) return WOTG_BADARG;
    if (P.solver != WOTG_SOLVER_DUALITY_GAP || P.batch_size < 1 || P.growth_iters < 1) return WOTG_BADARG;
    if (!(P.epsilon > 0) || !(P.epsilon0 > 0) || !(P.lambda1 > 0) || !(P.lambda2 > 0)) return WOTG_BADARG;
    if (it.row_offset < 0 || it.col_offset < 0 || it.growth_offset < 0) return WOTG_BADARG;
  }
  return WOTG_OK;
}

// Autotuner: fastest (KG, RW) of the speculative pass for one direction of a
// batch, timed on the batch's own segments with every item of every pair
// (zero weights, no epilogue). Cached per batch shape.
struct TuneKey {
  int dir, np, ni;
  long long work;
  bool operator<(const TuneKey& o) const {
    return std::tie(dir, np, ni, work) < std::tie(o.dir, o.np, o.ni, o.work);
  }
};
struct Tuned {
  int cfg;
  float ms;   // measured time of one pass of that configuration
};
static std::map<TuneKey, Tuned> g_tuned;
static std::mutex g_tune_mu;
// Replay profile of the last wotg_solve_batched call on this host thread:
// (active items read after replay n - 1, host milliseconds between successive
// waits) per replay (diagnostic, wotg_batch_replay_profile).
static thread_local std::vector<std::pair<int, float>> g_replay_prof;
// The last batch's choice and measured pass time per direction (wotg_batch_pass_timing).
static Tuned g_last_tuned[2] = {{-1, 0.f}, {-1, 0.f}};

static int autotune(const Layout& L, const int* chk_off, int dir, int np, int ni, long long work,
                    const std::vector<Entry>& probe, const std::vector<int>& probe_n, cudaStream_t st,
                    int* choice) {
  const TuneKey key{dir, np, ni, work};
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto f = g_tuned.find(key);
    if (f != g_tuned.end()) {
      *choice = f->second.cfg;
      g_last_tuned[dir] = f->second;
      return WOTG_OK;
    }
  }
  WOTG_CUDA(cudaMemcpyAsync(L.chk_list, probe.data(), probe.size() * sizeof(Entry), cudaMemcpyHostToDevice, st));
  WOTG_CUDA(cudaMemcpyAsync(L.chk_n, probe_n.data(), probe_n.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  cudaEvent_t e0, e1;
  WOTG_CUDA(cudaEventCreate(&e0));
  WOTG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_i = 0;
  int status = WOTG_OK;
  for (int c = 0; c < kNumCfgs && status == WOTG_OK; ++c) {
    const PassArgs A{L.segs,    dir,      L.tiles[dir][rw_slot(kCfgs[c].rw)], L.ntiles[dir][rw_slot(kCfgs[c].rw)],
                     L.chk_n,   L.chk_list, chk_off, L.items, L.counters + 6};
    float t_min = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaError_t e = cudaMemsetAsync(L.counters + 6, 0, sizeof(int), st);
      if (e == cudaSuccess) e = cudaEventRecord(e0, st);
      if (e == cudaSuccess) {
        kCfgs[c].spec<<<pass_grid(kCfgs[c].spec), kThreads, 0, st>>>(A);
        count_launch();
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        set_last_error("batch autotuner", e);
        status = WOTG_CUDA_ERROR;
        break;
      }
      if (rep > 0) t_min = std::min(t_min, ms);
    }
    if (t_min < best) {
      best = t_min;
      best_i = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status) return status;
  *choice = best_i;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tuned[key] = Tuned{best_i, best};
  g_last_tuned[dir] = Tuned{best_i, best};
  return WOTG_OK;
}

}  // namespace batch
}  // namespace wotg

using namespace wotg;
using namespace wotg::batch;

extern "C" int wotg_transpose_cost(const float* C, int64_t I, int64_t J, int64_t ldc, float* CT, int64_t ldct,
                                   void* stream) {
  if (!C || !CT || I <= 0 || J <= 0 || ldc < J || ldct < I || (ldct & 3)) return WOTG_BADARG;
  dim3 grid((unsigned)((J + 31) / 32), (unsigned)((ldct + 31) / 32));
  if (grid.y > 65535) return WOTG_BADARG;
  transpose_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(C, I, J, ldc, CT, ldct);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

extern "C" int wotg_coupling_from_potentials(const float* C, int64_t I, int64_t J, int64_t ldc, double cost_scale,
                                             double eps, const double* u_bar, const double* v_bar, double log_scale,
                                             double* out, void* stream) {
  if (!C || !u_bar || !v_bar || !out || I <= 0 || J <= 0 || ldc < J || !(eps > 0) || !(cost_scale > 0))
    return WOTG_BADARG;
  dim3 grid((unsigned)std::min<int64_t>((J + 255) / 256, 16), (unsigned)std::min<int64_t>(I, 65535));
  coupling_potentials_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(C, I, J, ldc, cost_scale / eps, 1.0 / eps,
                                                                      u_bar, v_bar, log_scale, out);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

extern "C" size_t wotg_batch_workspace_bytes(const wotg_pair* pairs, int32_t n_pairs, const wotg_item* items,
                                             int32_t n_items) {
  if (validate(pairs, n_pairs, items, n_items) != WOTG_OK) return 0;
  Layout L{};
  // + probe list offsets for the autotuner (n_pairs + 1 ints)
  return layout(nullptr, pairs, n_pairs, items, n_items, L, nullptr) + 256 + sizeof(int) * ((size_t)n_pairs + 1);
}

namespace {
constexpr int kBodies = 8;  // iterations of the whole batch per graph launch
}

extern "C" int wotg_solve_batched(const wotg_pair* pairs, int32_t n_pairs, const wotg_item* items, int32_t n_items,
                                  double* u_bar, double* v_bar, double* row_sums, double* learned_growth,
                                  wotg_stats* stats, int32_t* statuses, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  int s = validate(pairs, n_pairs, items, n_items);
  if (s) return s;
  if (!u_bar || !v_bar || !row_sums) return WOTG_BADARG;
  const size_t need = wotg_batch_workspace_bytes(pairs, n_pairs, items, n_items);
  if (!workspace || workspace_bytes < need) return WOTG_WORKSPACE;
  const int np = n_pairs, ni = n_items;

  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  Layout L{};
  std::vector<Item> hi(ni);
  layout(base, pairs, np, items, ni, L, &hi);
  // check-list offsets live right after the layout
  int* probe_off = reinterpret_cast<int*>(base + ((L.bytes - 256 + 255) & ~size_t(255)));

  // Host tables.
  std::vector<Seg> segs(2 * (size_t)np);
  std::vector<int> rows0(np), cols0(np), kp(np, 0);
  for (int p = 0; p < np; ++p) {
    segs[2 * p] = Seg{pairs[p].C, pairs[p].ldc, (int)pairs[p].I, (int)pairs[p].J};
    segs[2 * p + 1] = Seg{pairs[p].CT, pairs[p].ldct, (int)pairs[p].J, (int)pairs[p].I};
    rows0[p] = (int)pairs[p].I;
    cols0[p] = (int)pairs[p].J;
  }
  for (int k = 0; k < ni; ++k) kp[items[k].pair] += 1;
  std::vector<int> pair_off(np + 2, 0), pair_items(ni);
  for (int p = 0; p < np; ++p) pair_off[p + 1] = pair_off[p] + kp[p];
  {
    std::vector<int> fill(pair_off.begin(), pair_off.begin() + np);
    for (int k = 0; k < ni; ++k) pair_items[fill[items[k].pair]++] = k;
  }
  std::vector<const double*> G(ni);
  std::vector<ItemBlock> blk;
  long long work = 0;
  for (int k = 0; k < ni; ++k) {
    const wotg_item& in = items[k];
    const wotg_pair& pr = pairs[in.pair];
    const wotg_params& P = in.params;
    Item& it = hi[k];
    it.pair = in.pair;
    it.I = (int)pr.I;
    it.J = (int)pr.J;
    it.cost_scale = pr.cost_scale;
    it.epsilon = P.epsilon;
    it.lambda1 = P.lambda1;
    it.lambda2 = P.lambda2;
    it.epsilon0 = P.epsilon0;
    it.tau = P.tau;
    it.tolerance = P.tolerance;
    it.max_iter = P.max_iter;
    it.batch_size = P.batch_size;
    it.growth_iters = P.growth_iters;
    it.ubar = u_bar + in.row_offset;
    it.vbar = v_bar + in.col_offset;
    it.row_sums = row_sums + in.row_offset;
    it.learned = learned_growth ? learned_growth + in.growth_offset : nullptr;
    it.c.kappa2 = (float)(pr.cost_scale / P.epsilon * kLog2e);
    it.first_blk = (int)blk.size();
    it.nblk = item_blocks(pr.I, pr.J);
    for (int r = 0; r < it.nblk; ++r) blk.push_back(ItemBlock{k, r});
    G[k] = pr.G;
    work += (long long)pr.I * pr.J;
  }

  cudaStream_t user = (cudaStream_t)stream;
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev_in = nullptr, ev_done[2] = {nullptr, nullptr};
  int* pinned = nullptr;
  int status = WOTG_OK;
  auto cleanup = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev_done)
      if (e) cudaEventDestroy(e);
    if (ev_in) cudaEventDestroy(ev_in);
    if (cs) cudaStreamDestroy(cs);
    if (pinned) cudaFreeHost(pinned);
  };
#define WOTG_BCUDA(call)                    \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) {                \
      ::wotg::set_last_error(#call, e_);    \
      cleanup();                            \
      return WOTG_CUDA_ERROR;               \
    }                                       \
  } while (0)

  WOTG_BCUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  WOTG_BCUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  for (auto& e : ev_done) WOTG_BCUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  WOTG_BCUDA(cudaMallocHost(&pinned, 2 * sizeof(int)));
  WOTG_BCUDA(cudaEventRecord(ev_in, user));
  WOTG_BCUDA(cudaStreamWaitEvent(cs, ev_in, 0));

  // Upload tables (pageable host memory: these copies complete before return).
  WOTG_BCUDA(cudaMemcpyAsync(L.items, hi.data(), sizeof(Item) * ni, cudaMemcpyHostToDevice, cs));
  WOTG_BCUDA(cudaMemcpyAsync(L.segs, segs.data(), sizeof(Seg) * segs.size(), cudaMemcpyHostToDevice, cs));
  std::vector<Tile> tiles[2][3];
  for (int d = 0; d < 2; ++d)
    for (int sl = 0; sl < 3; ++sl) {
      tiles[d][sl] = make_tiles(d == 0 ? rows0 : cols0, d == 0 ? cols0 : rows0, kp, 8 * kRowsPerWarp[sl]);
      WOTG_BCUDA(cudaMemcpyAsync(L.tiles[d][sl], tiles[d][sl].data(), sizeof(Tile) * tiles[d][sl].size(),
                                 cudaMemcpyHostToDevice, cs));
    }
  WOTG_BCUDA(cudaMemcpyAsync(L.pair_items, pair_items.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, cs));
  WOTG_BCUDA(cudaMemcpyAsync(L.pair_off, pair_off.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice, cs));
  WOTG_BCUDA(cudaMemcpyAsync(L.G, G.data(), sizeof(double*) * ni, cudaMemcpyHostToDevice, cs));
  WOTG_BCUDA(cudaMemsetAsync(L.counters, 0, 8 * sizeof(int), cs));
  WOTG_BCUDA(cudaMemsetAsync(L.item_ctr, 0, ni * sizeof(int), cs));
  WOTG_BCUDA(cudaMemcpyAsync(L.blk, blk.data(), sizeof(ItemBlock) * blk.size(), cudaMemcpyHostToDevice, cs));
  size_t maxcols = 4;
  for (int p = 0; p < np; ++p) maxcols = std::max<size_t>(maxcols, round4(std::max(pairs[p].I, pairs[p].J)));
  WOTG_BCUDA(cudaMemsetAsync(L.zeros, 0, maxcols * sizeof(float), cs));

  BatchArgs B{L.items,  ni,         np,      L.pair_items, L.pair_off, L.row_n, L.row_list,
              L.col_n,  L.col_list, L.chk_n, L.chk_list,   L.counters, L.active, L.zeros,
              L.blk,    L.item_ctr, L.part};
  const int nblk = L.nblk;

  // The check list has 2 K_p slots per pair: its offsets are 2 * pair_off.
  int* chk_off = probe_off;
  {
    std::vector<int> h(np + 1);
    for (int p = 0; p <= np; ++p) h[p] = 2 * pair_off[p];
    WOTG_BCUDA(cudaMemcpyAsync(chk_off, h.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice, cs));
  }
  // Autotune each direction on probe lists (all items of each pair, zero weights).
  int cfg[2] = {0, 0};
  {
    std::vector<Entry> probe(2 * (size_t)ni);
    std::vector<int> probe_n(np);
    for (int p = 0; p < np; ++p) {
      probe_n[p] = kp[p];
      for (int k = pair_off[p]; k < pair_off[p + 1]; ++k) {
        const int idx = pair_items[k];
        Entry e{};
        e.w = L.zeros;
        e.o = nullptr;
        e.out = nullptr;
        e.nk2 = -hi[idx].c.kappa2;
        e.item = idx;
        e.mode = kNone;
        probe[2 * pair_off[p] + (k - pair_off[p])] = e;
      }
    }
    for (int d = 0; d < 2; ++d) {
      s = autotune(L, chk_off, d, np, ni, work, probe, probe_n, cs, &cfg[d]);
      if (s) {
        cleanup();
        return s;
      }
    }
  }

  init_kernel<<<nblk, kThreads, 0, cs>>>(B, L.G);
  WOTG_LAUNCHED();

  const PassCfg& c0 = kCfgs[cfg[0]];
  const PassCfg& c1 = kCfgs[cfg[1]];
  PassArgs Arow{L.segs, 0, L.tiles[0][rw_slot(c0.rw)], L.ntiles[0][rw_slot(c0.rw)], L.row_n, L.row_list, L.pair_off,
                L.items, L.counters + 0};
  PassArgs Acol{L.segs, 1, L.tiles[1][rw_slot(c1.rw)], L.ntiles[1][rw_slot(c1.rw)], L.col_n, L.col_list, L.pair_off,
                L.items, L.counters + 1};
  PassArgs Achk{L.segs, 0, L.tiles[0][rw_slot(c0.rw)], L.ntiles[0][rw_slot(c0.rw)], L.chk_n, L.chk_list, chk_off,
                L.items, L.counters + 2};
  const int grid_row = pass_grid(c0.spec), grid_col = pass_grid(c1.spec);

  WOTG_BCUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  for (int b = 0; b < kBodies; ++b) {
    c0.spec<<<grid_row, kThreads, 0, cs>>>(Arow);
    c1.spec<<<grid_col, kThreads, 0, cs>>>(Acol);
    item_kernel<<<nblk, kThreads, 0, cs>>>(B);
    c0.spec<<<grid_row, kThreads, 0, cs>>>(Achk);
    test_kernel<<<nblk, kThreads, 0, cs>>>(B);
    apply_kernel<<<nblk, kThreads, 0, cs>>>(B);
  }
  {
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (e != cudaSuccess) {
      set_last_error("cudaStreamEndCapture", e);
      cleanup();
      return WOTG_CUDA_ERROR;
    }
  }
  WOTG_BCUDA(cudaGetLastError());
  WOTG_BCUDA(cudaGraphInstantiate(&exec, graph, 0));

  // Replay until no item is active; the active count of launch n is read while
  // launch n + 1 runs.
  double max_iters = 0.0;
  for (int k = 0; k < ni; ++k)
    max_iters = std::max(max_iters, items[k].params.max_iter * std::max(1, items[k].params.growth_iters));
  const double max_launches = std::min(max_iters, 1e12) / kBodies + 4;
  long long launched = 0;
  g_replay_prof.clear();
  auto t_last = std::chrono::steady_clock::now();
  for (;;) {
    const int slot = (int)(launched & 1);
    WOTG_BCUDA(cudaGraphLaunch(exec, cs));
    for (int q = 0; q < kBodies * 6; ++q) count_launch();
    WOTG_BCUDA(cudaMemcpyAsync(pinned + slot, L.active, sizeof(int), cudaMemcpyDeviceToHost, cs));
    WOTG_BCUDA(cudaEventRecord(ev_done[slot], cs));
    ++launched;
    if (launched >= 2) {
      const int prev = slot ^ 1;
      WOTG_BCUDA(cudaEventSynchronize(ev_done[prev]));
      // replay profile: the host waits on replay n - 1 while replay n runs, so the
      // interval between these waits is one replay's device time once GPU-bound
      const auto t_now = std::chrono::steady_clock::now();
      g_replay_prof.push_back(std::make_pair(pinned[prev],
                                             std::chrono::duration<float, std::milli>(t_now - t_last).count()));
      t_last = t_now;
      if (pinned[prev] == 0) break;
    }
    if ((double)launched > max_launches) {
      set_last_message("wotg_solve_batched: iteration bound exceeded");
      status = WOTG_CUDA_ERROR;
      break;
    }
  }
  WOTG_BCUDA(cudaMemcpyAsync(hi.data(), L.items, sizeof(Item) * ni, cudaMemcpyDeviceToHost, cs));
  WOTG_BCUDA(cudaStreamSynchronize(cs));
  for (int k = 0; k < ni; ++k) {
    const Item& it = hi[k];
    if (stats) {
      wotg_stats& o = stats[k];
      o.iterations = it.it_total;
      o.absorptions = it.absorptions;
      o.checks = it.checks;
      o.gap = it.gap;
      o.final_epsilon = it.eps_i;
      o.hit_max_iter = it.hit_max_iter;
      o.exact_rows = 0;
    }
    if (statuses) {
      int32_t r = WOTG_OK;
      if (it.status == kNonfinite)
        r = WOTG_NONFINITE;
      else if (it.hit_max_iter)
        r = WOTG_MAX_ITER;
      else if (it.status != kDone)
        r = WOTG_CUDA_ERROR;
      statuses[k] = r;
    }
  }
  WOTG_BCUDA(cudaEventRecord(ev_in, cs));
  WOTG_BCUDA(cudaStreamWaitEvent(user, ev_in, 0));
  cleanup();
#undef WOTG_BCUDA
  return status;
}

extern "C" int32_t wotg_batch_replay_profile(int32_t* active, float* ms, int32_t cap) {
  const int32_t n = (int32_t)std::min<size_t>(g_replay_prof.size(), (size_t)std::max(0, cap));
  for (int32_t k = 0; k < n; ++k) {
    if (active) active[k] = g_replay_prof[k].first;
    if (ms) ms[k] = g_replay_prof[k].second;
  }
  return (int32_t)g_replay_prof.size();
}

extern "C" size_t wotg_lse_matvec_multi_workspace_bytes(int64_t I, int32_t K) {
  if (I <= 0 || K <= 0) return 0;
  Bump b{nullptr, 0};
  b.take<Seg>(2);
  b.take<Tile>((size_t)(I + 7) / 8);
  b.take<Entry>(K);
  b.take<int>(8);
  return b.off + 256;
}

extern "C" int wotg_lse_matvec_multi(const float* C, int64_t I, int64_t J, int64_t ldc, const float* W,
                                     int64_t ldw, const float* kappa2, int32_t K, double* L, int64_t ldl,
                                     void* workspace, size_t workspace_bytes, void* stream) {
  if (!C || !W || !kappa2 || !L || I <= 0 || J <= 0 || K <= 0 || ldc < J || (ldc & 3) || ldw < round4(J) ||
      (ldw & 3) || ldl < I || I > (1 << 30) || J > (1 << 30))
    return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(C) & 15) || (reinterpret_cast<uintptr_t>(W) & 15)) return WOTG_BADARG;
  for (int k = 0; k < K; ++k)
    if (!(kappa2[k] > 0.f)) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_lse_matvec_multi_workspace_bytes(I, K)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  Seg* segs = b.take<Seg>(2);
  const PassCfg& cfg = kCfgs[0];  // 8 entries per group, one row per warp
  Tile* tiles = b.take<Tile>((size_t)(I + 7) / 8);
  Entry* ent = b.take<Entry>(K);
  int* ints = b.take<int>(8);  // [0] n entries, [1] list offset 0, [2] counter
  Seg hs[2] = {Seg{C, ldc, (int)I, (int)J}, Seg{C, ldc, (int)I, (int)J}};
  std::vector<Tile> ht((size_t)(I + 7) / 8);
  for (size_t t = 0; t < ht.size(); ++t) ht[t] = Tile{0, (int)(t * 8)};
  std::vector<Entry> he(K);
  for (int k = 0; k < K; ++k) {
    he[k] = Entry{W + (int64_t)k * ldw, nullptr, L + (int64_t)k * ldl, -kappa2[k], 0, kOut, 0};
  }
  const int hi[4] = {K, 0, 0, 0};
  WOTG_CUDA(cudaMemcpyAsync(segs, hs, sizeof(hs), cudaMemcpyHostToDevice, st));
  WOTG_CUDA(cudaMemcpyAsync(tiles, ht.data(), sizeof(Tile) * ht.size(), cudaMemcpyHostToDevice, st));
  WOTG_CUDA(cudaMemcpyAsync(ent, he.data(), sizeof(Entry) * K, cudaMemcpyHostToDevice, st));
  WOTG_CUDA(cudaMemcpyAsync(ints, hi, sizeof(hi), cudaMemcpyHostToDevice, st));
  PassArgs A{segs, 0, tiles, (int)ht.size(), ints + 0, ent, ints + 1, nullptr, ints + 2};
  cfg.exact<<<pass_grid(cfg.exact), kThreads, 0, st>>>(A);
  WOTG_LAUNCHED();
  // the host tables above are pageable: the copies finished before this returns
  return WOTG_OK;
}

extern "C" int wotg_batch_pass_timing(float* ms_row, float* ms_col, int32_t* kg_rw) {
  using namespace wotg::batch;
  std::lock_guard<std::mutex> g(g_tune_mu);
  if (g_last_tuned[0].cfg < 0 || g_last_tuned[1].cfg < 0) return WOTG_BADARG;
  if (ms_row) *ms_row = g_last_tuned[0].ms;
  if (ms_col) *ms_col = g_last_tuned[1].ms;
  if (kg_rw) {
    kg_rw[0] = kCfgs[g_last_tuned[0].cfg].kg;
    kg_rw[1] = kCfgs[g_last_tuned[0].cfg].rw;
    kg_rw[2] = kCfgs[g_last_tuned[1].cfg].kg;
    kg_rw[3] = kCfgs[g_last_tuned[1].cfg].rw;
  }
  return WOTG_OK;
}
