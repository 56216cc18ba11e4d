// wotg_sinkhorn.cu — stabilised unbalanced Sinkhorn on a materialised FP32 cost (sm_103a).
//
// Reference: wot/ot/optimal_transport.py (wot 1.0.8)
//   compute_transport_matrix        :10-33   -> wotg_compute_transport_matrix (growth loop)
//   optimal_transport_duality_gap   :67-164  -> solve_duality_gap
//   transport_stablev2              :167-236 -> solve_fixed_iters
//   primal / dual                   :45-62   -> gap_partial_kernel (O(I+J), see below)
//
// State. The reference keeps FP64 absorbed potentials u, v, scalings a, b and
// the stabilised kernel K = exp((u_i - C_ij + v_j)/eps) as a dense matrix that
// it rebuilds at every absorption and epsilon change. Here the dense object is
// the FP32 cost C (written once per day pair) and the scalings are kept in the
// log domain (la = log a, lb = log b, FP64), so one half-step is
//   log(K (b dy))_i = u_i/eps + log sum_j exp(v_j/eps + lb_j - cost_scale C_ij/eps) - log J
// evaluated as a streaming base-2 log-sum-exp over the row of C, followed by the
// reference's update a = (p / K(b dy))^alpha1 exp(-u/(lambda1+eps)) in FP64.
// Absorption (u += eps log a, a = 1) then only touches O(I+J) vectors and no
// matrix is ever rebuilt; the sequence of (u, v, a, b) is the reference's.
//
// Duality gap. With R = diag(a) K diag(b) the identity
//   eps R_ij log R_ij + R_ij C_ij = R_ij (ubar_i + vbar_j),  ubar = u + eps log a,
// turns the reference's primal - dual (two I x J passes with log) into sums over
// the row sums x = R dy and column sums y = R^T dx only:
//   primal - dual = F1(x) + F2(y) + F1*(-eps log a~) + F2*(-eps log b~) + dx<ubar,x> + dy<vbar,y>
// (a~ = a exp(u/eps) evaluated as the reference does, overflow included), and
//   primal = F1(x) + F2(y) + dx<ubar,x> + dy<vbar,y> + eps (sum(exp(-C/eps))/(IJ) - dx sum x).
// The row sums with the current b are exactly the next iteration's first
// half-step, so a gap check costs one row pass that the next iteration reuses.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "wotg_coef.cuh"
#include "wotg_common.cuh"
#include "wotg_onthefly.cuh"
#include "wotg_tc_kernel.cuh"

namespace wotg {

// Per-solve vectors in the caller's workspace.
struct Vecs {
  double* u;       // I   absorbed potential (reference u)
  double* v;       // J
  double* la;      // I   log a
  double* lb;      // J   log b
  double* la_old;  // I   log a at the start of the last iteration (stage-exit test)
  double* lb_old;  // J
  double* logp;    // I   log p (p = G of this growth iteration)
  double* p;       // I
  double* Lrow;    // I   log sum_j exp(v_j/eps + lb_j - kappa C_ij)
  double* Lcol;    // J   log sum_i exp(u_i/eps + la_i - kappa C_ij)
  float* wrow;     // I   (u_i/eps + la_i) * log2(e), FP32 operand of the column pass (hi part, see split_weight)
  float* wcol;     // ldc (v_j/eps + lb_j) * log2(e), zero in padding columns (hi part)
  float* wrow_lo;  // I   remainders of the weights (lo parts)
  float* wcol_lo;  // ldc
  float4* rowc;    // I   per-row constants of the dense coupling (coupling_rows_kernel)
  float2* part;    // nrb x ldc column-pass partials (m, s) in base 2
  unsigned long long* maxslot;  // 2 slots of max(a, b) bits, alternating per iteration
  double* red;     // kRedBlocks x kNq reduction partials
  double* scal;    // kNq final sums + misc scalars
  int* counters;   // [0] absorptions
};

constexpr int kNq = 8;
constexpr int kRedBlocks = 296;


// Buffers of the on-the-fly (tensor-core) form.
struct TcState {
  bool on;
  int kp;                   // packed dimension (32 or 64)
  int n_xt, n_yt;           // 128-point tiles of X and Y
  int64_t I_pad, J_pad;
  int ctas_row, ctas_col;   // persistent grid of each pass
  __half* Xa;               // row form of X: [gamma x, 1, 1]   (repacked per epsilon)
  __half* Xb;               // column form of X: [x, bias columns] (bias per half-step)
  __half* Ya;
  __half* Yb;
  const float* X;
  const float* Y;
  int64_t ldx, ldy;
  int d;
  double* normX;            // |x_i|^2 (FP64)
  double* normY;
  float2* part;
  int* err;
  // Speculative half-steps: each row's base-2 log-sum-exp of the MMA exponents
  // from the previous half-step (row side offX, column side offY), valid while
  // epsilon is unchanged; rows whose sum left the safe range are listed in
  // redoX / redoY = [count, rows...] (row and column passes) and recomputed
  // exactly; each side's half-step empties the other side's list.
  float* offX;
  float* offY;
  int* redoX;
  int* redoY;
  int* tile_ctr;                   // per (row tile, lane quarter): partials written (CombineFin)
  unsigned long long* redo_total;  // rows recomputed exactly, over the solve (diagnostic)
  bool off_row_ok, off_col_ok;
  // Column-form biases of X (read by column passes) and Y (row passes) match
  // the current potentials: written by the row-tile finish of the half-step that
  // updated them, else packed before the pass that reads them.
  bool xb_ok, yb_ok;
};

struct Geom {
  int64_t I, J, ldc;
  int row_grid;
  int ncb, nrb;             // column-pass grid: column blocks x row blocks
  int64_t rows_per;
};

// The reference's a-update for row i; returns the new a_i (for the
// absorption test, reduced per block by the caller).
// exp(la) as the absorption test needs it: the test only compares the largest
// exp(la) with tau, so away from log(tau) the value is 0 (below) or +inf
// (above) with the same outcome, and the FP64 exp (slow on this part) is formed
// only within 1e-9 of log(tau). NaN stays NaN.
__device__ __forceinline__ double absorb_key(double la, const Coef& c) {
  if (la < c.ltau_lo) return 0.0;
  if (la > c.ltau_hi) return INFINITY;
  return exp(la);
}

__device__ __forceinline__ double a_update(int64_t i, double L, const Vecs& V, const Coef& c) {
  const double ui = V.u[i];
  const double logs = ui * c.inv_eps + L - c.logJ;                 // log (K (b dy))_i
  const double la_new = c.alpha1 * (V.logp[i] - logs) - ui * c.inv_l1e;
  V.la_old[i] = V.la[i];
  V.la[i] = la_new;
  split_weight((ui * c.inv_eps + la_new) * kLog2e, V.wrow, V.wrow_lo, i);
  return absorb_key(la_new, c);
}

__device__ __forceinline__ double b_update(int64_t j, double L, const Vecs& V, const Coef& c) {
  const double vj = V.v[j];
  const double logt = vj * c.inv_eps + L - c.logI;                 // log (K^T (a dx))_j
  const double lb_new = c.alpha2 * (c.logq - logt) - vj * c.inv_l2e;
  V.lb_old[j] = V.lb[j];
  V.lb[j] = lb_new;
  split_weight((vj * c.inv_eps + lb_new) * kLog2e, V.wcol, V.wcol_lo, j);
  return absorb_key(lb_new, c);
}

// Block-wide max of the threads' values, folded into the absorption slot with
// one atomic per block (every thread of the block must call it).
__device__ __forceinline__ void block_max_to_slot(double v, unsigned long long* slot) {
  __shared__ double sh[32];
  v = warp_maxd(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    w = warp_maxd(w);
    if (threadIdx.x == 0) atomic_max_nonneg(slot, w);
  }
}

// Exponent of one element: plain (w - k2 C, one rounding) or precise (relative
// to the grid offset o with the weight's and kappa2's low parts, see
// split_weight).
template <bool PREC>
__device__ __forceinline__ float expo(float cc, float w, float wl, float o, float k2, float k2l) {
  if (PREC) return fmaf(-k2, cc, w - o) + fmaf(-k2l, cc, wl);
  return fmaf(-k2, cc, w);
}

// Row pass: one warp per row, 128-bit streaming loads of C, online base-2 LSE.
// UPDATE_A additionally applies the a-update to the row (first half-step).
// PREC: the solver's precise form (weights hi + lo in V.wcol / V.wcol_lo, the
// row's previous log-sum-exp in V.Lrow as its offset); otherwise the plain form
// on one FP32 weight vector (the standalone half-step).
template <bool UPDATE_A, bool PREC>
__global__ void __launch_bounds__(256) row_pass_kernel(const float* __restrict__ C, Geom g,
                                                       Vecs V, Coef c, int parity) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nv = g.ldc >> 2;
  const float4* __restrict__ w4 = reinterpret_cast<const float4*>(V.wcol);
  const float4* __restrict__ wl4 = reinterpret_cast<const float4*>(PREC ? V.wcol_lo : V.wcol);
  const float k2 = c.kappa2, k2l = c.kappa2_lo;
  double amax = 0.0;
  for (int64_t i = warp; i < g.I; i += nwarps) {
    const float4* __restrict__ row = reinterpret_cast<const float4*>(C + i * g.ldc);
    const float o = PREC ? grid_offset(V.Lrow[i]) : 0.f;
    float m = kNegBig, s = 0.f, cmp = 0.f;   // PREC: compensated sum s - cmp
    int64_t k = lane;
    // the cost loads of the next 128-float4 chunk are issued before this
    // chunk's arithmetic (two chunks of loads in flight per lane)
    float4 cn[4];
    if (k + 96 < nv) {
#pragma unroll
      for (int t = 0; t < 4; ++t) cn[t] = ld_stream(row + k + 32 * t);
    }
    for (; k + 96 < nv; k += 128) {
      float4 cc[4], ww[4], wl[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) cc[t] = cn[t];
      if (k + 128 + 96 < nv) {
#pragma unroll
        for (int t = 0; t < 4; ++t) cn[t] = ld_stream(row + k + 128 + 32 * t);
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) ww[t] = __ldg(w4 + k + 32 * t);
#pragma unroll
      for (int t = 0; t < 4; ++t) wl[t] = PREC ? __ldg(wl4 + k + 32 * t) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const float x0 = expo<PREC>(cc[t].x, ww[t].x, wl[t].x, o, k2, k2l);
        const float x1 = expo<PREC>(cc[t].y, ww[t].y, wl[t].y, o, k2, k2l);
        const float x2 = expo<PREC>(cc[t].z, ww[t].z, wl[t].z, o, k2, k2l);
        const float x3 = expo<PREC>(cc[t].w, ww[t].w, wl[t].w, o, k2, k2l);
        const float mn = fmaxf(m, fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)));
        const float r = ex2(m - mn);
        const float v = (ex2(x0 - mn) + ex2(x1 - mn)) + (ex2(x2 - mn) + ex2(x3 - mn));
        if (PREC) {
          s = __fmul_rn(s, r);
          cmp = __fmul_rn(cmp, r);
          kahan_add(s, cmp, v);
        } else {
          s = s * r + v;
        }
        m = mn;
      }
    }
    for (; k < nv; k += 32) {
      const float4 cc = ld_stream(row + k);
      const float4 ww = __ldg(w4 + k);
      const float4 wl = PREC ? __ldg(wl4 + k) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float x0 = expo<PREC>(cc.x, ww.x, wl.x, o, k2, k2l);
      const float x1 = expo<PREC>(cc.y, ww.y, wl.y, o, k2, k2l);
      const float x2 = expo<PREC>(cc.z, ww.z, wl.z, o, k2, k2l);
      const float x3 = expo<PREC>(cc.w, ww.w, wl.w, o, k2, k2l);
      const float mn = fmaxf(m, fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)));
      const float r = ex2(m - mn);
      const float v = (ex2(x0 - mn) + ex2(x1 - mn)) + (ex2(x2 - mn) + ex2(x3 - mn));
      if (PREC) {
        s = __fmul_rn(s, r);
        cmp = __fmul_rn(cmp, r);
        kahan_add(s, cmp, v);
      } else {
        s = s * r + v;
      }
      m = mn;
    }
    double S = (double)s - (double)cmp;
    if (PREC) {
      warp_lse_f64(m, S);
    } else {
      warp_lse(m, s);
      S = (double)s;
    }
    if (lane == 0) {
      const double L = ((double)o + (double)m + log2(S)) * kLn2;
      V.Lrow[i] = L;
      if (UPDATE_A) amax = fmax(amax, a_update(i, L, V, c));
    }
  }
  if (UPDATE_A) block_max_to_slot(amax, V.maxslot + parity);
}

// a-update from a cached row LSE (the row pass of the preceding gap check).
__global__ void a_update_kernel(Geom g, Vecs V, Coef c, int parity) {
  double amax = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.I;
       i += (int64_t)gridDim.x * blockDim.x)
    amax = fmax(amax, a_update(i, V.Lrow[i], V, c));
  block_max_to_slot(amax, V.maxslot + parity);
}

// Column pass, phase 1: CTA = 1024 columns (float4 per thread) x rows_per rows;
// writes one (m, s) base-2 LSE partial per column and row block.
constexpr int kColRowChunk = 4;

// Offset of column j of the precise column pass (0 in padding columns); the
// combine recomputes the same value from the same V.Lcol.
__device__ __forceinline__ float col_offset(const Vecs& V, const Geom& g, int64_t j) {
  return j < g.J ? grid_offset(V.Lcol[j]) : 0.f;
}

template <bool PREC>
__global__ void __launch_bounds__(256) col_partial_kernel(const float* __restrict__ C, Geom g,
                                                          Vecs V, Coef c) {
  const int64_t c4 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nv = g.ldc >> 2;
  const int64_t r0 = (int64_t)blockIdx.y * g.rows_per;
  const int64_t r1 = min(g.I, r0 + g.rows_per);
  if (c4 >= nv) return;
  const float k2 = c.kappa2, k2l = c.kappa2_lo;
  float o[4] = {0.f, 0.f, 0.f, 0.f};
  if (PREC) {
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = col_offset(V, g, c4 * 4 + q);
  }
  float m[4] = {kNegBig, kNegBig, kNegBig, kNegBig};
  float s[4] = {0.f, 0.f, 0.f, 0.f};
  float cmp[4] = {0.f, 0.f, 0.f, 0.f};   // PREC: compensated sums s - cmp
  int64_t i = r0;
  // the next chunk's cost loads are issued before this chunk's arithmetic
  float4 cn[kColRowChunk];
  if (i + kColRowChunk <= r1) {
#pragma unroll
    for (int t = 0; t < kColRowChunk; ++t) cn[t] = ld_stream(reinterpret_cast<const float4*>(C + (i + t) * g.ldc) + c4);
  }
  for (; i + kColRowChunk <= r1; i += kColRowChunk) {
    float4 cc[kColRowChunk];
    float w[kColRowChunk], wl[kColRowChunk];
#pragma unroll
    for (int t = 0; t < kColRowChunk; ++t) cc[t] = cn[t];
    if (i + 2 * kColRowChunk <= r1) {
#pragma unroll
      for (int t = 0; t < kColRowChunk; ++t)
        cn[t] = ld_stream(reinterpret_cast<const float4*>(C + (i + kColRowChunk + t) * g.ldc) + c4);
    }
#pragma unroll
    for (int t = 0; t < kColRowChunk; ++t) w[t] = __ldg(V.wrow + i + t);
#pragma unroll
    for (int t = 0; t < kColRowChunk; ++t) wl[t] = PREC ? __ldg(V.wrow_lo + i + t) : 0.f;
    float x[4][kColRowChunk];
#pragma unroll
    for (int t = 0; t < kColRowChunk; ++t) {
      x[0][t] = expo<PREC>(cc[t].x, w[t], wl[t], o[0], k2, k2l);
      x[1][t] = expo<PREC>(cc[t].y, w[t], wl[t], o[1], k2, k2l);
      x[2][t] = expo<PREC>(cc[t].z, w[t], wl[t], o[2], k2, k2l);
      x[3][t] = expo<PREC>(cc[t].w, w[t], wl[t], o[3], k2, k2l);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float mx = x[q][0];
#pragma unroll
      for (int t = 1; t < kColRowChunk; ++t) mx = fmaxf(mx, x[q][t]);
      const float mn = fmaxf(m[q], mx);
      const float r = ex2(m[q] - mn);
      float v = 0.f;
#pragma unroll
      for (int t = 0; t < kColRowChunk; ++t) v += ex2(x[q][t] - mn);
      if (PREC) {
        s[q] = __fmul_rn(s[q], r);
        cmp[q] = __fmul_rn(cmp[q], r);
        kahan_add(s[q], cmp[q], v);
      } else {
        s[q] = s[q] * r + v;
      }
      m[q] = mn;
    }
  }
  for (; i < r1; ++i) {
    const float4 cc = ld_stream(reinterpret_cast<const float4*>(C + i * g.ldc) + c4);
    const float w = __ldg(V.wrow + i);
    const float wl = PREC ? __ldg(V.wrow_lo + i) : 0.f;
    const float xs[4] = {expo<PREC>(cc.x, w, wl, o[0], k2, k2l), expo<PREC>(cc.y, w, wl, o[1], k2, k2l),
                         expo<PREC>(cc.z, w, wl, o[2], k2, k2l), expo<PREC>(cc.w, w, wl, o[3], k2, k2l)};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float mn = fmaxf(m[q], xs[q]);
      const float r = ex2(m[q] - mn);
      if (PREC) {
        s[q] = __fmul_rn(s[q], r);
        cmp[q] = __fmul_rn(cmp[q], r);
        kahan_add(s[q], cmp[q], ex2(xs[q] - mn));
      } else {
        s[q] = s[q] * r + ex2(xs[q] - mn);
      }
      m[q] = mn;
    }
  }
  if (PREC) {
#pragma unroll
    for (int q = 0; q < 4; ++q) s[q] -= cmp[q];
  }
  float4* out = reinterpret_cast<float4*>(V.part + (int64_t)blockIdx.y * g.ldc + c4 * 4);
  out[0] = make_float4(m[0], s[0], m[1], s[1]);
  out[1] = make_float4(m[2], s[2], m[3], s[3]);
}

// Column pass, phase 2: merge the row-block partials of each column in FP64,
// then (UPDATE_B) the reference's b-update.
template <bool UPDATE_B, bool PREC>
__global__ void col_combine_kernel(Geom g, Vecs V, Coef c, int parity) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double bmax = 0.0;
  if (j < g.J) {
    const float o = PREC ? col_offset(V, g, j) : 0.f;
    double L;
    if (PREC) {
      // the row-block partials merged in FP64 against their largest exponent
      // (FP32 scale factors, 2 ulp; two passes: measured faster than one pass
      // with a running maximum, whose rescaling lengthens the FP64 chain)
      float m = kNegBig;
      for (int r = 0; r < g.nrb; ++r) m = fmaxf(m, V.part[(int64_t)r * g.ldc + j].x);
      double S = 0.0;
      for (int r = 0; r < g.nrb; ++r) {
        const float2 ps = V.part[(int64_t)r * g.ldc + j];
        S += (double)ps.y * (double)ex2(ps.x - m);
      }
      L = ((double)o + (double)m + log2(S)) * kLn2;
    } else {
      float m = kNegBig, s = 0.f;
      for (int r = 0; r < g.nrb; ++r) {
        const float2 ps = V.part[(int64_t)r * g.ldc + j];
        lse_merge(m, s, ps.x, ps.y);
      }
      L = lse2(m, s) * kLn2;
    }
    V.Lcol[j] = L;
    if (UPDATE_B) bmax = b_update(j, L, V, c);
  }
  if (UPDATE_B) block_max_to_slot(bmax, V.maxslot + parity);
}

// tau-absorption (optimal_transport.py:137-141 / :211-216): if max(a, b) > tau,
// u += eps log a, v += eps log b, a = b = 1. Also clears the other max slot.
// The on-the-fly form also rewrites the column-form biases of the absorbed
// points (bx, by; tiles = nullptr in the materialised form).
__global__ void absorb_kernel(Geom g, Vecs V, Coef c, double tau, int parity, TcBias bx, TcBias by) {
  pdl_wait();
  pdl_trigger();
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double mx = __longlong_as_double((long long)V.maxslot[parity]);
  if (idx == 0) V.maxslot[parity ^ 1] = 0ull;
  if (!(mx > tau)) return;
  if (idx == 0) V.counters[0] += 1;
  const double k2d = c.kappa * kLog2e;
  if (idx < g.I) {
    const double un = V.u[idx] + c.eps * V.la[idx];
    V.u[idx] = un;
    V.la[idx] = 0.0;
    split_weight(un * c.inv_eps * kLog2e, V.wrow, V.wrow_lo, idx);
    if (bx.tiles) tc_write_bias(idx, (un * c.inv_eps + 0.0) * kLog2e - k2d * bx.norm[idx], bx.d, bx.kp, bx.tiles);
  } else if (idx < g.I + g.J) {
    const int64_t j = idx - g.I;
    const double vn = V.v[j] + c.eps * V.lb[j];
    V.v[j] = vn;
    V.lb[j] = 0.0;
    split_weight(vn * c.inv_eps * kLog2e, V.wcol, V.wcol_lo, j);
    if (by.tiles) tc_write_bias(j, (vn * c.inv_eps + 0.0) * kLog2e - k2d * by.norm[j], by.d, by.kp, by.tiles);
  }
}

// Absorb with the old epsilon, switch to the new one, reset a = b = 1
// (stage start, optimal_transport.py:118-125; epsilon step, :218-228).
__global__ void rescale_kernel(Geom g, Vecs V, double eps_old, double inv_eps_new) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx == 0) {
    V.maxslot[0] = 0ull;
    V.maxslot[1] = 0ull;
  }
  if (idx < g.I) {
    const double un = V.u[idx] + eps_old * V.la[idx];
    V.u[idx] = un;
    V.la[idx] = 0.0;
    V.la_old[idx] = 0.0;
    split_weight(un * inv_eps_new * kLog2e, V.wrow, V.wrow_lo, idx);
  } else if (idx < g.I + g.J) {
    const int64_t j = idx - g.I;
    const double vn = V.v[j] + eps_old * V.lb[j];
    V.v[j] = vn;
    V.lb[j] = 0.0;
    V.lb_old[j] = 0.0;
    split_weight(vn * inv_eps_new * kLog2e, V.wcol, V.wcol_lo, j);
  }
}

// Zero state for a new solve; p = G; padding of wcol = 0.
__global__ void init_kernel(Geom g, Vecs V, const double* __restrict__ G) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx == 0) {
    V.maxslot[0] = 0ull;
    V.maxslot[1] = 0ull;
    V.counters[0] = 0;
  }
  if (idx < g.I) {
    V.u[idx] = 0.0;
    V.la[idx] = 0.0;
    V.la_old[idx] = 0.0;
    const double pi = G[idx];
    V.p[idx] = pi;
    V.logp[idx] = log(pi);
    V.wrow[idx] = 0.f;
    V.wrow_lo[idx] = 0.f;
    V.Lrow[idx] = 0.0;
  }
  if (idx < g.ldc) {
    V.wcol[idx] = 0.f;
    V.wcol_lo[idx] = 0.f;
    if (idx < g.J) {
      V.v[idx] = 0.0;
      V.lb[idx] = 0.0;
      V.lb_old[idx] = 0.0;
      V.Lcol[idx] = 0.0;
    }
  }
}

// Warm start from absorbed potentials: u = u_bar, v = v_bar, a = b = 1.
__global__ void load_potentials_kernel(Geom g, Vecs V, const double* __restrict__ ubar,
                                       const double* __restrict__ vbar, double inv_eps) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < g.I) {
    V.u[idx] = ubar[idx];
    V.la[idx] = 0.0;
    V.la_old[idx] = 0.0;
    V.Lrow[idx] = 0.0;
    split_weight(ubar[idx] * inv_eps * kLog2e, V.wrow, V.wrow_lo, idx);
  } else if (idx < g.I + g.J) {
    const int64_t j = idx - g.I;
    V.v[j] = vbar[j];
    V.lb[j] = 0.0;
    V.lb_old[j] = 0.0;
    V.Lcol[j] = 0.0;
    split_weight(vbar[j] * inv_eps * kLog2e, V.wcol, V.wcol_lo, j);
  }
}

// ---------------------------------------------------------------------------
// Deterministic two-level FP64 reductions: kRedBlocks blocks write partials,
// one block sums them.
// ---------------------------------------------------------------------------
template <int NQ>
__device__ __forceinline__ void block_reduce_store(double (&acc)[NQ], double* out) {
  __shared__ double sh[32][NQ];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = warp_sum(acc[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) sh[wid][q] = acc[q];
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double t = lane < nw ? sh[lane][q] : 0.0;
      t = warp_sum(t);
      if (lane == 0) out[q] = t;
    }
  }
}

__global__ void finalize_kernel(const double* __restrict__ red, int nblocks, double* out) {
  double acc[kNq];
#pragma unroll
  for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int q = 0; q < kNq; ++q) acc[q] += red[b * kNq + q];
  block_reduce_store<kNq>(acc, out);
}

// sum_ij exp(-kappa C_ij) over valid entries (the reference's sum of _K, used
// in the primal objective at the final stage).
__global__ void __launch_bounds__(256) sum_exp_kernel(const float* __restrict__ C, Geom g, float kappa2,
                                                      double* red) {
  const int64_t nv = g.ldc >> 2;
  double acc[kNq];
#pragma unroll
  for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
  for (int64_t i = blockIdx.x; i < g.I; i += gridDim.x) {
    const float4* row = reinterpret_cast<const float4*>(C + i * g.ldc);
    float s = 0.f;
    for (int64_t k = threadIdx.x; k < nv; k += blockDim.x) {
      const float4 cc = ld_stream(row + k);
      s += (ex2(-kappa2 * cc.x) + ex2(-kappa2 * cc.y)) + (ex2(-kappa2 * cc.z) + ex2(-kappa2 * cc.w));
    }
    acc[0] += (double)s;  // padding is +inf -> exp2(-inf) = 0
  }
  block_reduce_store<kNq>(acc, red + blockIdx.x * kNq);
}

// mean(G) (q = ones(J) * np.average(G), optimal_transport.py:108 / :192).
__global__ void sum_vec_kernel(const double* __restrict__ x, int64_t n, double* red) {
  double acc[kNq];
#pragma unroll
  for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc[0] += x[i];
  block_reduce_store<kNq>(acc, red + blockIdx.x * kNq);
}

// Stage-exit test (optimal_transport.py:158-160), FP64, as the reference
// evaluates it: a~ = a * exp(u/eps), old = old_a * exp(u/eps).
//   acc[0] = |a~ - old|^2, acc[1] = |a~|^2, acc[2], acc[3] likewise for b.
__global__ void stage_test_kernel(Geom g, Vecs V, Coef c, double* red) {
  double acc[kNq];
#pragma unroll
  for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.I; i += stride) {
    const double e = exp(V.u[i] * c.inv_eps);
    const double ta = exp(V.la[i]) * e;
    const double d = ta - exp(V.la_old[i]) * e;
    acc[0] += d * d;
    acc[1] += ta * ta;
  }
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.J; j += stride) {
    const double e = exp(V.v[j] * c.inv_eps);
    const double tb = exp(V.lb[j]) * e;
    const double d = tb - exp(V.lb_old[j]) * e;
    acc[2] += d * d;
    acc[3] += tb * tb;
  }
  block_reduce_store<kNq>(acc, red + blockIdx.x * kNq);
}

// Duality-gap terms (final stage). Needs Lrow with the current b and Lcol
// with the current a.
//   acc[0] = sum_i [lambda1 (x log(x/p) - x + p) + lambda1 p (exp(-eps log a~/lambda1) - 1) + ubar x]
//   acc[1] = same over j with lambda2, q, b~, vbar, y
//   acc[2] = sum_i (x log(x/p) - x + p)       acc[3] = sum_j (y log(y/q) - y + q)
//   acc[4] = sum_i ubar x                      acc[5] = sum_j vbar y
//   acc[6] = sum_i x
// The gap terms of one point: x = exp(t) its marginal sum (t = log x), p its
// target, the scaling a~ = exp(la) exp(u/eps) evaluated as the reference does.
// Where nothing overflows or underflows, log(x / p) = t - log p and
// log a~ = la + u/eps (to an ulp), which saves four of the six FP64
// transcendentals per point (slow on this part); at the edges the reference's
// own expressions run, so overflow, 0 log 0 and NaN behave as in the reference.
__device__ __forceinline__ void gap_terms(double t, double la, double ue, double p, double logp, double lambda,
                                          double eps, double* x_out, double* f_out, double* conj_out) {
  const double x = exp(t);
  double f, conj;
  if (x > 0.0 && fabs(t) < 700.0 && fabs(la) < 700.0 && fabs(ue) < 700.0 && fabs(la + ue) < 700.0 && p > 0.0) {
    f = x * (t - logp) - x + p;
    conj = lambda * p * (exp(-eps * (la + ue) / lambda) - 1.0);
  } else {
    const double at = exp(la) * exp(ue);
    f = x * log(x / p) - x + p;
    conj = lambda * p * (exp(-eps * log(at) / lambda) - 1.0);
  }
  *x_out = x;
  *f_out = f;
  *conj_out = conj;
}

__global__ void gap_partial_kernel(Geom g, Vecs V, Coef c, double* red) {
  double acc[kNq];
#pragma unroll
  for (int q = 0; q < kNq; ++q) acc[q] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.I; i += stride) {
    const double ui = V.u[i], lai = V.la[i], pi = V.p[i];
    const double ue = ui * c.inv_eps;
    double x, f, conj;
    gap_terms(lai + ue + V.Lrow[i] - c.logJ, lai, ue, pi, V.logp[i], c.lambda1, c.eps, &x, &f, &conj);
    const double ub = ui + c.eps * lai;
    acc[0] += c.lambda1 * f + conj + ub * x;
    acc[2] += f;
    acc[4] += ub * x;
    acc[6] += x;
  }
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.J; j += stride) {
    const double vj = V.v[j], lbj = V.lb[j];
    const double ve = vj * c.inv_eps;
    double y, f, conj;
    gap_terms(lbj + ve + V.Lcol[j] - c.logI, lbj, ve, c.q, c.logq, c.lambda2, c.eps, &y, &f, &conj);
    const double vb = vj + c.eps * lbj;
    acc[1] += c.lambda2 * f + conj + vb * y;
    acc[3] += f;
    acc[5] += vb * y;
  }
  block_reduce_store<kNq>(acc, red + blockIdx.x * kNq);
}

// Outputs. `log_scale` is the log of the factor applied to R = diag(a) K diag(b):
// -log J for the reference's normal return R / J, 0 for its max_iter return R.
// Row sums of the returned coupling (tmap.sum(axis=1)); needs Lrow with the final b.
__global__ void row_sums_kernel(Geom g, Vecs V, Coef c, double log_scale, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.I;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = exp(V.la[i] + V.u[i] * c.inv_eps + V.Lrow[i] + log_scale);
}

__global__ void potentials_kernel(Geom g, Vecs V, Coef c, double* __restrict__ ubar,
                                  double* __restrict__ vbar) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < g.I) {
    if (ubar) ubar[idx] = V.u[idx] + c.eps * V.la[idx];
  } else if (idx < g.I + g.J) {
    const int64_t j = idx - g.I;
    if (vbar) vbar[j] = V.v[j] + c.eps * V.lb[j];
  }
}

// Per-row constants of the dense coupling: the row's base-2 exponent
//   t_ij = wr_i + wc_j - k2 C_ij,   wr_i = (u_i / eps + la_i + log_scale) log2 e,
// is evaluated as t_ij = x_ij + E_i with x_ij = (wc_j - o_i) - k2 C_ij in FP32
// (the streamed passes' split arithmetic, o_i the row's grid offset from its
// log-sum-exp L_i, so x <= ~0 for the entries that carry mass) and
// E_i = o_i + wr_i = n_i + f_i in FP64: rowc = (o_i, 2^f_i, n_i, 1); w = 0 marks
// a row whose constants are not finite (its entries take the FP64 path).
__global__ void coupling_rows_kernel(Geom g, Vecs V, Coef c, double log_scale) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.I) return;
  const double wr = (V.u[i] * c.inv_eps + V.la[i] + log_scale) * kLog2e;
  const double L = V.Lrow[i];
  const float o = grid_offset(L);
  const double E = (double)o + wr;
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (fabs(L) < 1e30 && fabs(E) < 900.0) {
    const double n = floor(E);
    r = make_float4(o, (float)exp2(E - n), (float)n, 1.f);
  }
  V.rowc[i] = r;
}

// 2^t for an FP64 exponent t: the integer part exactly (as the FP64 exponent
// field), the fraction by FP32 ex2 (relative error ~2^-22); 0 below 2^-1020,
// NaN for NaN.
__device__ __forceinline__ double exp2_split(double t) {
  if (!(t > -1020.0)) return t != t ? t : 0.0;
  if (t >= 1024.0) return INFINITY;
  const double ti = floor(t);
  const double scale = __longlong_as_double((long long)(ti + 1023.0) << 52);
  return (double)ex2((float)(t - ti)) * scale;
}

// Dense coupling tmap_ij = a_i exp((u_i - C_ij + v_j)/eps) b_j * exp(log_scale), written
// FP64 row-major (stride J) like the reference's ndarray. 2^t_ij = (2^x_ij 2^f_i) 2^n_i
// (coupling_rows_kernel): x_ij = fma(-k2hi, C, wc_hi - o_i) + fma(-k2lo, C, wc_lo) as in
// the streamed passes (one FP32 rounding of a value that is small for the entries that
// carry mass, below the FP32 storage of C), 2^x 2^f in FP32, and the power 2^n_i put into
// the FP64 exponent field by integer arithmetic, so that no element needs FP64
// arithmetic (slow on this part) and the kernel streams C in and the map out. Entries
// whose 2^x or result leaves the normal ranges (far below a row's mass, or non-finite
// inputs) take the FP64 exponent (exp2_split), which is exact in the same way.
__global__ void __launch_bounds__(256) coupling_kernel(const float* __restrict__ C, Geom g, Vecs V,
                                                       Coef c, double log_scale, double* __restrict__ out) {
  for (int64_t j0 = (int64_t)blockIdx.x * blockDim.x; j0 < g.J; j0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = j0 + threadIdx.x;
    if (j >= g.J) continue;
    const float hi = V.wcol[j], lo = V.wcol_lo[j];   // once per column
    for (int64_t i = blockIdx.y; i < g.I; i += gridDim.y) {
      const float4 rc = V.rowc[i];
      const float cc = C[i * g.ldc + j];
      const float x = fmaf(-c.kappa2, cc, hi - rc.x) + fmaf(-c.kappa2_lo, cc, lo);
      double val;
      bool done = false;
      if (rc.w != 0.f && x > -125.f && x < 125.f) {
        const float y = ex2(x) * rc.y;                              // normal, positive
        const uint32_t yb = __float_as_uint(y);
        const int e = (int)(yb >> 23) - 127 + (int)rc.z;           // exponent of the result
        if (e > -1022 && e < 1023) {
          val = __longlong_as_double((long long)((uint64_t)(e + 1023) << 52 | (uint64_t)(yb & 0x7FFFFFu) << 29));
          done = true;
        }
      }
      if (!done) {
        const double wr = (V.u[i] * c.inv_eps + V.la[i] + log_scale) * kLog2e;
        const double wc = (V.v[j] * c.inv_eps + V.lb[j]) * kLog2e;
        val = exp2_split(wr + wc - c.kappa * kLog2e * (double)cc);
      }
      out[i * g.J + j] = val;
    }
  }
}

// ---------------------------------------------------------------------------
// On-the-fly form: the FP64 finish of the tensor-core kernel's partials. The
// exponent of element (i, j) is split as
//   bias_j + gamma (x_i . y_j) - kappa2 |x_i|^2,   gamma = 2 kappa2,
//   bias_j = (v_j / eps + lb_j) log2 e - kappa2 |y_j|^2     (FP64, carried by the MMA),
// i.e. (v_j/eps + lb_j - kappa C_ij) in base 2 with C = |x|^2 + |y|^2 - 2 x.y; the
// tensor-core kernel produces the first two terms, its row-tile finish
// (CombineFin, below) adds the third.
// ---------------------------------------------------------------------------
// Column-form bias of point i of the side a half-step just updated (ROW: a row
// point with its new log-scaling la, for the next column pass; else a column
// point with its new lb, for the next row pass).
template <bool ROW>
__device__ __forceinline__ void write_bias(int64_t i, const Vecs& V, const Coef& c, const TcBias& b) {
  const double pot = ROW ? V.u[i] : V.v[i];
  const double lsc = ROW ? V.la[i] : V.lb[i];
  tc_write_bias(i, (pot * c.inv_eps + lsc) * kLog2e - (c.kappa * kLog2e) * b.norm[i], b.d, b.kp, b.tiles);
}

// Exact half-step of the rows listed by a speculative half-step (a warp per row):
// L_i = log sum_j exp(w_j - kappa |x_i - y_j|^2) from the FP32 points with a
// running maximum, then the same update and offset as the row-tile finish.
template <bool ROW, bool UPDATE>
__global__ void tc_exact_rows_kernel(Geom g, Vecs V, Coef c, const float* __restrict__ P, int64_t ldp,
                                     const float* __restrict__ Q, int64_t ldq, int d, const double* __restrict__ norm,
                                     float* __restrict__ off, int* __restrict__ redo,
                                     unsigned long long* __restrict__ total, int parity, TcBias bias) {
  pdl_wait();
  pdl_trigger();
  const int cnt = redo[0];
  if (blockIdx.x == 0 && threadIdx.x == 0 && cnt > 0) atomicAdd(total, (unsigned long long)cnt);
  const int lane = threadIdx.x & 31;
  const int64_t m_cols = ROW ? g.J : g.I;
  const double* pot = ROW ? V.v : V.u;
  const double* lsc = ROW ? V.lb : V.la;
  const float k2 = (float)(c.kappa * kLog2e);
  for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < cnt; w += (int)((gridDim.x * blockDim.x) >> 5)) {
    const int64_t i = redo[1 + w];
    const float* x = P + i * ldp;
    float m = kNegBig, s = 0.f;
    for (int64_t j = lane; j < m_cols; j += 32) {
      const float* y = Q + j * ldq;
      float cc = 0.f;
      for (int t = 0; t < d; ++t) {
        const float df = x[t] - y[t];
        cc = fmaf(df, df, cc);
      }
      const float tt = (float)((pot[j] * c.inv_eps + lsc[j]) * kLog2e) - k2 * cc;
      const float mn = fmaxf(m, tt);
      s = s * ex2(m - mn) + ex2(tt - mn);
      m = mn;
    }
    warp_lse(m, s);
    if (lane == 0) {
      const double L2 = lse2(m, s);
      off[i] = (float)(L2 + (double)k2 * norm[i]);
      const double L = L2 * kLn2;
      double v = 0.0;
      if (ROW) {
        V.Lrow[i] = L;
        if (UPDATE) v = a_update(i, L, V, c);
      } else {
        V.Lcol[i] = L;
        if (UPDATE) v = b_update(i, L, V, c);
      }
      if (UPDATE) atomic_max_nonneg(V.maxslot + parity, v);
      if (UPDATE && bias.tiles) write_bias<ROW>(i, V, c, bias);
    }
  }
}

// Row-tile finish of an on-the-fly half-step inside lse_tc_kernel: the warp
// that writes the last partial of 32 rows (over the CTAs and column halves that
// covered their row tile) merges them in a fixed order (FP32 LSE merge), then
// per row either lists it for the exact recompute (a speculative sum outside
// [2^-80, 2^100]) or writes its offset and log-sum-exp and, with UPDATE, the
// FP64 a- or b-update, the point's column-form bias for the other side's next
// pass and the absorption maximum (the work of a separate merge pass, without
// its launch and its wait on the whole kernel). Ordering: every lane fences its partial, the warp synchronises, one
// atomic per warp counts it; the finishing warp fences again and reads the
// partials from L2.
template <bool ROW, bool UPDATE>
struct CombineFin {
  static constexpr bool kActive = true;
  Geom g;
  Vecs V;
  Coef c;
  const double* norm;
  float* off;
  int* redo;
  int* redo_other;
  TcBias bias;
  int* ctr;  // per (row tile, lane quarter): partials written so far
  int nq, ctas, parity, spec;

  // the other side's exact-row list was consumed by its last half-step
  __device__ __forceinline__ void start() const { redo_other[0] = 0; }

  __device__ void quarter_done(const float2* part, int t, int wq, int lane) const {
    __threadfence();
    __syncwarp();
    const int64_t n = ROW ? g.I : g.J;
    const int64_t total = ((n + 127) >> 7) * (int64_t)nq;
    const int64_t c_lo = tc_cta_of((int64_t)t * nq, total, ctas);
    const int64_t c_hi = tc_cta_of(((int64_t)t + 1) * nq - 1, total, ctas);
    const int expect = 2 * (int)(c_hi - c_lo + 1);
    int old = 0;
    if (lane == 0) old = atomicAdd(ctr + 4 * t + wq, 1);
    old = __shfl_sync(0xffffffffu, old, 0);
    if (old != expect - 1) return;
    if (lane == 0) ctr[4 * t + wq] = 0;   // for the next launch
    __threadfence();
    const int64_t i = (int64_t)t * 128 + 32 * wq + lane;
    double vmax = 0.0;
    if (i < n) {
      float m = kNegBig, s = 0.f;
      for (int64_t cc = c_lo; cc <= c_hi; ++cc) {
        const float2* pp = part + ((cc + t) * 128 + (i & 127)) * kTcParts;
#pragma unroll
        for (int k = 0; k < kTcParts; ++k) {
          const float2 u = __ldcg(pp + k);
          lse_merge(m, s, u.x, u.y);
        }
      }
      if (spec && !(s >= 0x1p-80f && s <= 0x1p100f)) {
        const int k = atomicAdd(redo, 1);
        redo[1 + k] = (int)i;
      } else {
        const double D = lse2(m, s);
        off[i] = (float)D;
        const double L = D * kLn2 - c.kappa * norm[i];
        if (ROW) {
          V.Lrow[i] = L;
          if (UPDATE) vmax = a_update(i, L, V, c);
        } else {
          V.Lcol[i] = L;
          if (UPDATE) vmax = b_update(i, L, V, c);
        }
        if (UPDATE && bias.tiles) write_bias<ROW>(i, V, c, bias);
      }
    }
    if (UPDATE) {
      vmax = warp_maxd(vmax);
      if (lane == 0) atomic_max_nonneg(V.maxslot + parity, vmax);
    }
  }
};

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct Solver {
  const float* C;
  Geom g;
  Vecs V;
  cudaStream_t st;
  double cost_scale;
  int small_grid;  // grid for O(I+J) kernels
  TcState tc;

  Coef coef(double eps, const wotg_params& P, double q) const {
    Coef c = make_coef(eps, P.lambda1, P.lambda2, cost_scale, g.I, g.J, q);
    c.ltau_lo = std::log(P.tau) - 1e-9;
    c.ltau_hi = std::log(P.tau) + 1e-9;
    return c;
  }

  int vec_blocks(int64_t n) const { return (int)std::max<int64_t>(1, (n + 255) / 256); }

  // On-the-fly row pass (K (b dy)) / column pass (K^T (a dx)).
  // Row forms carry gamma = 2 kappa2, which changes with epsilon. Column forms
  // hold sqrt(cost_scale) y and row forms (gamma / sqrt(cost_scale)) x, so that
  // both stay in median-normalised units whatever the units of the input points
  // (FP16 range); their product is gamma x . y.
  int tc_prepare(const Coef& c) {
    if (!tc.on) return WOTG_OK;
    tc.off_row_ok = false;  // a new epsilon: the offsets and biases of both sides are stale
    tc.off_col_ok = false;
    tc.xb_ok = tc.yb_ok = false;
    WOTG_CUDA(cudaMemsetAsync(tc.redoX, 0, sizeof(int), st));
    WOTG_CUDA(cudaMemsetAsync(tc.redoY, 0, sizeof(int), st));
    WOTG_CUDA(cudaMemsetAsync(tc.tile_ctr, 0, sizeof(int) * 4 * std::max(tc.n_xt, tc.n_yt), st));
    const float gamma = (float)(2.0 * c.kappa * kLog2e / std::sqrt(cost_scale));
    int s = tc_pack_points(tc.X, g.I, tc.ldx, tc.d, tc.kp, gamma, 1, tc.Xa, nullptr, st);
    if (s) return s;
    return tc_pack_points(tc.Y, g.J, tc.ldy, tc.d, tc.kp, gamma, 1, tc.Ya, nullptr, st);
  }

  // The half-steps run in the speculative form once the offsets of their side
  // exist for the current epsilon (the first half-step of each side after an
  // epsilon change or a new solve runs the exact form and writes them).
  TcBias bias_x() const { return TcBias{tc.Xb, tc.normX, tc.d, tc.kp}; }
  TcBias bias_y() const { return TcBias{tc.Yb, tc.normY, tc.d, tc.kp}; }

  // One on-the-fly half-step with its row-tile finish inside the kernel
  // (CombineFin), launched as a dependent of the previous kernel.
  template <bool ROW, bool UPDATE>
  int tc_fused_pass(const Coef& c, int parity, bool spec) {
    using F = CombineFin<ROW, UPDATE>;
    F fin;
    fin.g = g;
    fin.V = V;
    fin.c = c;
    fin.norm = ROW ? tc.normX : tc.normY;
    fin.off = ROW ? tc.offX : tc.offY;
    fin.redo = ROW ? tc.redoX : tc.redoY;
    fin.redo_other = ROW ? tc.redoY : tc.redoX;
    fin.bias = UPDATE ? (ROW ? bias_x() : bias_y()) : TcBias{};
    fin.ctr = tc.tile_ctr;
    fin.nq = ROW ? tc.n_yt : tc.n_xt;
    fin.ctas = ROW ? tc.ctas_row : tc.ctas_col;
    fin.parity = parity;
    fin.spec = spec ? 1 : 0;
    const __half* Pt = ROW ? tc.Xa : tc.Ya;
    const __half* Qt = ROW ? tc.Yb : tc.Xb;
    const int n_pt = ROW ? tc.n_xt : tc.n_yt;
    const float* offp = spec ? fin.off : nullptr;
    const float* no_w = nullptr;
    float* no_s = nullptr;
    if (tc.kp == 32) {
      WOTG_CUDA((tc_set_smem_attr<32, 0, F>()));
      WOTG_CUDA(launch_dependent(lse_tc_kernel<32, 0, F>, dim3(fin.ctas), dim3(kTcThreads), TcSmem<32>::kAlloc, st,
                                 Pt, Qt, n_pt, fin.nq, tc.part, offp, tc.err, kTcWaitTries, no_w, 0, 0, no_s, fin));
    } else {
      WOTG_CUDA((tc_set_smem_attr<64, 0, F>()));
      WOTG_CUDA(launch_dependent(lse_tc_kernel<64, 0, F>, dim3(fin.ctas), dim3(kTcThreads), TcSmem<64>::kAlloc, st,
                                 Pt, Qt, n_pt, fin.nq, tc.part, offp, tc.err, kTcWaitTries, no_w, 0, 0, no_s, fin));
    }
    WOTG_LAUNCHED();
    return WOTG_OK;
  }

  template <bool UPDATE>
  int tc_row_pass(const Coef& c, int parity) {
    if (!tc.yb_ok) {
      int s = tc_pack_bias(g.J, V.v, V.lb, tc.normY, c.inv_eps, c.kappa * kLog2e, tc.d, tc.kp, tc.Yb, st);
      if (s) return s;
      tc.yb_ok = true;
    }
    const bool spec = tc.off_row_ok;
    int s = tc_fused_pass<true, UPDATE>(c, parity, spec);
    if (s) return s;
    const TcBias bx = UPDATE ? bias_x() : TcBias{};
    if (spec) {
      WOTG_CUDA(launch_dependent(tc_exact_rows_kernel<true, UPDATE>, dim3(2 * sm_count()), dim3(256), 0, st, g, V, c,
                                 (const float*)tc.X, tc.ldx, (const float*)tc.Y, tc.ldy, tc.d,
                                 (const double*)tc.normX, tc.offX, tc.redoX, tc.redo_total, parity, bx));
      WOTG_LAUNCHED();
    }
    tc.off_row_ok = true;
    if (UPDATE) tc.xb_ok = true;
    return WOTG_OK;
  }
  int tc_col_pass(const Coef& c, int parity) {
    if (!tc.xb_ok) {
      int s = tc_pack_bias(g.I, V.u, V.la, tc.normX, c.inv_eps, c.kappa * kLog2e, tc.d, tc.kp, tc.Xb, st);
      if (s) return s;
      tc.xb_ok = true;
    }
    const bool spec = tc.off_col_ok;
    int s = tc_fused_pass<false, true>(c, parity, spec);
    if (s) return s;
    if (spec) {
      WOTG_CUDA(launch_dependent(tc_exact_rows_kernel<false, true>, dim3(2 * sm_count()), dim3(256), 0, st, g, V, c,
                                 (const float*)tc.Y, tc.ldy, (const float*)tc.X, tc.ldx, tc.d,
                                 (const double*)tc.normY, tc.offY, tc.redoY, tc.redo_total, parity, bias_y()));
      WOTG_LAUNCHED();
    }
    tc.off_col_ok = true;
    tc.yb_ok = true;
    return WOTG_OK;
  }

  int iteration(const Coef& c, bool lrow_valid, int parity, bool update_b_only = false) {
    (void)update_b_only;
    if (tc.on) {
      int s;
      if (lrow_valid) {
        a_update_kernel<<<vec_blocks(g.I), 256, 0, st>>>(g, V, c, parity);
        WOTG_LAUNCHED();
        tc.xb_ok = false;  // la changed without its biases: the column pass packs them
      } else {
        s = tc_row_pass<true>(c, parity);
        if (s) return s;
      }
      return tc_col_pass(c, parity);
    }
    if (lrow_valid) {
      a_update_kernel<<<vec_blocks(g.I), 256, 0, st>>>(g, V, c, parity);
    } else {
      row_pass_kernel<true, true><<<g.row_grid, 256, 0, st>>>(C, g, V, c, parity);
    }
    WOTG_LAUNCHED();
    col_partial_kernel<true><<<dim3(g.ncb, g.nrb), 256, 0, st>>>(C, g, V, c);
    WOTG_LAUNCHED();
    col_combine_kernel<true, true><<<vec_blocks(g.J), 256, 0, st>>>(g, V, c, parity);
    WOTG_LAUNCHED();
    return WOTG_OK;
  }

  int absorb(const Coef& c, double tau, int parity) {
    if (tc.on)
      WOTG_CUDA(launch_dependent(absorb_kernel, dim3(vec_blocks(g.I + g.J)), dim3(256), 0, st, g, V, c, tau, parity,
                                 bias_x(), bias_y()));
    else
      absorb_kernel<<<vec_blocks(g.I + g.J), 256, 0, st>>>(g, V, c, tau, parity, TcBias{}, TcBias{});
    WOTG_LAUNCHED();
    return WOTG_OK;
  }

  int rescale(double eps_old, double eps_new) {
    rescale_kernel<<<vec_blocks(g.I + g.J), 256, 0, st>>>(g, V, eps_old, 1.0 / eps_new);
    WOTG_LAUNCHED();
    return WOTG_OK;
  }

  int reduce_to_host(double* host8) {
    finalize_kernel<<<1, 256, 0, st>>>(V.red, kRedBlocks, V.scal);
    WOTG_LAUNCHED();
    WOTG_CUDA(cudaMemcpyAsync(host8, V.scal, kNq * sizeof(double), cudaMemcpyDeviceToHost, st));
    WOTG_CUDA(cudaStreamSynchronize(st));
    return WOTG_OK;
  }

  int mean_of(const double* x, int64_t n, double* out) {
    sum_vec_kernel<<<kRedBlocks, 256, 0, st>>>(x, n, V.red);
    WOTG_LAUNCHED();
    double h[kNq];
    int s = reduce_to_host(h);
    if (s) return s;
    *out = h[0] / (double)n;
    return WOTG_OK;
  }

  int sum_exp(const Coef& c, double* out) {
    sum_exp_kernel<<<kRedBlocks, 256, 0, st>>>(C, g, c.kappa2, V.red);
    WOTG_LAUNCHED();
    double h[kNq];
    int s = reduce_to_host(h);
    if (s) return s;
    *out = h[0];
    return WOTG_OK;
  }

  int fresh_lrow(const Coef& c) {
    if (tc.on) return tc_row_pass<false>(c, 0);
    row_pass_kernel<false, true><<<g.row_grid, 256, 0, st>>>(C, g, V, c, 0);
    WOTG_LAUNCHED();
    return WOTG_OK;
  }

  // CUDA-graph replay of the final stage's batches between duality-gap checks.
  // In that stage a batch starts right after a check (L_row fresh) with both
  // sides' speculative offsets and column-form biases current, and ends in the
  // same host state, so its launches (nb iterations with their absorption
  // tests, all arguments fixed for the stage) are captured once per starting
  // parity and replayed; a new epsilon drops them.
  struct BatchGraph {
    cudaGraphExec_t exec = nullptr;
    unsigned long long launches = 0;
    int nb = 0;
  };
  BatchGraph bg[2] = {};
  cudaStream_t gs = nullptr;                 // private stream of the captures and replays
  cudaEvent_t gev[2] = {nullptr, nullptr};
  bool graphs_off = false;                   // no private stream: plain launches

  bool steady() const { return !tc.on || (tc.off_row_ok && tc.off_col_ok && tc.xb_ok && tc.yb_ok); }

  void drop_graphs() {
    for (auto& b : bg) {
      if (b.exec) cudaGraphExecDestroy(b.exec);
      b = BatchGraph{};
    }
  }
  void release_graphs() {
    drop_graphs();
    for (auto& e : gev)
      if (e) cudaEventDestroy(e);
    gev[0] = gev[1] = nullptr;
    if (gs) cudaStreamDestroy(gs);
    gs = nullptr;
  }

  // One batch of nb iterations from a fresh L_row at `parity`, as a graph;
  // *used = false when graphs are unavailable (the caller launches plainly).
  int batch_graph(const Coef& c, int nb, int parity, double tau, bool* used) {
    *used = false;
    if (graphs_off) return WOTG_OK;
    if (!gs) {
      if (cudaStreamCreateWithFlags(&gs, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&gev[0], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&gev[1], cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        release_graphs();
        graphs_off = true;
        return WOTG_OK;
      }
    }
    BatchGraph& G = bg[parity & 1];
    if (G.exec && G.nb != nb) {
      cudaGraphExecDestroy(G.exec);
      G = BatchGraph{};
    }
    bool fresh = false;
    if (!G.exec) {
      const unsigned long long before = launches_so_far();
      WOTG_CUDA(cudaStreamBeginCapture(gs, cudaStreamCaptureModeThreadLocal));
      const cudaStream_t user = st;
      st = gs;
      int s = WOTG_OK;
      int p = parity;
      for (int t = 0; t < nb && s == WOTG_OK; ++t) {
        s = iteration(c, t == 0, p);
        if (s == WOTG_OK) s = absorb(c, tau, p);
        p ^= 1;
      }
      st = user;
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(gs, &graph);
      cudaError_t ei = e;
      if (s == WOTG_OK && e == cudaSuccess) ei = cudaGraphInstantiate(&G.exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (s != WOTG_OK || ei != cudaSuccess) {
        // nothing of the batch ran (capture only) and the host state is the one
        // it started from: fall back to plain launches for the rest of the solve
        G = BatchGraph{};
        cudaGetLastError();
        graphs_off = true;
        return WOTG_OK;
      }
      G.launches = launches_so_far() - before;   // counted at capture, for the first replay
      G.nb = nb;
      fresh = true;
    }
    WOTG_CUDA(cudaEventRecord(gev[0], st));
    WOTG_CUDA(cudaStreamWaitEvent(gs, gev[0], 0));
    WOTG_CUDA(cudaGraphLaunch(G.exec, gs));
    WOTG_CUDA(cudaEventRecord(gev[1], gs));
    WOTG_CUDA(cudaStreamWaitEvent(st, gev[1], 0));
    if (!fresh) count_launches(G.launches);
    *used = true;
    return WOTG_OK;
  }

  // Solver outputs for one solve: learned row sums (device), optionally the
  // dense coupling and potentials.
  int outputs(const Coef& c, bool no_div_j, double* tmap, double* row_sums, double* ubar,
              double* vbar) {
    const double log_scale = no_div_j ? 0.0 : -c.logJ;
    if (row_sums) {
      row_sums_kernel<<<vec_blocks(g.I), 256, 0, st>>>(g, V, c, log_scale, row_sums);
      WOTG_LAUNCHED();
    }
    if (ubar || vbar) {
      potentials_kernel<<<vec_blocks(g.I + g.J), 256, 0, st>>>(g, V, c, ubar, vbar);
      WOTG_LAUNCHED();
    }
    if (tmap) {
      coupling_rows_kernel<<<vec_blocks(g.I), 256, 0, st>>>(g, V, c, log_scale);
      WOTG_LAUNCHED();
      // every column in one wave of x blocks (its weight read once per thread), rows over y
      dim3 grid((unsigned)std::min<int64_t>((g.J + 255) / 256, 65535), (unsigned)std::min<int64_t>(g.I, 128));
      coupling_kernel<<<grid, 256, 0, st>>>(C, g, V, c, log_scale, tmap);
      WOTG_LAUNCHED();
    }
    return WOTG_OK;
  }
};

// Frees a solver's captured graphs, stream and events when its entry point
// returns (every replay has completed by then: each batch is followed by a
// duality-gap check that synchronises the stream).
struct SolverGraphs {
  Solver& s;
  ~SolverGraphs() { s.release_graphs(); }
};

// Set for the duration of a no-alloc call: its solver creates no stream, event
// or graph of its own (plain launches on the caller's stream only).
static thread_local bool t_plain_launches = false;

struct SolveResult {
  int status = WOTG_OK;
  bool max_iter = false;
  int64_t iterations = 0;
  int64_t checks = 0;
  double gap = NAN;
  double eps = 0.0;
  Coef final_coef{};
};

// Python's max(x, y): returns x unless y > x (so a NaN in first position wins).
static inline double py_max(double x, double y) { return (y > x) ? y : x; }

static int solve_duality_gap(Solver& S, const wotg_params& P, double q, SolveResult& res) {
  const int n_scalings = 5;
  const double scale_factor = std::exp(-std::log(P.epsilon) / n_scalings);
  double eps_i = P.epsilon0 * scale_factor;
  int64_t it = 0;
  int parity = 0;
  double gap = INFINITY;
  Coef c{};
  bool lrow_valid = false;
  for (int stage = 0; stage <= n_scalings; ++stage) {
    gap = INFINITY;
    const double eps_old = eps_i;
    eps_i = eps_i / scale_factor;
    c = S.coef(eps_i, P, q);
    int s = S.rescale(eps_old, eps_i);
    if (s) return s;
    s = S.tc_prepare(c);
    if (s) return s;
    parity = 0;
    lrow_valid = false;
    const bool final = stage == n_scalings;
    const double threshold = final ? P.tolerance : 1e-6;
    double sumK = 0.0;
    if (final) {
      s = S.sum_exp(c, &sumK);
      if (s) return s;
    }
    S.drop_graphs();
    while (gap > threshold) {
      const int nb = final ? P.batch_size : 5;
      bool replayed = false;
      if (final && lrow_valid && S.steady() && (double)(it + nb) < P.max_iter) {
        s = S.batch_graph(c, nb, parity, P.tau, &replayed);
        if (s) return s;
      }
      if (replayed) {
        it += nb;
        lrow_valid = false;
        parity ^= (nb & 1);
      }
      for (int t = 0; t < nb && !replayed; ++t) {
        ++it;
        s = S.iteration(c, lrow_valid, parity);
        if (s) return s;
        lrow_valid = false;
        s = S.absorb(c, P.tau, parity);
        if (s) return s;
        parity ^= 1;
        if ((double)it >= P.max_iter) {
          res.max_iter = true;
          res.iterations = it;
          res.gap = gap;
          res.eps = eps_i;
          res.final_coef = c;
          s = S.fresh_lrow(c);
          if (s) return s;
          return WOTG_OK;
        }
      }
      double h[kNq];
      ++res.checks;
      if (final) {
        s = S.fresh_lrow(c);
        if (s) return s;
        lrow_valid = true;
        gap_partial_kernel<<<kRedBlocks, 256, 0, S.st>>>(S.g, S.V, c, S.V.red);
        WOTG_LAUNCHED();
        s = S.reduce_to_host(h);
        if (s) return s;
        const double I = (double)S.g.I, J = (double)S.g.J;
        const double dx = 1.0 / I, dy = 1.0 / J;
        const double gap_abs = dx * h[0] + dy * h[1];
        const double pri = P.lambda1 * dx * h[2] + P.lambda2 * dy * h[3] + dx * h[4] + dy * h[5] +
                           eps_i * (sumK / (I * J) - dx * h[6]);
        gap = gap_abs / std::fabs(pri);
      } else {
        stage_test_kernel<<<kRedBlocks, 256, 0, S.st>>>(S.g, S.V, c, S.V.red);
        WOTG_LAUNCHED();
        s = S.reduce_to_host(h);
        if (s) return s;
        const double ga = std::sqrt(h[0]) / (1.0 + std::sqrt(h[1]));
        const double gb = std::sqrt(h[2]) / (1.0 + std::sqrt(h[3]));
        gap = py_max(ga, gb);
      }
    }
  }
  res.iterations = it;
  res.gap = gap;
  res.eps = eps_i;
  res.final_coef = c;
  if (std::isnan(gap)) return WOTG_NONFINITE;
  // Lrow is valid (last gap check ran with the current b).
  return WOTG_OK;
}

static int solve_fixed_iters(Solver& S, const wotg_params& P, double q, SolveResult& res) {
  const double eps_final = P.epsilon;
  double eps_i = P.epsilon0;  // tau is never None here (the host rejects it)
  Coef c = S.coef(eps_i, P, q);
  int s = S.rescale(0.0, eps_i);
  if (s) return s;
  s = S.tc_prepare(c);
  if (s) return s;
  int parity = 0;
  int since = 0, index = 0;
  for (int it = 0; it < P.scaling_iter; ++it) {
    s = S.iteration(c, false, parity);
    if (s) return s;
    ++since;
    s = S.absorb(c, P.tau, parity);
    if (s) return s;
    parity ^= 1;
    if (since == P.inner_iter_max) {
      ++index;
      since = 0;
      const double eps_new = (P.epsilon0 - eps_final) * std::exp(-(double)index) + eps_final;
      s = S.rescale(eps_i, eps_new);
      if (s) return s;
      parity = 0;
      eps_i = eps_new;
      c = S.coef(eps_i, P, q);
      s = S.tc_prepare(c);
      if (s) return s;
    }
  }
  for (int it = 0; it < P.extra_iter; ++it) {
    s = S.iteration(c, false, parity);
    if (s) return s;
  }
  s = S.fresh_lrow(c);
  if (s) return s;
  res.iterations = (int64_t)P.scaling_iter + P.extra_iter;
  res.eps = eps_i;
  res.final_coef = c;
  return WOTG_OK;
}

// Resident 256-thread CTAs per SM of a kernel (6 when the query fails).
template <class K>
static int occupancy(K kernel) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, 256, 0) != cudaSuccess || n <= 0) return 6;
  return n;
}

static Geom make_geom(int64_t I, int64_t J, int64_t ldc) {
  Geom g;
  g.I = I;
  g.J = J;
  g.ldc = ldc;
  const int sms = sm_count();
  static const int occ_row = occupancy(row_pass_kernel<true, true>);
  static const int occ_col = occupancy(col_partial_kernel<true>);
  const int64_t max_warps = (int64_t)sms * occ_row * 8;
  const int64_t rows_per_warp = (I + max_warps - 1) / max_warps;
  const int64_t warps = (I + rows_per_warp - 1) / rows_per_warp;
  g.row_grid = (int)std::max<int64_t>(1, (warps + 7) / 8);
  const int64_t nv = ldc >> 2;
  g.ncb = (int)std::max<int64_t>(1, (nv + 255) / 256);
  int64_t nrb = std::max<int64_t>(1, ((int64_t)sms * occ_col) / g.ncb);
  nrb = std::min<int64_t>(nrb, std::max<int64_t>(1, I / 8));
  int64_t rows_per = (I + nrb - 1) / nrb;
  rows_per = (rows_per + kColRowChunk - 1) / kColRowChunk * kColRowChunk;
  g.rows_per = rows_per;
  g.nrb = (int)((I + rows_per - 1) / rows_per);
  return g;
}

static size_t layout(Bump& b, const Geom& g, Vecs& V) {
  V.u = b.take<double>(g.I);
  V.la = b.take<double>(g.I);
  V.la_old = b.take<double>(g.I);
  V.logp = b.take<double>(g.I);
  V.p = b.take<double>(g.I);
  V.Lrow = b.take<double>(g.I);
  V.v = b.take<double>(g.J);
  V.lb = b.take<double>(g.J);
  V.lb_old = b.take<double>(g.J);
  V.Lcol = b.take<double>(g.J);
  V.rowc = b.take<float4>(g.I);
  V.wrow = b.take<float>(g.I);
  V.wcol = b.take<float>(g.ldc);
  V.wrow_lo = b.take<float>(g.I);
  V.wcol_lo = b.take<float>(g.ldc);
  V.part = b.take<float2>((size_t)g.nrb * g.ldc);
  V.maxslot = b.take<unsigned long long>(2);
  V.red = b.take<double>((size_t)kRedBlocks * kNq);
  V.scal = b.take<double>(16);
  V.counters = b.take<int>(8);
  V.scal = V.scal;
  return b.off + 256;
}

}  // namespace wotg

using namespace wotg;

extern "C" size_t wotg_lse_matvec_workspace_bytes(int64_t I, int64_t J, int64_t ldc) {
  if (I <= 0 || J <= 0 || ldc < J) return 0;
  Geom g = make_geom(I, J, ldc);
  return (size_t)g.nrb * (size_t)ldc * sizeof(float2) + 256;
}

extern "C" int wotg_lse_matvec(const float* C, int64_t I, int64_t J, int64_t ldc, const float* w, float kappa2,
                               int32_t axis, double* L, void* workspace, size_t workspace_bytes, void* stream) {
  if (!C || !w || !L || I <= 0 || J <= 0 || ldc < J || (ldc & 3) || (axis != 0 && axis != 1)) return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(C) & 15) || (axis == 0 && (reinterpret_cast<uintptr_t>(w) & 15)))
    return WOTG_BADARG;
  Geom g = make_geom(I, J, ldc);
  Vecs V{};
  Coef c{};
  c.kappa2 = kappa2;
  cudaStream_t st = (cudaStream_t)stream;
  if (axis == 0) {
    V.wcol = const_cast<float*>(w);
    V.Lrow = L;
    row_pass_kernel<false, false><<<g.row_grid, 256, 0, st>>>(C, g, V, c, 0);
    WOTG_LAUNCHED();
    return WOTG_OK;
  }
  if (!workspace || workspace_bytes < wotg_lse_matvec_workspace_bytes(I, J, ldc)) return WOTG_WORKSPACE;
  V.wrow = const_cast<float*>(w);
  V.Lcol = L;
  V.part = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  col_partial_kernel<false><<<dim3(g.ncb, g.nrb), 256, 0, st>>>(C, g, V, c);
  WOTG_LAUNCHED();
  col_combine_kernel<false, false><<<(unsigned)((J + 255) / 256), 256, 0, st>>>(g, V, c, 0);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

static bool tc_requested(const wotg_problem* prob) { return prob->form == WOTG_FORM_ONTHEFLY; }

static int tc_valid(const wotg_problem* prob) {
  if (!tc_requested(prob)) return prob->form == WOTG_FORM_MATERIALIZED ? WOTG_OK : WOTG_BADARG;
  if (!(prob->cost_scale > 0)) return WOTG_BADARG;
  if (!prob->X || !prob->Y || prob->d < 1 || prob->d > tc_max_dim() || prob->ldx < prob->d || prob->ldy < prob->d)
    return WOTG_BADARG;
  return WOTG_OK;
}

static void tc_layout(Bump& b, const wotg_problem* prob, TcState& tc) {
  tc.on = true;
  tc.kp = tc_kp(prob->d);
  tc.n_xt = (int)((prob->I + 127) / 128);
  tc.n_yt = (int)((prob->J + 127) / 128);
  tc.I_pad = (int64_t)tc.n_xt * 128;
  tc.J_pad = (int64_t)tc.n_yt * 128;
  const int slots = sm_count() * std::max(1, tc_ctas_per_sm(tc.kp));
  tc.ctas_row = (int)std::min<int64_t>(slots, (int64_t)tc.n_xt * tc.n_yt);
  tc.ctas_col = (int)std::min<int64_t>(slots, (int64_t)tc.n_yt * tc.n_xt);
  const size_t tb = tc_tile_bytes(tc.kp);
  tc.Xa = reinterpret_cast<__half*>(b.take<unsigned char>(tb * tc.n_xt));
  tc.Xb = reinterpret_cast<__half*>(b.take<unsigned char>(tb * tc.n_xt));
  tc.Ya = reinterpret_cast<__half*>(b.take<unsigned char>(tb * tc.n_yt));
  tc.Yb = reinterpret_cast<__half*>(b.take<unsigned char>(tb * tc.n_yt));
  tc.X = prob->X;
  tc.Y = prob->Y;
  tc.ldx = prob->ldx;
  tc.ldy = prob->ldy;
  tc.d = prob->d;
  tc.normX = b.take<double>(prob->I);
  tc.normY = b.take<double>(prob->J);
  tc.part = b.take<float2>((size_t)(std::max(tc.ctas_row, tc.ctas_col) + std::max(tc.n_xt, tc.n_yt)) * 128 *
                           tc_parts());
  tc.err = b.take<int>(4);
  tc.offX = b.take<float>(tc.I_pad);
  tc.offY = b.take<float>(tc.J_pad);
  tc.redoX = b.take<int>(2 + prob->I);
  tc.redoY = b.take<int>(2 + prob->J);
  tc.tile_ctr = b.take<int>((size_t)4 * std::max(tc.n_xt, tc.n_yt));
  tc.redo_total = b.take<unsigned long long>(1);
  tc.off_row_ok = tc.off_col_ok = false;
  tc.xb_ok = tc.yb_ok = false;
}

extern "C" size_t wotg_problem_workspace_bytes(const wotg_problem* prob) {
  if (!prob || prob->I <= 0 || prob->J <= 0 || prob->ldc < prob->J || tc_valid(prob) != WOTG_OK) return 0;
  Geom g = make_geom(prob->I, prob->J, prob->ldc);
  Bump b{nullptr, 0};
  Vecs V{};
  b.take<double>(prob->I);
  size_t n = layout(b, g, V);
  if (tc_requested(prob)) {
    TcState tc{};
    tc_layout(b, prob, tc);
    n = b.off + 256;
  }
  return n;
}

extern "C" size_t wotg_solve_workspace_bytes(int64_t I, int64_t J, int64_t ldc) {
  if (I <= 0 || J <= 0 || ldc < J) return 0;
  Geom g = make_geom(I, J, ldc);
  Bump b{nullptr, 0};
  Vecs V{};
  // extra I doubles: learned-growth carry between growth iterations
  b.take<double>(I);
  return layout(b, g, V);
}

extern "C" int wotg_compute_transport_matrix(const wotg_problem* prob, const wotg_params* params,
                                             double* tmap, double* learned_growth, double* row_sums,
                                             double* u_bar, double* v_bar, wotg_stats* stats,
                                             void* workspace, size_t workspace_bytes, void* stream) {
  if (!prob || !params) return WOTG_BADARG;
  const wotg_params P = *params;
  const int64_t I = prob->I, J = prob->J, ldc = prob->ldc;
  if (I <= 0 || J <= 0 || ldc < J || (ldc & 3) || !prob->C || !prob->G) return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(prob->C) & 15) != 0) return WOTG_BADARG;
  if (!(P.epsilon > 0) || !(P.epsilon0 > 0) || P.growth_iters < 1) return WOTG_BADARG;
  if (P.solver == WOTG_SOLVER_DUALITY_GAP) {
    if (P.batch_size < 1) return WOTG_BADARG;
  } else if (P.solver == WOTG_SOLVER_FIXED_ITERS) {
    if (P.scaling_iter < 1 || P.extra_iter < 0) return WOTG_BADARG;
  } else {
    return WOTG_BADARG;
  }
  if (tc_valid(prob) != WOTG_OK) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_problem_workspace_bytes(prob)) return WOTG_WORKSPACE;

  Geom g = make_geom(I, J, ldc);
  // layout() leaves 256 bytes of slack for aligning the caller's base pointer
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  double* carry = b.take<double>(I);
  Vecs V{};
  layout(b, g, V);
  cudaStream_t st = (cudaStream_t)stream;
  Solver S{prob->C, g, V, st, prob->cost_scale, 0, TcState{}};
  SolverGraphs graphs_guard{S};
  S.graphs_off = t_plain_launches;
  if (tc_requested(prob)) {
    tc_layout(b, prob, S.tc);
    WOTG_CUDA(cudaMemsetAsync(S.tc.err, 0, sizeof(int), st));
    WOTG_CUDA(cudaMemsetAsync(S.tc.redo_total, 0, sizeof(unsigned long long), st));
    // column forms (coordinates; bias columns written per half-step) and norms
    const float sigma = (float)std::sqrt(prob->cost_scale);
    int s = tc_pack_points(prob->X, I, prob->ldx, prob->d, S.tc.kp, sigma, 0, S.tc.Xb, S.tc.normX, st);
    if (s) return s;
    s = tc_pack_points(prob->Y, J, prob->ldy, prob->d, S.tc.kp, sigma, 0, S.tc.Yb, S.tc.normY, st);
    if (s) return s;
  }

  wotg_stats total{};
  int status = WOTG_OK;
  const double* G = prob->G;
  for (int gi = 0; gi < P.growth_iters; ++gi) {
    if (learned_growth) {
      WOTG_CUDA(cudaMemcpyAsync(learned_growth + (int64_t)gi * I, G, I * sizeof(double),
                                cudaMemcpyDeviceToDevice, st));
    }
    init_kernel<<<S.vec_blocks(std::max(I, ldc)), 256, 0, st>>>(g, V, G);
    WOTG_LAUNCHED();
    double q = 0.0;
    int s = S.mean_of(V.p, I, &q);
    if (s) return s;
    SolveResult res;
    s = (P.solver == WOTG_SOLVER_DUALITY_GAP) ? solve_duality_gap(S, P, q, res)
                                              : solve_fixed_iters(S, P, q, res);
    int absorptions = 0;
    WOTG_CUDA(cudaMemcpyAsync(&absorptions, V.counters, sizeof(int), cudaMemcpyDeviceToHost, st));
    WOTG_CUDA(cudaStreamSynchronize(st));
    total.iterations += res.iterations;
    total.absorptions += absorptions;
    total.checks += res.checks;
    total.gap = res.gap;
    total.final_epsilon = res.eps;
    if (s == WOTG_NONFINITE) {
      status = WOTG_NONFINITE;
      break;
    }
    if (s) return s;
    if (res.max_iter) {
      total.hit_max_iter = 1;
      status = WOTG_MAX_ITER;
    }
    const bool last = gi == P.growth_iters - 1;
    if (!last) {
      s = S.outputs(res.final_coef, res.max_iter, nullptr, carry, nullptr, nullptr);
      if (s) return s;
      G = carry;
    } else {
      s = S.outputs(res.final_coef, res.max_iter, tmap, row_sums, u_bar, v_bar);
      if (s) return s;
    }
  }
  WOTG_CUDA(cudaStreamSynchronize(st));
  if (S.tc.on) {
    int err = 0;
    WOTG_CUDA(cudaMemcpy(&err, S.tc.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      set_last_message("tensor-core half-step: a bounded wait timed out");
      return WOTG_CUDA_ERROR;
    }
    unsigned long long redo = 0;
    WOTG_CUDA(cudaMemcpy(&redo, S.tc.redo_total, sizeof(redo), cudaMemcpyDeviceToHost));
    total.exact_rows = (int32_t)std::min<unsigned long long>(redo, 0x7fffffffull);
  }
  if (stats) *stats = total;
  return status;
}

// Warm-started fixed-epsilon iterations (no counterpart in the reference; its
// iterations at the final epsilon are optimal_transport.py:131-141): from
// absorbed potentials (u_bar, v_bar), n_iter iterations of the reference's a/b
// updates with tau-absorption at `epsilon`, potentials written back in place.
// Polishes a solve stopped on the duality gap towards the exact optimum (used
// before differentiating the objective).
extern "C" int wotg_refine_potentials(const wotg_problem* prob, const wotg_params* params, double epsilon,
                                      int32_t n_iter, double* u_bar, double* v_bar, wotg_stats* stats,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  if (!prob || !params || !u_bar || !v_bar || n_iter < 0 || !(epsilon > 0)) return WOTG_BADARG;
  const wotg_params P = *params;
  const int64_t I = prob->I, J = prob->J, ldc = prob->ldc;
  if (I <= 0 || J <= 0 || ldc < J || (ldc & 3) || !prob->C || !prob->G) return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(prob->C) & 15) != 0) return WOTG_BADARG;
  if (tc_valid(prob) != WOTG_OK) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_problem_workspace_bytes(prob)) return WOTG_WORKSPACE;
  Geom g = make_geom(I, J, ldc);
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  b.take<double>(I);
  Vecs V{};
  layout(b, g, V);
  cudaStream_t st = (cudaStream_t)stream;
  Solver S{prob->C, g, V, st, prob->cost_scale, 0, TcState{}};
  SolverGraphs graphs_guard{S};
  S.graphs_off = t_plain_launches;
  if (tc_requested(prob)) {
    tc_layout(b, prob, S.tc);
    WOTG_CUDA(cudaMemsetAsync(S.tc.err, 0, sizeof(int), st));
    WOTG_CUDA(cudaMemsetAsync(S.tc.redo_total, 0, sizeof(unsigned long long), st));
    const float sigma = (float)std::sqrt(prob->cost_scale);
    int s = tc_pack_points(prob->X, I, prob->ldx, prob->d, S.tc.kp, sigma, 0, S.tc.Xb, S.tc.normX, st);
    if (s) return s;
    s = tc_pack_points(prob->Y, J, prob->ldy, prob->d, S.tc.kp, sigma, 0, S.tc.Yb, S.tc.normY, st);
    if (s) return s;
  }
  init_kernel<<<S.vec_blocks(std::max(I, ldc)), 256, 0, st>>>(g, V, prob->G);
  WOTG_LAUNCHED();
  double q = 0.0;
  int s = S.mean_of(V.p, I, &q);
  if (s) return s;
  const Coef c = S.coef(epsilon, P, q);
  load_potentials_kernel<<<S.vec_blocks(I + J), 256, 0, st>>>(g, V, u_bar, v_bar, c.inv_eps);
  WOTG_LAUNCHED();
  s = S.tc_prepare(c);
  if (s) return s;
  int parity = 0;
  for (int it = 0; it < n_iter; ++it) {
    s = S.iteration(c, false, parity);
    if (s) return s;
    s = S.absorb(c, P.tau, parity);
    if (s) return s;
    parity ^= 1;
  }
  s = S.outputs(c, false, nullptr, nullptr, u_bar, v_bar);
  if (s) return s;
  WOTG_CUDA(cudaStreamSynchronize(st));
  wotg_stats out{};
  out.iterations = n_iter;
  out.final_epsilon = epsilon;
  out.gap = NAN;
  {
    int absorptions = 0;
    WOTG_CUDA(cudaMemcpy(&absorptions, V.counters, sizeof(int), cudaMemcpyDeviceToHost));
    out.absorptions = absorptions;
  }
  if (S.tc.on) {
    int err = 0;
    WOTG_CUDA(cudaMemcpy(&err, S.tc.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      set_last_message("tensor-core half-step: a bounded wait timed out");
      return WOTG_CUDA_ERROR;
    }
    unsigned long long redo = 0;
    WOTG_CUDA(cudaMemcpy(&redo, S.tc.redo_total, sizeof(redo), cudaMemcpyDeviceToHost));
    out.exact_rows = (int32_t)std::min<unsigned long long>(redo, 0x7fffffffull);
  }
  if (stats) *stats = out;
  return WOTG_OK;
}

// ---------------------------------------------------------------------------
// No-allocation variant of wotg_compute_transport_matrix.
//
// Some callers cannot call cudaMalloc: hosts whose device memory is owned by
// another allocator or pool (a JVM or Go service handing out pre-sized
// buffers, a framework that forbids raw device allocations) and code paths
// where cudaMalloc's implicit device synchronisation is not acceptable. They
// still pass every input and output buffer, but get the solver's scratch from
// the file-scope array below instead of a caller workspace.
//
// The array is wotg_noalloc_scratch_bytes() = 32 MiB on every device that
// loads this module and stays allocated until the process exits. Its device
// address is looked up once per device, on that device's first call, with
// cudaGetSymbolAddress (host code cannot use the symbol itself: on the host it
// names a stand-in, not device memory); make that first call before any stream
// capture. The looked-up address is cached per device for the life of the
// process; it does not survive cudaDeviceReset (or any other teardown of the
// device's primary context), after which this entry point must not be called
// again in the process. All calls share the array: calls whose work overlaps
// on the GPU (other streams, other host threads) race on it, so serialise
// them. The solver re-initialises everything it reads from the scratch at the
// start of each solve (state vectors, max slots, counters, the tensor-core
// form's packed points and error word), so no clearing between calls is
// needed.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
constexpr int kNoAllocMaxDevices = 64;
std::atomic<void*> g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

extern "C" size_t wotg_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int wotg_compute_transport_matrix_noalloc(const wotg_problem* prob, const wotg_params* params,
                                                     double* tmap, double* learned_growth, double* row_sums,
                                                     double* u_bar, double* v_bar, wotg_stats* stats,
                                                     void* stream) {
  if (!prob || !params) return WOTG_BADARG;
  const int64_t I = prob->I, J = prob->J, ldc = prob->ldc;
  if (I <= 0 || J <= 0 || ldc < J || (ldc & 3) || !prob->C || !prob->G || tc_valid(prob) != WOTG_OK)
    return WOTG_BADARG;
  const size_t need = wotg_problem_workspace_bytes(prob);
  if (need == 0) return WOTG_BADARG;
  if (need > kNoAllocScratchBytes) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "wotg_compute_transport_matrix_noalloc: a %lld x %lld problem needs %zu bytes of scratch, "
             "more than the %zu-byte static array",
             (long long)I, (long long)J, need, kNoAllocScratchBytes);
    wotg::set_last_message(msg);
    return WOTG_TOO_LARGE;
  }
  int dev = 0;
  WOTG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return WOTG_BADARG;
  void* scratch = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    // set-up, once per device with that device current (two threads racing here
    // look up and store the same address)
    WOTG_CUDA(cudaGetSymbolAddress(&scratch, g_noalloc_scratch));
    g_noalloc_ptr[dev].store(scratch, std::memory_order_release);
  }
  struct Plain {
    Plain() { t_plain_launches = true; }
    ~Plain() { t_plain_launches = false; }
  } plain;
  return wotg_compute_transport_matrix(prob, params, tmap, learned_growth, row_sums, u_bar, v_bar, stats,
                                       scratch, kNoAllocScratchBytes, stream);
}
