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
#include "wotg_tc_kernel.cuh"

namespace wotg {

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

// Resident CTAs per SM of the half-step kernel.
int tc_ctas_per_sm(int kp) {
  (void)kp;
  return kTcCtasPerSm;
}
int tc_parts() { return kTcParts; }

int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nq, int kp, int ctas, float2* part,
                  const float* off, int* err, cudaStream_t st, uint32_t wait_tries) {
  if (kp == 32) {
    WOTG_CUDA(tc_set_smem_attr<32>());
    lse_tc_kernel<32, 0><<<ctas, kTcThreads, TcSmem<32>::kAlloc, st>>>(Pt, Qt, n_ptiles, nq, part, off, err,
                                                                        wait_tries, nullptr, 0, 0, nullptr, NoFin{});
  } else if (kp == 64) {
    WOTG_CUDA(tc_set_smem_attr<64>());
    lse_tc_kernel<64, 0><<<ctas, kTcThreads, TcSmem<64>::kAlloc, st>>>(Pt, Qt, n_ptiles, nq, part, off, err,
                                                                        wait_tries, nullptr, 0, 0, nullptr, NoFin{});
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
          P.Xa, P.Yb, P.n_xt, P.n_yt, P.part, nullptr, P.err, kTcWaitTries, popw, kc, (int)jpad, psum, NoFin{});
    } else {
      WOTG_CUDA((tc_set_smem_attr<64, kTcPops>()));
      lse_tc_kernel<64, kTcPops><<<P.ctas, kTcThreads, TcSmem<64>::kAlloc, st>>>(
          P.Xa, P.Yb, P.n_xt, P.n_yt, P.part, nullptr, P.err, kTcWaitTries, popw, kc, (int)jpad, psum, NoFin{});
    }
    WOTG_LAUNCHED();
    pop_finish_kernel<<<(unsigned)((I + 255) / 256), 256, 0, st>>>(I, P.n_yt, P.ctas, kTcParts, P.part, psum,
                                                                  kTcPops, k0, kc, P.normX, scale, bias, out);
    WOTG_LAUNCHED();
  }
  return WOTG_OK;
}
