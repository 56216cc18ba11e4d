// wotg_adjoint.cu — gradient of the converged unbalanced entropic OT objective
// with respect to the point sets and the source growth (sm_103a).
//
// The objective is the reference's dual at convergence (optimal_transport.py:56-62,
// the quantity its duality-gap test drives to the primal):
//   D = - lambda1 dx sum_i p_i (exp(-ubar_i / lambda1) - 1)
//       - lambda2 dy q sum_j   (exp(-vbar_j / lambda2) - 1)
//       - eps / (I J) sum_ij (R_ij - K0_ij),
//   R_ij = exp((ubar_i + vbar_j - C_ij) / eps),  K0_ij = exp(-C_ij / eps),
//   C_ij = s |x_i - y_j|^2,  dx = 1/I, dy = 1/J, q = mean(p)  (optimal_transport.py:106-108),
// with (ubar, vbar) = (u + eps log a, v + eps log b) its maximisers. By the
// envelope theorem the gradient at the optimum is the partial derivative with
// the potentials held fixed:
//   dD/dx_i = 2 s / (I J) sum_j (R_ij - K0_ij) (x_i - y_j)
//   dD/dy_j = 2 s / (I J) sum_i (R_ij - K0_ij) (y_j - x_i)
//   dD/dp_i = - lambda1 dx (exp(-ubar_i / lambda1) - 1) + (1 / I) dD/dq,
//   dD/dq   = - lambda2 dy sum_j (exp(-vbar_j / lambda2) - 1).
// The two point-set terms are one pass each over the implicit coupling, with the
// cost recomputed from the points tile by tile (never stored): a warp per point,
// 64 partner points per shared-memory tile, the distance in difference form
// (no |x|^2 + |y|^2 - 2 x.y cancellation), FP32 per-lane sums merged in FP64.
#include <algorithm>
#include <cmath>

#include "wotg_common.cuh"

namespace wotg {
namespace adj {

constexpr int kTile = 64;
constexpr int kWarps = 8;

// One side: for every point i of P (n x d), with partners Q (m x d):
//   r_i = sum_j R_ij, k_i = sum_j K0_ij, g_i = coef (x_i (r_i - k_i) - sum_j (R_ij - K0_ij) y_j)
// in base 2: R_ij = 2^(A_i + B_j - sk2 c_ij), K0_ij = 2^(-sk2 c_ij).
template <int D>
__global__ void __launch_bounds__(kWarps * 32) side_kernel(const float* __restrict__ P, int64_t ldp, int64_t n,
                                                           const float* __restrict__ Q, int64_t ldq, int64_t m, int d,
                                                           const double* __restrict__ pot_p,
                                                           const double* __restrict__ pot_q, float inv_eps2,
                                                           float sk2, double coef, double* __restrict__ grad,
                                                           double* __restrict__ rk) {
  __shared__ float sQ[kTile][D + 1];
  __shared__ float sB[kTile];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kWarps + warp;
  const bool valid = i < n;
  float x[D], acc[D];
#pragma unroll
  for (int t = 0; t < D; ++t) {
    x[t] = (valid && t < d) ? P[i * ldp + t] : 0.f;
    acc[t] = 0.f;
  }
  const float A = valid ? (float)(pot_p[i] * (double)inv_eps2) : 0.f;
  float r = 0.f, k = 0.f;
  for (int64_t j0 = 0; j0 < m; j0 += kTile) {
    __syncthreads();
    for (int e = threadIdx.x; e < kTile * D; e += blockDim.x) {
      const int jj = e / D, t = e % D;
      const int64_t j = j0 + jj;
      sQ[jj][t] = (j < m && t < d) ? Q[j * ldq + t] : 0.f;
    }
    for (int jj = threadIdx.x; jj < kTile; jj += blockDim.x) {
      const int64_t j = j0 + jj;
      sB[jj] = j < m ? (float)(pot_q[j] * (double)inv_eps2) : -INFINITY;
    }
    __syncthreads();
    if (!valid) continue;
#pragma unroll
    for (int h = 0; h < kTile / 32; ++h) {
      const int jj = lane + 32 * h;
      float c = 0.f;
#pragma unroll
      for (int t = 0; t < D; ++t) {
        const float df = x[t] - sQ[jj][t];
        c = fmaf(df, df, c);
      }
      const float e1 = ex2(A + sB[jj] - sk2 * c);
      const float e2 = j0 + jj < m ? ex2(-sk2 * c) : 0.f;
      const float w = e1 - e2;
      r += e1;
      k += e2;
#pragma unroll
      for (int t = 0; t < D; ++t) acc[t] = fmaf(w, sQ[jj][t], acc[t]);
    }
  }
  if (!valid) return;
  const double rd = warp_sum((double)r), kd = warp_sum((double)k);
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const double a = warp_sum((double)acc[t]);
    if (lane == 0 && t < d) grad[i * d + t] = coef * ((double)x[t] * (rd - kd) - a);
  }
  if (lane == 0) {
    rk[2 * i] = rd;
    rk[2 * i + 1] = kd;
  }
}

// Growth gradient and the objective's terms (one CTA; FP64):
//   out[0] = sum_i r_i - sum_i k_i    out[1] = sum_i p_i (exp(-ubar_i/lambda1) - 1)
//   out[2] = sum_j (exp(-vbar_j/lambda2) - 1)   out[3] = sum_i p_i
__global__ void terms_kernel(const double* __restrict__ rk, int64_t I, int64_t J, const double* __restrict__ ubar,
                             const double* __restrict__ vbar, const double* __restrict__ p, double lambda1,
                             double lambda2, double* __restrict__ out) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = threadIdx.x; i < I; i += blockDim.x) {
    acc[0] += rk[2 * i] - rk[2 * i + 1];
    acc[1] += p[i] * (exp(-ubar[i] / lambda1) - 1.0);
    acc[3] += p[i];
  }
  for (int64_t j = threadIdx.x; j < J; j += blockDim.x) acc[2] += exp(-vbar[j] / lambda2) - 1.0;
  __shared__ double sh[4][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double v = warp_sum(acc[q]);
    if (lane == 0) sh[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[threadIdx.x][w];
    out[threadIdx.x] = t;
  }
}

__global__ void grad_p_kernel(int64_t I, int64_t J, const double* __restrict__ ubar, double lambda1,
                              double lambda2, const double* __restrict__ terms, double* __restrict__ gp) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= I) return;
  const double dx = 1.0 / (double)I, dy = 1.0 / (double)J;
  const double dq = -lambda2 * dy * terms[2];
  gp[i] = -lambda1 * dx * (exp(-ubar[i] / lambda1) - 1.0) + dq / (double)I;
}

template <int D>
static void launch_side(const float* P, int64_t ldp, int64_t n, const float* Q, int64_t ldq, int64_t m, int d,
                        const double* pp, const double* pq, float inv_eps2, float sk2, double coef, double* grad,
                        double* rk, cudaStream_t st) {
  const unsigned blocks = (unsigned)((n + kWarps - 1) / kWarps);
  side_kernel<D><<<blocks, kWarps * 32, 0, st>>>(P, ldp, n, Q, ldq, m, d, pp, pq, inv_eps2, sk2, coef, grad, rk);
}

}  // namespace adj
}  // namespace wotg

using namespace wotg;

extern "C" size_t wotg_ot_adjoint_workspace_bytes(int64_t I, int64_t J) {
  if (I <= 0 || J <= 0) return 0;
  return (size_t)(2 * std::max(I, J) + 8) * sizeof(double) + 512;
}

extern "C" int wotg_ot_adjoint(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy,
                               int32_t d, double cost_scale, double epsilon, double lambda1, double lambda2,
                               const double* u_bar, const double* v_bar, const double* p, double* grad_x,
                               double* grad_y, double* grad_p, double* objective, void* workspace,
                               size_t workspace_bytes, void* stream) {
  if (!X || !Y || !u_bar || !v_bar || !p || !grad_x || I <= 0 || J <= 0 || d < 1 || d > 64 || ldx < d ||
      ldy < d)
    return WOTG_BADARG;
  if (!(cost_scale > 0) || !(epsilon > 0) || !(lambda1 > 0) || !(lambda2 > 0)) return WOTG_BADARG;
  if (I > (int64_t)1 << 31 || J > (int64_t)1 << 31) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_ot_adjoint_workspace_bytes(I, J)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  double* base = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  double* rk = base;                                   // 2 max(I, J)
  double* terms = base + 2 * std::max(I, J);           // 4
  const double log2e = 1.4426950408889634;
  const float inv_eps2 = (float)(log2e / epsilon);
  const float sk2 = (float)(cost_scale / epsilon * log2e);
  const double coef = 2.0 * cost_scale / ((double)I * (double)J);
  // column side first (its r, k are not needed), then the row side, whose r, k feed the objective
  if (grad_y) {
    if (d <= 32)
      adj::launch_side<32>(Y, ldy, J, X, ldx, I, d, v_bar, u_bar, inv_eps2, sk2, coef, grad_y, rk, st);
    else
      adj::launch_side<64>(Y, ldy, J, X, ldx, I, d, v_bar, u_bar, inv_eps2, sk2, coef, grad_y, rk, st);
    WOTG_LAUNCHED();
  }
  // the row side (its r, k feed the objective)
  if (d <= 32)
    adj::launch_side<32>(X, ldx, I, Y, ldy, J, d, u_bar, v_bar, inv_eps2, sk2, coef, grad_x, rk, st);
  else
    adj::launch_side<64>(X, ldx, I, Y, ldy, J, d, u_bar, v_bar, inv_eps2, sk2, coef, grad_x, rk, st);
  WOTG_LAUNCHED();
  adj::terms_kernel<<<1, 1024, 0, st>>>(rk, I, J, u_bar, v_bar, p, lambda1, lambda2, terms);
  WOTG_LAUNCHED();
  if (grad_p) {
    adj::grad_p_kernel<<<(unsigned)((I + 255) / 256), 256, 0, st>>>(I, J, u_bar, lambda1, lambda2, terms, grad_p);
    WOTG_LAUNCHED();
  }
  if (objective) {
    double h[4];
    WOTG_CUDA(cudaMemcpyAsync(h, terms, sizeof(h), cudaMemcpyDeviceToHost, st));
    WOTG_CUDA(cudaStreamSynchronize(st));
    const double dx = 1.0 / (double)I, dy = 1.0 / (double)J;
    const double q = h[3] / (double)I;
    *objective = -lambda1 * dx * h[1] - lambda2 * dy * q * h[2] - epsilon * dx * dy * h[0];
  }
  return WOTG_OK;
}
