// wotg_onthefly.cuh — host-side launchers of the tensor-core (on-the-fly) cost path.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "wotg_tc.cuh"

namespace wotg {

// Bytes of one packed 128-point tile (FP16 hi + lo blocks of 128 x kp halfs).
inline size_t tc_tile_bytes(int kp) { return (size_t)2 * 128 * kp * sizeof(__half); }
// Padded dimension of the packed tiles (multiple of 16 halfs: one MMA K-step),
// with two spare columns for the bias; d <= tc_max_dim().
inline int tc_kp(int d) { return d + 2 <= 32 ? 32 : 64; }
inline int tc_max_dim() { return 62; }

// Row form (row_form = 1): [scale x, 1, 1]; column form: [x, bias columns];
// norm (optional) receives |x_i|^2 in FP64.
int tc_pack_points(const float* X, int64_t n, int64_t ldx, int d, int kp, float scale, int row_form,
                   __half* tiles, double* norm, cudaStream_t st);
// Column-form bias columns: bias_i = (pot_i / eps + lsc_i) log2 e - kappa2 norm_i.
int tc_pack_bias(int64_t n, const double* pot, const double* lsc, const double* norm, double inv_eps,
                 double kappa2d, int d, int kp, __half* tiles, cudaStream_t st);
// Column-form bias of point i in tiles packed by tc_pack_points: the FP64 bias
// carried as beta1 + beta2 (beta1 = fp32(bias), beta2 the remainder after
// beta1's FP16 hi/lo split; ~44 bits), each split into the hi and lo halves of
// the two bias columns d and d + 1. -inf (and below -60000) -> -60000, i.e.
// weight 0; NaN / +inf -> NaN, so that non-finite potentials propagate.
__device__ __forceinline__ void tc_write_bias(int64_t i, double beta, int d, int kp, __half* tiles) {
  __half h1, l1, h2, l2;
  const __half zero = __float2half_rn(0.f);
  if (beta != beta || beta == INFINITY) {
    h1 = __float2half_rn(NAN);
    l1 = h2 = l2 = zero;
  } else if (beta < -60000.0) {
    h1 = __float2half_rn(-60000.f);
    l1 = h2 = l2 = zero;
  } else {
    const float b1 = (float)beta;
    tc::split_f16(b1, h1, l1);
    const float b2 = (float)(beta - (double)__half2float(h1) - (double)__half2float(l1));
    tc::split_f16(b2, h2, l2);
  }
  __half* tile = tiles + (i / 128) * ((int64_t)2 * 128 * kp);
  const uint32_t o1 = tc::core_offset((int)(i % 128), d, kp) >> 1;
  const uint32_t o2 = tc::core_offset((int)(i % 128), d + 1, kp) >> 1;
  tile[o1] = h1;
  tile[o2] = h2;
  tile[128 * kp + o1] = l1;
  tile[128 * kp + o2] = l2;
}

// Where a kernel that changes the potential or the log-scaling of a point
// writes that point's column-form bias (tiles = nullptr: nowhere):
//   bias_i = (pot_i / eps + lsc_i) log2 e - kappa log2 e |x_i|^2.
struct TcBias {
  __half* tiles;
  const double* norm;
  int d, kp;
};

// Resident CTAs per SM of the tensor-core half-step kernel.
int tc_ctas_per_sm(int kp);
// First flattened (row tile, column tile) index of CTA c's stretch, and the CTA
// whose stretch holds index f, for `total` tiles cut into `ctas` stretches.
__host__ __device__ __forceinline__ int64_t tc_stretch_begin(int64_t c, int64_t total, int64_t ctas) {
  return c * total / ctas;
}
__host__ __device__ __forceinline__ int64_t tc_cta_of(int64_t f, int64_t total, int64_t ctas) {
  return ((f + 1) * ctas - 1) / total;
}

// Partials per row and segment (column groups of the epilogue warps).
int tc_parts();
// Persistent launch over n_ptiles x nq tile pairs with `ctas` CTAs; partial of
// (CTA c, row tile t, row r, column group k) at part[((c + t) * 128 + r) * tc_parts() + k]:
// (ctas + n_ptiles) * 128 * tc_parts() float2.
// off (optional, n_ptiles x 128 floats): speculative form, each row's partial
// is (off_row, sum 2^(d - off_row)); NULL: exact running-maximum form.
// wait_tries bounds each of the kernel's mbarrier waits (tries of up to 1 us);
// a wait that runs out sets *err (see lse_tc_kernel).
constexpr uint32_t kTcDefaultWaitTries = 4000000;
int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nq, int kp, int ctas, float2* part,
                  const float* off, int* err, cudaStream_t st, uint32_t wait_tries = kTcDefaultWaitTries);

}  // namespace wotg
