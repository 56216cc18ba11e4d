// wotg_onthefly.cuh — host-side launchers of the tensor-core (on-the-fly) cost path.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

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
