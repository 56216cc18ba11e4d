// wotg_onthefly.cuh — host-side launchers of the tensor-core (on-the-fly) cost path.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace wotg {

// Bytes of one packed 128-point tile (FP16 hi + lo blocks of 128 x kp halfs).
inline size_t tc_tile_bytes(int kp) { return (size_t)2 * 128 * kp * sizeof(__half); }
// Padded dimension of the packed tiles (multiple of 16 halfs: one MMA K-step).
inline int tc_kp(int d) { return d <= 32 ? 32 : 64; }

int tc_pack_points(const float* X, int64_t n, int64_t ldx, int d, int kp, __half* tiles, double* norm,
                   cudaStream_t st);
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

// Persistent launch over n_ptiles x nq tile pairs with `ctas` CTAs; partial of
// (CTA c, row tile t, row r, column quarter k) at part[((c + t) * 128 + r) * 4 + k]:
// (ctas + n_ptiles) * 512 float2.
int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nq, const float* bias, int kp,
                  float gamma, int ctas, float2* part, int* err, cudaStream_t st);

}  // namespace wotg
