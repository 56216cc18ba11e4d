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
int tc_lse_launch(const __half* Pt, int n_ptiles, const __half* Qt, int nqt, const float* bias, int kp,
                  float gamma, int nsplit, float2* part, int64_t n_pad, int* err, cudaStream_t st);

}  // namespace wotg
