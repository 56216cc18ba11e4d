// wotg_common.cuh — shared device helpers of libwotg (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/wotg.h"

namespace wotg {

constexpr double kLog2e = 1.4426950408889634074;
constexpr double kLn2 = 0.69314718055994530942;
// Finite stand-in for -inf in running maxima, so that (m - m_new) never
// evaluates to (-inf) - (-inf).
constexpr float kNegBig = -1.0e30f;

// Records the text of the last failing CUDA call (host side, per process).
void set_last_error(const char* what, cudaError_t err);
// Records a plain message as the last error text.
void set_last_message(const char* msg);

#define WOTG_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) {                              \
      ::wotg::set_last_error(#call, e_);                  \
      return WOTG_CUDA_ERROR;                             \
    }                                                     \
  } while (0)

// Host-side count of kernels this library launched (wotg_launch_count).
void count_launch();

#define WOTG_LAUNCHED()                                   \
  do {                                                    \
    ::wotg::count_launch();                               \
    cudaError_t e_ = cudaGetLastError();                  \
    if (e_ != cudaSuccess) {                              \
      ::wotg::set_last_error("kernel launch", e_);        \
      return WOTG_CUDA_ERROR;                             \
    }                                                     \
  } while (0)

// 2^x on the SFU (PTX ex2.approx, flush-to-zero); max relative error ~2 ulp.
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Streaming 128-bit load that is not kept in L1 (each cost element is read
// once per pass; the matrix is far larger than L2).
__device__ __forceinline__ float4 ld_stream(const float4* p) { return __ldcs(p); }

// Merge two base-2 log-sum-exp partials (m, s): value = s * 2^m.
__device__ __forceinline__ void lse_merge(float& m, float& s, float m2, float s2) {
  float mn = fmaxf(m, m2);
  s = s * ex2(m - mn) + s2 * ex2(m2 - mn);
  m = mn;
}

__device__ __forceinline__ void warp_lse(float& m, float& s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float m2 = __shfl_xor_sync(0xffffffffu, m, o);
    float s2 = __shfl_xor_sync(0xffffffffu, s, o);
    lse_merge(m, s, m2, s2);
  }
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ double warp_maxd(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Max of non-negative doubles through their bit patterns (monotone for x >= 0).
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* slot, double x) {
  if (x > 0.0) atomicMax(slot, (unsigned long long)__double_as_longlong(x));
}

struct Bump {
  char* base;
  size_t off;
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += n * sizeof(T);
    return p;
  }
};

int sm_count();

}  // namespace wotg
