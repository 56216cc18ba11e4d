// wotg_common.cuh — shared device helpers of libwotg (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include <utility>

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
// n kernels launched by one replay of a captured graph; the count so far.
void count_launches(unsigned long long n);
unsigned long long launches_so_far();

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

// 2^z of a pair on the FMA pipe (the tensor-core epilogue computes a share of
// its exponentials here, beside the SFU): Cody-Waite style reduction
// z = n + f with n = rint(z) (the 1.5 * 2^23 shift), f in [-1/2, 1/2]; 2^f by
// the degree-5 relative-error minimax polynomial on [-1/2, 1/2] (Remez
// exchange, max 7.5e-8; its FP32 Horner evaluation 2.2e-7 of 2^z); 2^n from
// the exponent bits. z is clamped to [-125, 126] with NaN kept, so 2^n stays a
// normal number and a NaN exponent gives NaN.
__device__ __forceinline__ float2 ex2_fma2(float2 z) {
  float zx, zy;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(zx) : "f"(z.x), "f"(126.f));
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(zy) : "f"(z.y), "f"(126.f));
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(zx) : "f"(zx), "f"(-125.f));
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(zy) : "f"(zy), "f"(-125.f));
  const float2 zz = make_float2(zx, zy);
  const float2 t = __fadd2_rn(zz, make_float2(12582912.f, 12582912.f));        // 1.5 * 2^23 + n
  const float2 n = __fadd2_rn(t, make_float2(-12582912.f, -12582912.f));
  const float2 f = __fadd2_rn(zz, make_float2(-n.x, -n.y));                     // exact
  float2 p = make_float2(1.3276472e-3f, 1.3276472e-3f);
  p = __ffma2_rn(p, f, make_float2(9.675541e-3f, 9.675541e-3f));
  p = __ffma2_rn(p, f, make_float2(5.550713e-2f, 5.550713e-2f));
  p = __ffma2_rn(p, f, make_float2(0.2402212f, 0.2402212f));
  p = __ffma2_rn(p, f, make_float2(0.69314694f, 0.69314694f));
  p = __ffma2_rn(p, f, make_float2(1.0000001f, 1.0000001f));
  // low bits of t hold n (two's complement): (t << 23) + (127 << 23) = the bits of 2^n
  const float2 sc = make_float2(__int_as_float((__float_as_int(t.x) << 23) + (127 << 23)),
                                __int_as_float((__float_as_int(t.y) << 23) + (127 << 23)));
  return __fmul2_rn(p, sc);
}

// L2 = o + log2(s) for an FP32 sum s = m 2^e: the exponent exactly, the FP32
// log2 of the mantissa taken in [1/sqrt 2, sqrt 2), so that for s near 1 (the
// speculative half-steps, whose sums are relative to the previous log-sum-exp)
// log2 m is small and its 1-ulp error negligible, and at most 3e-8 elsewhere
// (below the FP32 sum's own rounding); no FP64 transcendental (slow on this
// part). s = 0 gives -inf.
__device__ __forceinline__ double lse2(float o, float s) {
  int e;
  float m = frexpf(s, &e);
  if (m < 0.70710678f) {
    m *= 2.f;
    e -= 1;
  }
  return (double)o + (double)e + (double)log2f(m);
}

// Programmatic dependent launch. A kernel launched with launch_dependent()
// may be scheduled while the kernel before it in the stream still runs: it
// calls pdl_wait() before touching any global memory (the wait returns once
// that kernel has completed and its writes are visible; without the launch
// attribute it returns at once), then pdl_trigger() to let the next dependent
// launch be scheduled in turn.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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

// Merge of base-2 partials (m, s) in FP64 across a warp: every lane ends with
// the warp's total as (m, S), value S 2^m (S in FP64).
__device__ __forceinline__ void warp_lse_f64(float& m, double& S) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
    const double S2 = __shfl_xor_sync(0xffffffffu, S, o);
    const float mn = fmaxf(m, m2);
    // the scale factors by the FP32 ex2 (2 ulp), the sums themselves in FP64
    S = S * (double)ex2(m - mn) + S2 * (double)ex2(m2 - mn);
    m = mn;
  }
}

// Compensated (Kahan) accumulation of v into (s, c): s - c carries the sum of
// many FP32 terms with one rounding's error instead of one per term.
// (Written with the _rn intrinsics so that no step is contracted into an FMA.)
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
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

// ---------------------------------------------------------------------------
// Precision of the streamed half-steps. The exponent of element (i, j) of a row
// pass is w_j - kappa2 C_ij (base 2), whose terms are tens to hundreds while
// the entries that carry mass have exponents within a few units of the row's
// log-sum-exp. Rounding the weight or the exponent to FP32 at that magnitude
// (|x| 2^-24) would put an error of ~1e-6 (1e-5 at eps = 0.01) on every entry,
// which the iterations carry into the potentials. Instead:
//  * a weight w (FP64) is kept as hi + lo: hi on a 2^-14 grid (exact in FP32
//    for |w| < 512), lo the FP32 remainder;
//  * each row (column) is summed relative to an offset o on the same grid, the
//    previous half-step's log-sum-exp of that row, so that hi - o is exact;
//  * kappa2 is split into hi + lo (Coef) and the exponent is
//        x = fma(-k2hi, C, hi - o) + fma(-k2lo, C, lo),
//    small for the entries that matter, rounded once; o is added back in FP64.
// What remains is the FP32 storage of C itself.
// ---------------------------------------------------------------------------
constexpr double kWeightGrid = 16384.0;  // 2^14

__device__ __forceinline__ void split_weight(double w, float* hi, float* lo, int64_t k) {
  if (!(fabs(w) < 1e30)) {  // -inf (zero weight), +inf, NaN: carried by hi alone
    hi[k] = (float)w;
    lo[k] = 0.f;
    return;
  }
  const float h = (float)(rint(w * kWeightGrid) / kWeightGrid);
  hi[k] = h;
  lo[k] = (float)(w - (double)h);
}

// x on the weight grid; 0 when x is not finite.
__device__ __forceinline__ float grid_value(double x) {
  return fabs(x) < 1e30 ? (float)(rint(x * kWeightGrid) / kWeightGrid) : 0.f;
}
// Base-2 grid offset of a row whose previous log-sum-exp (natural log) is L;
// 0 when L is not finite.
__device__ __forceinline__ float grid_offset(double L) { return grid_value(L * kLog2e); }

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

// Launch with programmatic stream serialisation (see pdl_wait): the launch's
// latency and the kernel's prologue overlap the tail of the previous kernel.
template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                             Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace wotg
