// wotg_diag.cu — measured exp2 throughput of this GPU (diagnostic; no counterpart
// in the reference). The half-steps of every form spend one ex2.approx.ftz per
// cost element, so their ceiling is this rate, which no vendor table gives; the
// bench quotes the on-the-fly and batched kernels against it.
#include "wotg_common.cuh"

namespace wotg {
namespace {

__device__ float g_exp2_sink;

// Four independent accumulation chains per thread, one ex2 and one add per element.
__global__ void __launch_bounds__(256) exp2_rate_kernel(int n) {
  float x = -3.0f + 1e-6f * (float)threadIdx.x, a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  for (int i = 0; i < n; ++i) {
    a0 += ex2(x);
    a1 += ex2(x + 1.f);
    a2 += ex2(x + 2.f);
    a3 += ex2(x + 3.f);
    x -= 1e-3f;
  }
  const float s = (a0 + a1) + (a2 + a3);
  if (s == 1234.5f) g_exp2_sink = s;  // keeps the loop live
}

}  // namespace
}  // namespace wotg

using namespace wotg;

extern "C" int wotg_exp2_rate(double* exp2_per_s, void* stream) {
  if (!exp2_per_s) return WOTG_BADARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = sm_count() * 8, n = 4096;
  cudaEvent_t e0, e1;
  WOTG_CUDA(cudaEventCreate(&e0));
  WOTG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, st);
    exp2_rate_kernel<<<blocks, 256, 0, st>>>(n);
    count_launch();
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      set_last_error("exp2 rate", e);
      return WOTG_CUDA_ERROR;
    }
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *exp2_per_s = (double)blocks * 256.0 * n * 4.0 / (best * 1e-3);
  return WOTG_OK;
}

namespace wotg {
namespace {

__global__ void exp2_fma_kernel(const float* __restrict__ z, float* __restrict__ out, int64_t n) {
  const int64_t i = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (i + 1 < n) {
    const float2 r = ex2_fma2(make_float2(z[i], z[i + 1]));
    out[i] = r.x;
    out[i + 1] = r.y;
  } else if (i < n) {
    out[i] = ex2_fma2(make_float2(z[i], 0.f)).x;
  }
}

}  // namespace
}  // namespace wotg

extern "C" int wotg_exp2_fma(const float* z, float* out, int64_t n, void* stream) {
  if (!z || !out || n <= 0) return WOTG_BADARG;
  const int64_t pairs = (n + 1) / 2;
  const int64_t blocks = (pairs + 255) / 256;
  if (blocks > 2147483647LL) return WOTG_BADARG;
  wotg::exp2_fma_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(z, out, n);
  WOTG_LAUNCHED();
  return WOTG_OK;
}
