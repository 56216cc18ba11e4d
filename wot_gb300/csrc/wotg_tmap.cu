// wotg_tmap.cu — population transport through dense FP64 couplings (sm_103a).
//
// Replaces the NumPy products of the reference's TransportMapModel:
//   push_forward: p = p @ tmap.X                 wot/tmap/transport_map_model.py:290
//   pull_back:    p = (tmap.X @ p.T).T           wot/tmap/transport_map_model.py:356
// plus the optional row normalisation p = (p.T / p.sum(axis=1)).T (:291-292, :357-358).
// Accumulation is FP64 like the reference (k populations at a time, k <= 16 per
// pass); X is read once per pass with coalesced loads.
#include <algorithm>

#include "wotg_common.cuh"

namespace wotg {

constexpr int kMaxK = 16;

// out[r][i] = sum_j X[i][j] P[r][j]; one warp per row i of X.
template <int KC>
__global__ void __launch_bounds__(256) pull_kernel(const double* __restrict__ X, int64_t I, int64_t J,
                                                   const double* __restrict__ P, int k0, int k,
                                                   double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < I; i += nwarps) {
    double acc[KC];
#pragma unroll
    for (int r = 0; r < KC; ++r) acc[r] = 0.0;
    const double* row = X + i * J;
    for (int64_t j = lane; j < J; j += 32) {
      const double x = row[j];
#pragma unroll
      for (int r = 0; r < KC; ++r)
        if (k0 + r < k) acc[r] = fma(x, __ldg(P + (int64_t)(k0 + r) * J + j), acc[r]);
    }
#pragma unroll
    for (int r = 0; r < KC; ++r) {
      const double t = warp_sum(acc[r]);
      if (lane == 0 && k0 + r < k) out[(int64_t)(k0 + r) * I + i] = t;
    }
  }
}

// out[r][j] += sum_{i in block rows} P[r][i] X[i][j]; thread per column, grid.y
// splits the rows, FP64 atomics merge the row blocks.
template <int KC>
__global__ void __launch_bounds__(256) push_kernel(const double* __restrict__ X, int64_t I, int64_t J,
                                                   const double* __restrict__ P, int k0, int k,
                                                   int64_t rows_per, double* __restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per;
  const int64_t r1 = min(I, r0 + rows_per);
  if (j >= J) return;
  double acc[KC];
#pragma unroll
  for (int r = 0; r < KC; ++r) acc[r] = 0.0;
  for (int64_t i = r0; i < r1; ++i) {
    const double x = X[i * J + j];
#pragma unroll
    for (int r = 0; r < KC; ++r)
      if (k0 + r < k) acc[r] = fma(__ldg(P + (int64_t)(k0 + r) * I + i), x, acc[r]);
  }
#pragma unroll
  for (int r = 0; r < KC; ++r)
    if (k0 + r < k) atomicAdd(out + (int64_t)(k0 + r) * J + j, acc[r]);
}

// Divide each of the k rows (length n) by its sum; one CTA per row.
__global__ void normalize_rows_kernel(double* __restrict__ out, int64_t n) {
  __shared__ double sh[32];
  double* row = out + (int64_t)blockIdx.x * n;
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) s += row[t];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) sh[0] = t;
  }
  __syncthreads();
  const double total = sh[0];
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) row[t] = row[t] / total;
}

}  // namespace wotg

using namespace wotg;

extern "C" int wotg_apply_coupling_f64(const double* X, int64_t I, int64_t J, const double* P, int32_t k,
                                       int32_t transpose, int32_t normalize, double* out, void* stream) {
  if (!X || !P || !out || I <= 0 || J <= 0 || k <= 0) return WOTG_BADARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  if (transpose) {
    const int grid = (int)std::min<int64_t>((I + 7) / 8, (int64_t)sms * 8);
    for (int k0 = 0; k0 < k; k0 += kMaxK) {
      pull_kernel<kMaxK><<<grid, 256, 0, st>>>(X, I, J, P, k0, k, out);
      WOTG_LAUNCHED();
    }
    if (normalize) {
      normalize_rows_kernel<<<k, 256, 0, st>>>(out, I);
      WOTG_LAUNCHED();
    }
  } else {
    WOTG_CUDA(cudaMemsetAsync(out, 0, (size_t)k * J * sizeof(double), st));
    const int64_t ncb = (J + 255) / 256;
    int64_t nrb = std::max<int64_t>(1, ((int64_t)sms * 8) / ncb);
    nrb = std::min<int64_t>(nrb, std::max<int64_t>(1, I / 16));
    nrb = std::min<int64_t>(nrb, 65535);
    const int64_t rows_per = (I + nrb - 1) / nrb;
    nrb = (I + rows_per - 1) / rows_per;
    for (int k0 = 0; k0 < k; k0 += kMaxK) {
      push_kernel<kMaxK><<<dim3((unsigned)ncb, (unsigned)nrb), 256, 0, st>>>(X, I, J, P, k0, k, rows_per, out);
      WOTG_LAUNCHED();
    }
    if (normalize) {
      normalize_rows_kernel<<<k, 256, 0, st>>>(out, J);
      WOTG_LAUNCHED();
    }
  }
  return WOTG_OK;
}
