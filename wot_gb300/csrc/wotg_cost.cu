// wotg_cost.cu — cost matrix construction and its exact median (sm_103a).
//
// Replaces, on the device:
//   sklearn pairwise_distances(a, b, metric='sqeuclidean')   wot/ot/ot_model.py:249-251
//   cost_matrix / np.median(cost_matrix)                     wot/ot/ot_model.py:252
//   np.asarray(C, dtype=np.float64) for user costs           wot/ot/optimal_transport.py:100
//
// The cost is written once per day pair and then streamed by every Sinkhorn
// half-step, so it is stored FP32 (the FP32 rounding of C is the accuracy floor
// of the whole path; see the solver file). The squared distance is summed as
// sum_k (x_k - y_k)^2, which has no cancellation, instead of the
// |x|^2 - 2x.y + |y|^2 expansion the reference evaluates in FP64.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "wotg_common.cuh"

namespace wotg {

static char g_last_error[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

void set_last_error(const char* what, cudaError_t err) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(err));
}

void set_last_message(const char* msg) { snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
  return n > 0 ? n : 148;
}

// ---------------------------------------------------------------------------
// Squared-Euclidean cost. CTA tile: 64 rows x 128 columns, 256 threads as
// 8 (row groups of 8) x 32 (column groups of 4); coordinates staged through
// shared memory transposed, 32 dimensions at a time.
// ---------------------------------------------------------------------------
constexpr int kCostRows = 64;
constexpr int kCostCols = 128;
constexpr int kCostK = 32;

__global__ void __launch_bounds__(256) cost_sqeuclidean_kernel(
    const float* __restrict__ X, int64_t I, int64_t ldx, const float* __restrict__ Y, int64_t J,
    int64_t ldy, int d, float* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) float xs[kCostK * kCostRows];
  __shared__ __align__(16) float ys[kCostK * kCostCols];
  const int tid = threadIdx.x;
  const int tx = tid & 31;
  const int ty = tid >> 5;
  const int64_t i0 = (int64_t)blockIdx.y * kCostRows;
  const int64_t j0 = (int64_t)blockIdx.x * kCostCols;
  float acc[8][4];
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;

  for (int k0 = 0; k0 < d; k0 += kCostK) {
    const int kc = min(kCostK, d - k0);
    __syncthreads();
    for (int idx = tid; idx < kCostK * kCostRows; idx += 256) {
      const int r = idx / kCostK, k = idx % kCostK;
      const int64_t i = i0 + r;
      xs[k * kCostRows + r] = (k < kc && i < I) ? X[i * ldx + k0 + k] : 0.f;
    }
    for (int idx = tid; idx < kCostK * kCostCols; idx += 256) {
      const int c = idx / kCostK, k = idx % kCostK;
      const int64_t j = j0 + c;
      ys[k * kCostCols + c] = (k < kc && j < J) ? Y[j * ldy + k0 + k] : 0.f;
    }
    __syncthreads();
    for (int k = 0; k < kc; ++k) {
      const float4 xa = *reinterpret_cast<const float4*>(&xs[k * kCostRows + ty * 8]);
      const float4 xb = *reinterpret_cast<const float4*>(&xs[k * kCostRows + ty * 8 + 4]);
      const float4 yv = *reinterpret_cast<const float4*>(&ys[k * kCostCols + tx * 4]);
      const float xr[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
      const float yc[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float t = xr[r] - yc[c];
          acc[r][c] = fmaf(t, t, acc[r][c]);
        }
    }
  }
  const int64_t jc = j0 + tx * 4;
  if (jc >= ldc) return;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int64_t i = i0 + ty * 8 + r;
    if (i >= I) break;
    float4 o;
    o.x = (jc + 0 < J) ? acc[r][0] : INFINITY;
    o.y = (jc + 1 < J) ? acc[r][1] : INFINITY;
    o.z = (jc + 2 < J) ? acc[r][2] : INFINITY;
    o.w = (jc + 3 < J) ? acc[r][3] : INFINITY;
    *reinterpret_cast<float4*>(C + i * ldc + jc) = o;
  }
}

__global__ void cost_from_f64_kernel(const double* __restrict__ C64, int64_t I, int64_t J,
                                     float* __restrict__ C, int64_t ldc) {
  const int64_t nv = ldc >> 2;
  for (int64_t i = blockIdx.y; i < I; i += gridDim.y) {
    for (int64_t c4 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c4 < nv;
         c4 += (int64_t)gridDim.x * blockDim.x) {
      const int64_t j = c4 * 4;
      float4 o;
      o.x = (j + 0 < J) ? (float)C64[i * J + j + 0] : INFINITY;
      o.y = (j + 1 < J) ? (float)C64[i * J + j + 1] : INFINITY;
      o.z = (j + 2 < J) ? (float)C64[i * J + j + 2] : INFINITY;
      o.w = (j + 3 < J) ? (float)C64[i * J + j + 3] : INFINITY;
      *reinterpret_cast<float4*>(C + i * ldc + j) = o;
    }
  }
}

// ---------------------------------------------------------------------------
// Exact order statistics of the FP32 costs by radix select on the bit
// patterns (non-negative floats order like their unsigned bits): three
// histogram passes over bits 31..20, 19..8 and 7..0 of the keys that share the
// prefix found so far.
// ---------------------------------------------------------------------------
constexpr int kHistBins = 4096;

__global__ void __launch_bounds__(512) radix_hist_kernel(const float* __restrict__ C, int64_t I,
                                                         int64_t J, int64_t ldc, uint32_t prefix,
                                                         uint32_t pmask, int shift, uint32_t bmask,
                                                         unsigned long long* __restrict__ ghist) {
  __shared__ unsigned int h[kHistBins];
  for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const int64_t nv = ldc >> 2;
  for (int64_t i = blockIdx.x; i < I; i += gridDim.x) {
    const float4* row = reinterpret_cast<const float4*>(C + i * ldc);
    for (int64_t c4 = threadIdx.x; c4 < nv; c4 += blockDim.x) {
      const float4 v = ld_stream(row + c4);
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (c4 * 4 + t < J) {
          const uint32_t key = __float_as_uint(vv[t]);
          if ((key & pmask) == prefix) atomicAdd(&h[(key >> shift) & bmask], 1u);
        }
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kHistBins; b += blockDim.x)
    if (h[b]) atomicAdd(&ghist[b], (unsigned long long)h[b]);
}

}  // namespace wotg

using namespace wotg;

extern "C" {

const char* wotg_version(void) { return "wotg 0.1 (sm_103a)"; }
const char* wotg_last_error(void) { return g_last_error; }
unsigned long long wotg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int wotg_cost_sqeuclidean(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J,
                          int64_t ldy, int32_t d, float* C, int64_t ldc, void* stream) {
  if (I <= 0 || J <= 0 || d <= 0 || ldc < J || (ldc & 3) || ldx < d || ldy < d || !X || !Y || !C)
    return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(C) & 15) != 0) return WOTG_BADARG;
  dim3 grid((unsigned)((ldc + kCostCols - 1) / kCostCols), (unsigned)((I + kCostRows - 1) / kCostRows));
  if (grid.y > 65535u) {
    // Launch in row slabs so that gridDim.y stays within limits.
    const int64_t slab = (int64_t)65535 * kCostRows;
    for (int64_t r0 = 0; r0 < I; r0 += slab) {
      const int64_t rows = std::min(slab, I - r0);
      dim3 g(grid.x, (unsigned)((rows + kCostRows - 1) / kCostRows));
      cost_sqeuclidean_kernel<<<g, 256, 0, (cudaStream_t)stream>>>(X + r0 * ldx, rows, ldx, Y, J, ldy,
                                                                   d, C + r0 * ldc, ldc);
      WOTG_LAUNCHED();
    }
    return WOTG_OK;
  }
  cost_sqeuclidean_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(X, I, ldx, Y, J, ldy, d, C, ldc);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

int wotg_cost_from_f64(const double* C64, int64_t I, int64_t J, float* C, int64_t ldc, void* stream) {
  if (I <= 0 || J <= 0 || ldc < J || (ldc & 3) || !C64 || !C) return WOTG_BADARG;
  if ((reinterpret_cast<uintptr_t>(C) & 15) != 0) return WOTG_BADARG;
  const int64_t nv = ldc >> 2;
  dim3 grid((unsigned)std::min<int64_t>((nv + 255) / 256, 64), (unsigned)std::min<int64_t>(I, 65535));
  cost_from_f64_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(C64, I, J, C, ldc);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

size_t wotg_median_workspace_bytes(void) { return kHistBins * sizeof(unsigned long long); }

}  // extern "C"

namespace {

struct RadixSelector {
  const float* C;
  int64_t I, J, ldc;
  unsigned long long* dhist;
  cudaStream_t stream;
  int grid;
  struct Level {
    uint32_t prefix, pmask;
    int shift;
    std::vector<unsigned long long> hist;
  };
  std::vector<Level> cache;

  int histogram(uint32_t prefix, uint32_t pmask, int shift, uint32_t bmask,
                const std::vector<unsigned long long>** out) {
    for (auto& l : cache)
      if (l.prefix == prefix && l.pmask == pmask && l.shift == shift) {
        *out = &l.hist;
        return WOTG_OK;
      }
    WOTG_CUDA(cudaMemsetAsync(dhist, 0, kHistBins * sizeof(unsigned long long), stream));
    radix_hist_kernel<<<grid, 512, 0, stream>>>(C, I, J, ldc, prefix, pmask, shift, bmask, dhist);
    WOTG_LAUNCHED();
    Level l{prefix, pmask, shift, std::vector<unsigned long long>(kHistBins)};
    WOTG_CUDA(cudaMemcpyAsync(l.hist.data(), dhist, kHistBins * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, stream));
    WOTG_CUDA(cudaStreamSynchronize(stream));
    cache.push_back(std::move(l));
    *out = &cache.back().hist;
    return WOTG_OK;
  }

  // k-th smallest (0-based) valid key.
  int select(unsigned long long k, uint32_t* key_out) {
    uint32_t prefix = 0, pmask = 0;
    const int shifts[3] = {20, 8, 0};
    const uint32_t bmasks[3] = {0xFFFu, 0xFFFu, 0xFFu};
    const uint32_t pmasks[3] = {0xFFF00000u, 0xFFFFFF00u, 0xFFFFFFFFu};
    for (int lvl = 0; lvl < 3; ++lvl) {
      const std::vector<unsigned long long>* h = nullptr;
      int st = histogram(prefix, pmask, shifts[lvl], bmasks[lvl], &h);
      if (st != WOTG_OK) return st;
      unsigned long long cum = 0;
      int bin = -1;
      for (int b = 0; b <= (int)bmasks[lvl]; ++b) {
        if (cum + (*h)[b] > k) {
          bin = b;
          break;
        }
        cum += (*h)[b];
      }
      if (bin < 0) return WOTG_BADARG;
      k -= cum;
      prefix |= (uint32_t)bin << shifts[lvl];
      pmask = pmasks[lvl];
    }
    *key_out = prefix;
    return WOTG_OK;
  }
};

}  // namespace

extern "C" int wotg_median(const float* C, int64_t I, int64_t J, int64_t ldc, double* median_out,
                           void* workspace, size_t workspace_bytes, void* stream) {
  if (I <= 0 || J <= 0 || ldc < J || (ldc & 3) || !C || !median_out) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_median_workspace_bytes()) return WOTG_WORKSPACE;
  RadixSelector sel{C, I, J, ldc, reinterpret_cast<unsigned long long*>(workspace),
                    (cudaStream_t)stream, (int)std::min<int64_t>(I, (int64_t)sm_count() * 4), {}};
  const unsigned long long n = (unsigned long long)I * (unsigned long long)J;
  const unsigned long long klo = (n - 1) / 2, khi = n / 2;
  uint32_t key_lo = 0, key_hi = 0;
  int st = sel.select(klo, &key_lo);
  if (st != WOTG_OK) return st;
  key_hi = key_lo;
  if (khi != klo) {
    st = sel.select(khi, &key_hi);
    if (st != WOTG_OK) return st;
  }
  float flo, fhi;
  std::memcpy(&flo, &key_lo, 4);
  std::memcpy(&fhi, &key_hi, 4);
  *median_out = ((double)flo + (double)fhi) / 2.0;
  return WOTG_OK;
}
