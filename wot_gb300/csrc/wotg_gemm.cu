// wotg_gemm.cu — dense FP64 product for chaining transport maps (sm_103a).
//
// The long-range coupling of the reference is the matrix product of
// consecutive dense maps (wot/tmap/util.py:74-94, np.dot of tmap_0.X with the
// rows of tmap_1.X that tmap_0's columns name; chained by
// wot/tmap/chaining.py:4-40). Here: C (M x N) = A (M x K) . B[rows] (K x N),
// row-major FP64, the rows of B gathered by an optional index.
//
// FP64 runs at 1/64 of the FP32 rate on this part, so the product is bound by
// the FP64 FMA pipe, not by memory: each CTA computes a 64 x 64 tile of C from
// 64 x 16 and 16 x 64 tiles of A and B staged in shared memory (double
// buffered), every thread a 4 x 4 block of C in registers, i.e. 16 FMAs per 8
// shared-memory loads.
#include <algorithm>

#include "wotg_common.cuh"

namespace wotg {

constexpr int kGemmTile = 64;
constexpr int kGemmK = 16;
constexpr int kGemmThreads = 256;

__global__ void __launch_bounds__(kGemmThreads) gemm_f64_kernel(const double* __restrict__ A, int64_t lda,
                                                                const double* __restrict__ B, int64_t ldb,
                                                                const int64_t* __restrict__ b_rows,
                                                                double* __restrict__ C, int64_t ldc, int64_t M,
                                                                int64_t N, int64_t K) {
  __shared__ double sA[2][kGemmK][kGemmTile + 1];   // A tile transposed: [k][m], padded against bank conflicts
  __shared__ double sB[2][kGemmK][kGemmTile];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;           // thread (ty, tx) owns rows 4 ty.., columns 4 tx..
  const int64_t m0 = (int64_t)blockIdx.y * kGemmTile, n0 = (int64_t)blockIdx.x * kGemmTile;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  // loads of one K-chunk: A is 64 x 16 (4 per thread), B is 16 x 64 (4 per thread)
  auto load = [&](int buf, int64_t k0) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int idx = tid + t * kGemmThreads;       // 0 .. 1023
      const int am = idx >> 4, ak = idx & 15;       // A: row am, column ak
      const int64_t gm = m0 + am, gk = k0 + ak;
      sA[buf][ak][am] = (gm < M && gk < K) ? A[gm * lda + gk] : 0.0;
      const int bk = idx >> 6, bn = idx & 63;       // B: row bk, column bn
      const int64_t gk2 = k0 + bk, gn = n0 + bn;
      double v = 0.0;
      if (gk2 < K && gn < N) {
        const int64_t r = b_rows ? b_rows[gk2] : gk2;
        v = B[r * ldb + gn];
      }
      sB[buf][bk][bn] = v;
    }
  };

  const int64_t nk = (K + kGemmK - 1) / kGemmK;
  load(0, 0);
  __syncthreads();
  for (int64_t c = 0; c < nk; ++c) {
    const int buf = (int)(c & 1);
    if (c + 1 < nk) load(buf ^ 1, (c + 1) * kGemmK);
#pragma unroll
    for (int k = 0; k < kGemmK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) a[t] = sA[buf][k][ty * 4 + t];
#pragma unroll
      for (int t = 0; t < 4; ++t) b[t] = sB[buf][k][tx * 4 + t];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gn = n0 + tx * 4 + j;
      if (gn < N) C[gm * ldc + gn] = acc[i][j];
    }
  }
}

}  // namespace wotg

using namespace wotg;

extern "C" int wotg_gemm_f64(const double* A, int64_t lda, const double* B, int64_t ldb, const int64_t* b_rows,
                             double* C, int64_t ldc, int64_t M, int64_t N, int64_t K, void* stream) {
  if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || lda < K || ldb < N || ldc < N) return WOTG_BADARG;
  const int64_t gx = (N + kGemmTile - 1) / kGemmTile, gy = (M + kGemmTile - 1) / kGemmTile;
  if (gx > 2147483647LL || gy > 65535) return WOTG_BADARG;
  gemm_f64_kernel<<<dim3((unsigned)gx, (unsigned)gy), kGemmThreads, 0, (cudaStream_t)stream>>>(
      A, lda, B, ldb, b_rows, C, ldc, M, N, K);
  WOTG_LAUNCHED();
  return WOTG_OK;
}
