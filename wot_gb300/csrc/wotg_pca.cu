// wotg_pca.cu — the products of the local PCA on the device (sm_103a).
//
// The reference's local PCA (wot/ot/util.py:240-255) fits scikit-learn's PCA on
// the double-centred genes x cells matrix of a day pair; scikit-learn's
// randomized solver then multiplies that matrix and its transpose with thin
// blocks of vectors (range finder with power iterations) and orthonormalises
// the blocks. The expression matrix is mostly zeros (log1p of counts), so the
// products run on its sparse form, with the two centrings applied as rank-one
// corrections in the products' epilogue (never forming the dense centred
// matrix):
//   * wotg_csr_count / wotg_csr_fill: CSR of a dense FP64 row-major matrix (row
//     sums as a by-product), columns in ascending order per row;
//   * wotg_csr_transpose: the CSR of its transpose by a stable counting sort
//     (per-block column counts, fixed-order offsets), so that every product's
//     summation order, and the result, is the same from run to run;
//   * wotg_spmm_centred: Y = X Q - 1 a^T - c b^T for a CSR X and a thin dense Q
//     (r <= 64 columns), a warp per row, FP64;
//   * wotg_gram_f64: G = A^T A of a thin dense block (r <= 64), per-block
//     partial Gram matrices summed in a fixed order (the Cholesky QR of the
//     range finder factorises the r x r result).
#include <algorithm>

#include "wotg_common.cuh"

namespace wotg {

constexpr int kPcaThreads = 256;
constexpr int kPcaMaxR = 64;

// nnz and sum of each row (a warp per row).
__global__ void csr_count_kernel(const double* __restrict__ X, int64_t n, int64_t p, int64_t ldx,
                                 int64_t* __restrict__ cnt, double* __restrict__ rowsum) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    int64_t c = 0;
    double s = 0.0;
    for (int64_t j = lane; j < p; j += 32) {
      const double v = X[i * ldx + j];
      c += v != 0.0;
      s += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, o);
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
      cnt[i] = c;
      if (rowsum) rowsum[i] = s;
    }
  }
}

// Exclusive prefix sum of cnt[0..n) into out[0..n] (out[n] = total), one block
// of 1024 threads, each scanning a contiguous chunk (in place allowed: out == cnt).
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(const int64_t* cnt, int64_t n, int64_t* out) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (n + 1023) / 1024;
  const int64_t b = (int64_t)t * chunk, e = min(n, b + chunk);
  int64_t s = 0;
  for (int64_t k = b; k < e; ++k) s += cnt[k];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int64_t v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int64_t run = part[t] - s;  // exclusive prefix of this chunk
  for (int64_t k = b; k < e; ++k) {
    const int64_t c = cnt[k];
    out[k] = run;
    run += c;
  }
  if (t == 1023) out[n] = part[1023];
}

// Column indices and values of each row in ascending column order (a warp per row).
__global__ void csr_fill_kernel(const double* __restrict__ X, int64_t n, int64_t p, int64_t ldx,
                                const int64_t* __restrict__ rowptr, int32_t* __restrict__ colidx,
                                double* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    int64_t pos = rowptr[i];
    for (int64_t j0 = 0; j0 < p; j0 += 32) {
      const int64_t j = j0 + lane;
      const double v = j < p ? X[i * ldx + j] : 0.0;
      const unsigned nz = __ballot_sync(0xffffffffu, v != 0.0);
      if (v != 0.0) {
        const int64_t k = pos + __popc(nz & below);
        colidx[k] = (int32_t)j;
        vals[k] = v;
      }
      pos += __popc(nz);
    }
  }
}

// Stable transpose, step 1: per-block column counts of rows [b * rpb, (b + 1) * rpb).
__global__ void __launch_bounds__(kPcaThreads) csr_tcount_kernel(const int64_t* __restrict__ rowptr,
                                                                 const int32_t* __restrict__ colidx, int64_t n,
                                                                 int64_t p, int64_t rpb,
                                                                 int32_t* __restrict__ cntb) {
  extern __shared__ int32_t hist[];
  for (int64_t j = threadIdx.x; j < p; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  const int64_t r0 = (int64_t)blockIdx.x * rpb, r1 = min(n, r0 + rpb);
  for (int64_t k = rowptr[r0] + threadIdx.x; k < rowptr[r1]; k += blockDim.x) atomicAdd(&hist[colidx[k]], 1);
  __syncthreads();
  for (int64_t j = threadIdx.x; j < p; j += blockDim.x) cntb[(int64_t)blockIdx.x * p + j] = hist[j];
}

// Step 2: column totals (a thread per column, blocks summed in order).
__global__ void csr_ttotal_kernel(const int32_t* __restrict__ cntb, int64_t nb, int64_t p,
                                  int64_t* __restrict__ total) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p) return;
  int64_t s = 0;
  for (int64_t b = 0; b < nb; ++b) s += cntb[b * p + j];
  total[j] = s;
}

// Step 3: each block's first slot in each column (after the column start).
__global__ void csr_toffset_kernel(int32_t* __restrict__ cntb, int64_t nb, int64_t p,
                                   const int64_t* __restrict__ t_rowptr) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p) return;
  int64_t run = t_rowptr[j];
  for (int64_t b = 0; b < nb; ++b) {
    const int32_t c = cntb[b * p + j];
    cntb[b * p + j] = (int32_t)(run - t_rowptr[j]);   // offset within the column
    run += c;
  }
}

// Step 4: a block writes its rows one after another, so that each column's
// entries stay in row order; within a row the columns are distinct.
__global__ void __launch_bounds__(kPcaThreads) csr_tfill_kernel(const int64_t* __restrict__ rowptr,
                                                                const int32_t* __restrict__ colidx,
                                                                const double* __restrict__ vals, int64_t n,
                                                                int64_t p, int64_t rpb,
                                                                const int32_t* __restrict__ cntb,
                                                                const int64_t* __restrict__ t_rowptr,
                                                                int32_t* __restrict__ t_colidx,
                                                                double* __restrict__ t_vals) {
  extern __shared__ int32_t next[];
  for (int64_t j = threadIdx.x; j < p; j += blockDim.x) next[j] = cntb[(int64_t)blockIdx.x * p + j];
  __syncthreads();
  const int64_t r0 = (int64_t)blockIdx.x * rpb, r1 = min(n, r0 + rpb);
  for (int64_t i = r0; i < r1; ++i) {
    for (int64_t k = rowptr[i] + threadIdx.x; k < rowptr[i + 1]; k += blockDim.x) {
      const int32_t j = colidx[k];
      const int64_t dst = t_rowptr[j] + next[j];
      t_colidx[dst] = (int32_t)i;
      t_vals[dst] = vals[k];
      next[j] += 1;
    }
    __syncthreads();
  }
}

// Y (n x r) = X Q - 1 a^T - c b^T (a, b: r; c: n; any may be NULL). A group of
// G warps per row of the CSR X (G = 1 for short rows, 8 for the thousands of
// entries of a gene's row in the transpose): warp w of the group takes entries
// w, w + G, ... four at a time (independent loads in flight), lane l owns
// output columns l and l + 32; the group's partial rows are summed in warp
// order through shared memory, so the result does not depend on timing.
template <int G>
__global__ void __launch_bounds__(kPcaThreads) spmm_centred_kernel(const int64_t* __restrict__ rowptr,
                                                                   const int32_t* __restrict__ colidx,
                                                                   const double* __restrict__ vals, int64_t n,
                                                                   const double* __restrict__ Q, int r,
                                                                   const double* __restrict__ a,
                                                                   const double* __restrict__ c,
                                                                   const double* __restrict__ b,
                                                                   double* __restrict__ Y) {
  constexpr int kGroups = kPcaThreads / 32 / G;
  __shared__ double red[kPcaThreads / 32][2][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp / G, w = warp % G;
  const bool h0 = lane < r, h1 = lane + 32 < r;
  for (int64_t i0 = (int64_t)blockIdx.x * kGroups; i0 < n; i0 += (int64_t)gridDim.x * kGroups) {
    const int64_t i = i0 + grp;
    double y0 = 0.0, y1 = 0.0;
    if (i < n) {
      const int64_t e = rowptr[i + 1];
      int64_t k = rowptr[i] + w;
      for (; k + 3 * G < e; k += 4 * G) {
        int64_t j[4];
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          j[u] = colidx[k + u * G];
          v[u] = vals[k + u * G];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (h0) y0 = fma(v[u], Q[j[u] * r + lane], y0);
          if (h1) y1 = fma(v[u], Q[j[u] * r + lane + 32], y1);
        }
      }
      for (; k < e; k += G) {
        const int64_t j = colidx[k];
        const double v = vals[k];
        if (h0) y0 = fma(v, Q[j * r + lane], y0);
        if (h1) y1 = fma(v, Q[j * r + lane + 32], y1);
      }
    }
    if (G > 1) {
      red[warp][0][lane] = y0;
      red[warp][1][lane] = y1;
      __syncthreads();
      if (w == 0) {
        for (int q = 1; q < G; ++q) {
          y0 += red[warp + q][0][lane];
          y1 += red[warp + q][1][lane];
        }
      }
      __syncthreads();
    }
    if (i < n && w == 0) {
      const double ci = c ? c[i] : 0.0;
      if (h0) Y[i * r + lane] = y0 - (a ? a[lane] : 0.0) - ci * (b ? b[lane] : 0.0);
      if (h1) Y[i * r + lane + 32] = y1 - (a ? a[lane + 32] : 0.0) - ci * (b ? b[lane + 32] : 0.0);
    }
  }
}

// Partial Gram matrices of row blocks: part[blk] = sum over its rows of a_i^T a_i.
__global__ void __launch_bounds__(kPcaThreads) gram_partial_kernel(const double* __restrict__ A, int64_t n, int r,
                                                                   int64_t rpb, double* __restrict__ part) {
  __shared__ double row[32][kPcaMaxR];
  const int64_t r0 = (int64_t)blockIdx.x * rpb, r1 = min(n, r0 + rpb);
  const int rr = r * r;
  double acc[16];   // entries e = threadIdx.x + 256 t of the r x r matrix (r <= 64)
#pragma unroll
  for (int t = 0; t < 16; ++t) acc[t] = 0.0;
  for (int64_t i0 = r0; i0 < r1; i0 += 32) {
    const int rows = (int)((r1 - i0) < 32 ? (r1 - i0) : 32);
    for (int e = threadIdx.x; e < rows * r; e += blockDim.x) row[e / r][e % r] = A[(i0 + e / r) * r + e % r];
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int e = threadIdx.x + kPcaThreads * t;
      if (e < rr) {
        const int k = e / r, l = e % r;
        double s = acc[t];
        for (int q = 0; q < rows; ++q) s = fma(row[q][k], row[q][l], s);
        acc[t] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    const int e = threadIdx.x + kPcaThreads * t;
    if (e < rr) part[(int64_t)blockIdx.x * rr + e] = acc[t];
  }
}

__global__ void gram_final_kernel(const double* __restrict__ part, int64_t nb, int rr, double* __restrict__ G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rr) return;
  double s = 0.0;
  for (int64_t b = 0; b < nb; ++b) s += part[b * rr + e];
  G[e] = s;
}

// Partial vector-matrix products of K ranges: part[blk] = sum over its k of w_k Q_k
// (Q row-major, r <= 64 columns; lane l owns columns l and l + 32, warps take
// interleaved rows, summed in warp order).
__global__ void __launch_bounds__(kPcaThreads) vecmat_partial_kernel(const double* __restrict__ w,
                                                                     const double* __restrict__ Q, int64_t K, int r,
                                                                     int64_t kpb, double* __restrict__ part) {
  __shared__ double red[kPcaThreads / 32][2][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t k0 = (int64_t)blockIdx.x * kpb, k1 = min(K, k0 + kpb);
  const bool h0 = lane < r, h1 = lane + 32 < r;
  double y0 = 0.0, y1 = 0.0;
  for (int64_t k = k0 + warp; k < k1; k += kPcaThreads / 32) {
    const double wk = w[k];
    if (h0) y0 = fma(wk, Q[k * r + lane], y0);
    if (h1) y1 = fma(wk, Q[k * r + lane + 32], y1);
  }
  red[warp][0][lane] = y0;
  red[warp][1][lane] = y1;
  __syncthreads();
  if (warp == 0) {
    for (int q = 1; q < kPcaThreads / 32; ++q) {
      y0 += red[q][0][lane];
      y1 += red[q][1][lane];
    }
    if (h0) part[(int64_t)blockIdx.x * r + lane] = y0;
    if (h1) part[(int64_t)blockIdx.x * r + lane + 32] = y1;
  }
}

static int blocks_for(int64_t warps_needed) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((warps_needed + 7) / 8, (int64_t)sm_count() * 16));
}

}  // namespace wotg

using namespace wotg;

extern "C" int wotg_csr_count(const double* X, int64_t n, int64_t p, int64_t ldx, int64_t* rowptr, double* rowsum,
                              void* stream) {
  if (!X || !rowptr || n <= 0 || p <= 0 || ldx < p) return WOTG_BADARG;
  cudaStream_t st = (cudaStream_t)stream;
  csr_count_kernel<<<blocks_for(n), kPcaThreads, 0, st>>>(X, n, p, ldx, rowptr, rowsum);
  WOTG_LAUNCHED();
  exclusive_scan_kernel<<<1, 1024, 0, st>>>(rowptr, n, rowptr);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

extern "C" int wotg_csr_fill(const double* X, int64_t n, int64_t p, int64_t ldx, const int64_t* rowptr,
                             int32_t* colidx, double* vals, void* stream) {
  if (!X || !rowptr || !colidx || !vals || n <= 0 || p <= 0 || p > 2147483647LL || ldx < p) return WOTG_BADARG;
  csr_fill_kernel<<<blocks_for(n), kPcaThreads, 0, (cudaStream_t)stream>>>(X, n, p, ldx, rowptr, colidx, vals);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

static int64_t transpose_rpb(int64_t n) { return std::max<int64_t>(64, (n + 1023) / 1024); }

extern "C" size_t wotg_csr_transpose_workspace_bytes(int64_t n, int64_t p) {
  if (n <= 0 || p <= 0) return 0;
  const int64_t nb = (n + transpose_rpb(n) - 1) / transpose_rpb(n);
  return (size_t)nb * (size_t)p * sizeof(int32_t) + (size_t)p * sizeof(int64_t) + 512;
}

extern "C" int wotg_csr_transpose(const int64_t* rowptr, const int32_t* colidx, const double* vals, int64_t n,
                                  int64_t p, int64_t* t_rowptr, int32_t* t_colidx, double* t_vals, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  if (!rowptr || !colidx || !vals || !t_rowptr || !t_colidx || !t_vals || n <= 0 || p <= 0 ||
      n > 2147483647LL || p > 32768)
    return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_csr_transpose_workspace_bytes(n, p)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rpb = transpose_rpb(n), nb = (n + rpb - 1) / rpb;
  Bump b{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255)), 0};
  int32_t* cntb = b.take<int32_t>((size_t)nb * p);
  int64_t* total = b.take<int64_t>(p);
  const size_t smem = (size_t)p * sizeof(int32_t);
  static const cudaError_t attr1 = cudaFuncSetAttribute(csr_tcount_kernel,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 131072);
  static const cudaError_t attr2 = cudaFuncSetAttribute(csr_tfill_kernel,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 131072);
  WOTG_CUDA(attr1);
  WOTG_CUDA(attr2);
  csr_tcount_kernel<<<(unsigned)nb, kPcaThreads, smem, st>>>(rowptr, colidx, n, p, rpb, cntb);
  WOTG_LAUNCHED();
  csr_ttotal_kernel<<<(unsigned)((p + 255) / 256), 256, 0, st>>>(cntb, nb, p, total);
  WOTG_LAUNCHED();
  exclusive_scan_kernel<<<1, 1024, 0, st>>>(total, p, t_rowptr);
  WOTG_LAUNCHED();
  csr_toffset_kernel<<<(unsigned)((p + 255) / 256), 256, 0, st>>>(cntb, nb, p, t_rowptr);
  WOTG_LAUNCHED();
  csr_tfill_kernel<<<(unsigned)nb, kPcaThreads, smem, st>>>(rowptr, colidx, vals, n, p, rpb, cntb, t_rowptr,
                                                             t_colidx, t_vals);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

extern "C" int wotg_spmm_centred(const int64_t* rowptr, const int32_t* colidx, const double* vals, int64_t n,
                                 const double* Q, int32_t r, const double* a, const double* c, const double* b,
                                 double* Y, void* stream) {
  if (!rowptr || !colidx || !vals || !Q || !Y || n <= 0 || r < 1 || r > kPcaMaxR) return WOTG_BADARG;
  cudaStream_t st = (cudaStream_t)stream;
  // rows longer than a few hundred entries (a gene's row of the transpose) get a whole CTA each
  int64_t nnz = 0;
  WOTG_CUDA(cudaMemcpyAsync(&nnz, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  WOTG_CUDA(cudaStreamSynchronize(st));
  if (nnz > 256 * n) {
    const int grid = (int)std::min<int64_t>(n, (int64_t)sm_count() * 8);
    spmm_centred_kernel<8><<<grid, kPcaThreads, 0, st>>>(rowptr, colidx, vals, n, Q, r, a, c, b, Y);
  } else {
    const int grid = (int)std::min<int64_t>((n + 7) / 8, (int64_t)sm_count() * 16);
    spmm_centred_kernel<1><<<grid, kPcaThreads, 0, st>>>(rowptr, colidx, vals, n, Q, r, a, c, b, Y);
  }
  WOTG_LAUNCHED();
  return WOTG_OK;
}

static int64_t gram_rpb(int64_t n) { return std::max<int64_t>(256, (n + 2 * 152 - 1) / (2 * 152)); }

extern "C" size_t wotg_gram_workspace_bytes(int64_t n, int32_t r) {
  if (n <= 0 || r < 1 || r > kPcaMaxR) return 0;
  const int64_t nb = (n + gram_rpb(n) - 1) / gram_rpb(n);
  return (size_t)nb * r * r * sizeof(double) + 256;
}

extern "C" int wotg_gram_f64(const double* A, int64_t n, int32_t r, double* G, void* workspace,
                             size_t workspace_bytes, void* stream) {
  if (!A || !G || n <= 0 || r < 1 || r > kPcaMaxR) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_gram_workspace_bytes(n, r)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rpb = gram_rpb(n), nb = (n + rpb - 1) / rpb;
  double* part = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  gram_partial_kernel<<<(unsigned)nb, kPcaThreads, 0, st>>>(A, n, r, rpb, part);
  WOTG_LAUNCHED();
  gram_final_kernel<<<(r * r + 255) / 256, 256, 0, st>>>(part, nb, r * r, G);
  WOTG_LAUNCHED();
  return WOTG_OK;
}

static int64_t vecmat_kpb(int64_t K) { return std::max<int64_t>(1024, (K + 2 * 152 - 1) / (2 * 152)); }

extern "C" size_t wotg_vecmat_workspace_bytes(int64_t K, int32_t r) {
  if (K <= 0 || r < 1 || r > kPcaMaxR) return 0;
  return (size_t)((K + vecmat_kpb(K) - 1) / vecmat_kpb(K)) * r * sizeof(double) + 256;
}

extern "C" int wotg_vecmat_f64(const double* w, const double* Q, int64_t K, int32_t r, double* out, void* workspace,
                               size_t workspace_bytes, void* stream) {
  if (!w || !Q || !out || K <= 0 || r < 1 || r > kPcaMaxR) return WOTG_BADARG;
  if (!workspace || workspace_bytes < wotg_vecmat_workspace_bytes(K, r)) return WOTG_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t kpb = vecmat_kpb(K), nb = (K + kpb - 1) / kpb;
  double* part = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  vecmat_partial_kernel<<<(unsigned)nb, kPcaThreads, 0, st>>>(w, Q, K, r, kpb, part);
  WOTG_LAUNCHED();
  gram_final_kernel<<<1, 64, 0, st>>>(part, nb, r, out);   // fixed-order sum of the block partials
  WOTG_LAUNCHED();
  return WOTG_OK;
}
