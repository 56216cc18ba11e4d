/*
 * wotg.h — C ABI of the GB300-native transport-map library (libwotg.so).
 *
 * The reference (wot 1.0.8) is pure Python/NumPy; it has no FFI of its own.
 * Each entry point below replaces one NumPy-level operation or Python function
 * of the reference's transport-map path, cited as file:line inside the
 * reference project, and is what a ctypes / cffi binding of that path binds.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller; the library
 *    keeps no state between calls and allocates no device memory: every call
 *    that needs scratch takes a caller-provided workspace whose size comes from
 *    the matching *_workspace_bytes() query.
 *  - Dense cost matrices are FP32, row-major, I rows of `ldc` floats with
 *    ldc >= J and ldc % 4 == 0 (16-byte rows for 128-bit loads); columns
 *    [J, ldc) are padding and must hold +INFINITY (the cost writers do this).
 *  - `stream` is a cudaStream_t passed as void* (0 = legacy default stream).
 *  - Every function returns a wotg_status. WOTG_MAX_ITER is a warning: outputs
 *    are valid and follow the reference's max_iter behaviour.
 */
#ifndef WOTG_H
#define WOTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum wotg_status {
  WOTG_OK = 0,
  WOTG_MAX_ITER = 1,      /* reference: logger.warning + early return, optimal_transport.py:143-145 */
  WOTG_NONFINITE = 2,     /* reference: RuntimeError on NaN duality gap, optimal_transport.py:162-163 */
  WOTG_BADARG = 3,        /* reference: ValueError / TypeError on bad inputs */
  WOTG_CUDA_ERROR = 4,    /* a CUDA runtime call failed; see wotg_last_error() */
  WOTG_WORKSPACE = 5,     /* workspace pointer NULL or smaller than *_workspace_bytes() */
  WOTG_TOO_LARGE = 6      /* problem needs more scratch than the no-allocation entry point holds */
} wotg_status;

typedef enum wotg_form {
  WOTG_FORM_MATERIALIZED = 0, /* stream the FP32 cost matrix every half-step (HBM-bound) */
  WOTG_FORM_ONTHEFLY = 1      /* recompute cost tiles from the points on the tensor cores */
} wotg_form;

typedef enum wotg_solver {
  WOTG_SOLVER_DUALITY_GAP = 0, /* optimal_transport_duality_gap, optimal_transport.py:67-164 (default) */
  WOTG_SOLVER_FIXED_ITERS = 1  /* transport_stablev2, optimal_transport.py:167-236 */
} wotg_solver;

/* The reference's ot_config keys that reach the solver (ot_model.py:85-87). */
typedef struct wotg_params {
  double epsilon;
  double lambda1;
  double lambda2;
  double epsilon0;
  double tau;
  double tolerance;
  double max_iter;
  int32_t batch_size;
  int32_t scaling_iter;
  int32_t inner_iter_max;
  int32_t extra_iter;
  int32_t growth_iters;
  int32_t solver;         /* wotg_solver */
} wotg_params;

/* Counters of one compute_transport_matrix call (no counterpart in the reference). */
typedef struct wotg_stats {
  int64_t iterations;     /* Sinkhorn iterations summed over growth iterations */
  int64_t absorptions;    /* tau-absorptions (max|a|,|b| > tau) */
  int64_t checks;         /* stage-exit / duality-gap evaluations */
  double gap;             /* last relative duality gap (duality_gap solver) */
  double final_epsilon;   /* epsilon of the last stage */
  int32_t hit_max_iter;
  int32_t exact_rows;     /* rows the speculative on-the-fly half-step recomputed exactly (diagnostic) */
} wotg_stats;

/* One transport problem: a dense cost and the source growth G.
 * The reference's cost is cost_scale * C (cost_scale = 1/median for the default
 * cost, ot_model.py:252; 1 for a user-supplied cost, ot_model.py:307-311). */
typedef struct wotg_problem {
  int64_t I;              /* source cells (rows) */
  int64_t J;              /* target cells (columns) */
  const float* C;         /* device, I x ldc */
  int64_t ldc;
  double cost_scale;
  const double* G;        /* device, I (growth at the source day) */
  /* On-the-fly form only (form == WOTG_FORM_ONTHEFLY): the FP32 points whose
   * squared distances are C (row strides ldx, ldy floats, d <= 64). C is still
   * required: it serves the median, sum exp(-C/eps) and the dense output. */
  const float* X;
  int64_t ldx;
  const float* Y;
  int64_t ldy;
  int32_t d;
  int32_t form;           /* wotg_form; 0 (materialised) when zero-initialised */
} wotg_problem;

/* Library version string and last CUDA error text (host memory, static). */
const char* wotg_version(void);
const char* wotg_last_error(void);
/* Number of kernels this library has launched in this process (no counterpart
 * in the reference; used to attribute device work). */
unsigned long long wotg_launch_count(void);

/* Squared-Euclidean cost |x_i - y_j|^2 between FP32 points (I x d, J x d, row
 * strides ldx, ldy floats), written as an FP32 I x ldc matrix with +INF padding.
 * Replaces sklearn pairwise_distances(metric='sqeuclidean') at
 * wot/ot/ot_model.py:249-251 (coordinates already multiplied by the singular
 * values, ot_model.py:245-247). */
int wotg_cost_sqeuclidean(const float* X, int64_t I, int64_t ldx,
                          const float* Y, int64_t J, int64_t ldy, int32_t d,
                          float* C, int64_t ldc, void* stream);

/* Dense FP64 cost (row-major, I x J, as the reference's C) -> FP32 I x ldc with
 * +INF padding. Replaces np.asarray(C, dtype=np.float64) at
 * wot/ot/optimal_transport.py:100 for user-supplied cost matrices. */
int wotg_cost_from_f64(const double* C64, int64_t I, int64_t J, float* C, int64_t ldc,
                       void* stream);

/* np.median of the I x J valid entries of C (mean of the two middle values when
 * I*J is even), exact on the FP32 values, result in FP64 on the HOST.
 * Replaces np.median at wot/ot/ot_model.py:252. */
size_t wotg_median_workspace_bytes(void);
int wotg_median(const float* C, int64_t I, int64_t J, int64_t ldc, double* median_out,
                void* workspace, size_t workspace_bytes, void* stream);

/* Growth-iteration driver + solver: wot.ot.compute_transport_matrix
 * (wot/ot/optimal_transport.py:10-33) with solver = params->solver.
 * Outputs (device, any may be NULL):
 *   tmap            I x J FP64 row-major, the coupling the reference returns
 *                   (R / J, or R without / J when max_iter was hit)
 *   learned_growth  growth_iters x I FP64, the reference's learned_growth list
 *   row_sums        I FP64, tmap.sum(axis=1) of the returned coupling
 *                   (appended by OTModel, ot_model.py:319)
 *   u_bar, v_bar    I and J FP64 absorbed log-potentials (u + eps log a,
 *                   v + eps log b) of the last solve, so that
 *                   tmap = exp((u_bar_i + v_bar_j - cost_scale C_ij) / eps) / J
 *                   with eps = stats->final_epsilon.
 * stats (host) may be NULL. The final epsilon stage's batches of iterations
 * between duality-gap checks run as CUDA graphs, captured once per stage on a
 * stream of the call's own (ordered with `stream` by events; the stream, two
 * events and at most two graphs live for the call); the no-alloc entry point
 * launches plainly on `stream`. Results are the same either way. */
size_t wotg_solve_workspace_bytes(int64_t I, int64_t J, int64_t ldc);   /* materialised form */
size_t wotg_problem_workspace_bytes(const wotg_problem* problem);       /* any form */
int wotg_compute_transport_matrix(const wotg_problem* problem, const wotg_params* params,
                                  double* tmap, double* learned_growth, double* row_sums,
                                  double* u_bar, double* v_bar, wotg_stats* stats,
                                  void* workspace, size_t workspace_bytes, void* stream);

/* Warm-started fixed-epsilon iterations (no counterpart in the reference; its
 * iterations at the final epsilon are optimal_transport.py:131-141): from the
 * absorbed potentials (u_bar, v_bar, device, in/out), n_iter iterations of the
 * reference's a/b updates with tau-absorption at `epsilon`, same problem and
 * workspace as wotg_compute_transport_matrix. Polishes the potentials of a solve
 * stopped on the duality gap towards the exact optimum (before wotg_ot_adjoint).
 * stats (HOST, may be NULL): iterations = n_iter, absorptions, exact_rows. */
int wotg_refine_potentials(const wotg_problem* problem, const wotg_params* params, double epsilon, int32_t n_iter,
                           double* u_bar, double* v_bar, wotg_stats* stats, void* workspace, size_t workspace_bytes,
                           void* stream);

/* wotg_compute_transport_matrix for callers that cannot call cudaMalloc (a host
 * whose device memory is owned by another allocator or pool, or a path where
 * cudaMalloc's implicit device synchronisation is not acceptable). No counterpart
 * in the reference. Same inputs, outputs and results; the solver's scratch comes
 * from a static 32 MiB device array (wotg_noalloc_scratch_bytes()) held by every
 * device that loads the library until exit, instead of a caller workspace.
 * Problems whose wotg_problem_workspace_bytes() exceeds it return WOTG_TOO_LARGE
 * (message in wotg_last_error()); invalid problems return WOTG_BADARG as the
 * workspace entry point does. The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) and caches it for the life of
 * the process; make that call before any stream capture, and make no call
 * after cudaDeviceReset (the cached address does not survive a reset of the
 * device's context). Calls that overlap on the GPU share the array and race:
 * serialise them. Allocates nothing. */
size_t wotg_noalloc_scratch_bytes(void);
int wotg_compute_transport_matrix_noalloc(const wotg_problem* problem, const wotg_params* params,
                                          double* tmap, double* learned_growth, double* row_sums,
                                          double* u_bar, double* v_bar, wotg_stats* stats, void* stream);

/* One stabilised Sinkhorn half-step in the log domain, base 2:
 *   axis 0:  L[i] = ln2 * log2 sum_j 2^(w[j] - kappa2 C_ij)   (w: ldc floats, padding 0)
 *   axis 1:  L[j] = ln2 * log2 sum_i 2^(w[i] - kappa2 C_ij)   (w: I floats)
 * i.e. log(K v) and log(K^T u) of the reference's K.dot(b * dy) / K.T.dot(a * dx)
 * (wot/ot/optimal_transport.py:133-134) with K, a, b folded into w and C.
 * axis 1 needs wotg_lse_matvec_workspace_bytes() of workspace; axis 0 none. */
size_t wotg_lse_matvec_workspace_bytes(int64_t I, int64_t J, int64_t ldc);
int wotg_lse_matvec(const float* C, int64_t I, int64_t J, int64_t ldc, const float* w, float kappa2,
                    int32_t axis, double* L, void* workspace, size_t workspace_bytes, void* stream);

/* The same half-step from points, on the tensor cores (the on-the-fly form):
 *   L[i] = log sum_j exp(w[j] - scale |x_i - y_j|^2)
 * with X (I x d), Y (J x d) FP32 device points (row strides ldx, ldy; d <= 62),
 * w and L FP64 device vectors, scale > 0 (the reference's cost_scale / eps).
 * The K.dot(b * dy) of wot/ot/optimal_transport.py:133 in the log domain, with
 * the cost of ot_model.py:249-252 recomputed tile by tile instead of stored. */
size_t wotg_lse_points_workspace_bytes(int64_t I, int64_t J, int32_t d);
int wotg_lse_points(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy, int32_t d,
                    double scale, const double* w, double* L, void* workspace, size_t workspace_bytes,
                    void* stream);

/* wotg_lse_points with each of the tensor-core kernel's mbarrier waits bounded
 * to wait_tries tries (each suspends up to 1 us; wotg_lse_points and the
 * solvers use 4,000,000, about 4 s; wait_tries <= 4,000,000). No counterpart in
 * the reference, which has no device waits: this is the failure path of the
 * on-the-fly half-step made testable. A wait that runs out makes the kernel
 * stop issuing work, wait for every bulk copy and tensor-core product it has
 * issued to finish (with the full budget), free its tensor memory and return;
 * the call then returns WOTG_CUDA_ERROR with a message in wotg_last_error()
 * and the device stays usable. With wait_tries = 0 every wait runs out at once.
 * Synchronises the stream (to read the kernel's error word). */
int wotg_lse_points_bounded(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy,
                            int32_t d, double scale, const double* w, double* L, uint32_t wait_tries,
                            void* workspace, size_t workspace_bytes, void* stream);

/* A coupling held as potentials applied to k populations at once, on the
 * tensor cores with one exp per (i, j) for all of them:
 *   out[p * I + i] = exp(bias_i) sum_j exp(w[j] - scale |x_i - y_j|^2) P[p * ldp + j],  p < k
 * X (I x d), Y (J x d) FP32 points (d <= 62), w (J) and bias (I, may be NULL) FP64,
 * P FP64 k rows of ldp >= J weights (populations), out FP64 k x I, all on the
 * device. With w = v_bar / eps, bias = u_bar / eps + log scale and the
 * coupling's cost scale over eps it is the pull-back (tmap @ P.T).T of
 * transport_map_model.py:356 (push_forward, :290, with the roles of the two
 * point sets exchanged), for a map tmap = exp((u_bar + v_bar - C) / eps) scale
 * that is never formed. The populations go through the kernel eight at a time. */
size_t wotg_apply_points_workspace_bytes(int64_t I, int64_t J, int32_t d);
int wotg_apply_points(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy, int32_t d,
                      double scale, const double* w, const double* bias, const double* P, int64_t ldp, int32_t k,
                      double* out, void* workspace, size_t workspace_bytes, void* stream);

/* Diagnostic (no counterpart in the reference): the mean device time of the
 * tensor-core kernel of wotg_lse_points alone (no packing, no finish), over
 * n_launch back-to-back launches timed with CUDA events on `stream`. With
 * speculative != 0 each launch runs the form the solver uses once a row's
 * previous log-sum-exp is known (sums taken against that offset, no running
 * maximum); the offsets come from one exact launch first. Same arguments and
 * workspace as wotg_lse_points; synchronises the stream. */
int wotg_lse_points_timing(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy,
                           int32_t d, double scale, const double* w, int32_t speculative, int32_t n_launch,
                           float* ms_per_launch, void* workspace, size_t workspace_bytes, void* stream);

/* Diagnostics (no counterpart in the reference): one 128 x 128 x 32 tensor-core
 * product D = A B^T through the FP16 split used by the on-the-fly form
 * (terms = 1: hi.hi; 3: hi.hi + hi.lo + lo.hi), with the shared-memory
 * descriptor strides given (lbo, sbo <= 512 bytes). A, B: 128 x 32 FP32
 * row-major; D: 128 x 128 FP32; *err is set to 1 if a bounded wait timed out. */
int wotg_tc_selftest(const float* A, const float* B, float* D, uint32_t lbo, uint32_t sbo, int32_t terms,
                     int32_t* err, void* stream);

/* Dense population transport through one FP64 coupling X (I x J, row-major):
 *   transpose == 0:  out (k x J) = P (k x I) @ X      push_forward, transport_map_model.py:290
 *   transpose == 1:  out (k x I) = (X @ P^T)^T        pull_back,    transport_map_model.py:356
 * with optional per-row normalisation of out to sum 1 (:291-292, :357-358).
 * P and out are row-major FP64 on the device. */
int wotg_apply_coupling_f64(const double* X, int64_t I, int64_t J, const double* P, int32_t k,
                            int32_t transpose, int32_t normalize, double* out, void* stream);

/* ------------------------------------------------------------------------
 * Products of the local PCA (wot/ot/util.py:240-255: scikit-learn's PCA of the
 * double-centred genes x cells matrix of a day pair, whose randomized solver
 * multiplies that matrix and its transpose with thin blocks of vectors and
 * orthonormalises them). The expression matrix X (cells x genes, FP64) is taken
 * in CSR form; the centrings enter the products as rank-one terms.
 * ------------------------------------------------------------------------ */

/* CSR of the dense row-major X (n x p, row stride ldx): wotg_csr_count writes
 * rowptr (n + 1 int64: exclusive prefix sums of the row counts, rowptr[n] =
 * nnz) and, if rowsum is not NULL, each row's sum (n FP64); wotg_csr_fill then
 * writes colidx (int32) and vals (FP64) of nnz entries, ascending columns within
 * each row. */
int wotg_csr_count(const double* X, int64_t n, int64_t p, int64_t ldx, int64_t* rowptr, double* rowsum,
                   void* stream);
int wotg_csr_fill(const double* X, int64_t n, int64_t p, int64_t ldx, const int64_t* rowptr, int32_t* colidx,
                  double* vals, void* stream);

/* CSR of the transpose (p x n) of an n x p CSR matrix (p <= 32768), rows of
 * each output row in increasing order (a stable counting sort, so that products
 * with it sum in the same order on every run). */
size_t wotg_csr_transpose_workspace_bytes(int64_t n, int64_t p);
int wotg_csr_transpose(const int64_t* rowptr, const int32_t* colidx, const double* vals, int64_t n, int64_t p,
                       int64_t* t_rowptr, int32_t* t_colidx, double* t_vals, void* workspace,
                       size_t workspace_bytes, void* stream);

/* Y (n x r) = X Q - 1 a^T - c b^T for the n-row CSR X and Q (rows x r, row-major),
 * r <= 64; a, b (r) and c (n) may each be NULL (zero). With X the expression
 * matrix, a = mu^T Q, b = 1^T Q and c the per-cell centring it is the product of
 * the double-centred matrix the reference decomposes. */
int wotg_spmm_centred(const int64_t* rowptr, const int32_t* colidx, const double* vals, int64_t n, const double* Q,
                      int32_t r, const double* a, const double* c, const double* b, double* Y, void* stream);

/* G (r x r) = A^T A of a dense row-major A (n x r), r <= 64 (the Gram matrix of
 * the range finder's Cholesky QR), summed in a fixed order. */
size_t wotg_gram_workspace_bytes(int64_t n, int32_t r);
int wotg_gram_f64(const double* A, int64_t n, int32_t r, double* G, void* workspace, size_t workspace_bytes,
                  void* stream);

/* out (r) = w^T Q for w (K) and Q (K x r, row-major), r <= 64, summed in a fixed
 * order (the rank-one centring terms mu^T Q, 1^T Q, c^T Q of the PCA products). */
size_t wotg_vecmat_workspace_bytes(int64_t K, int32_t r);
int wotg_vecmat_f64(const double* w, const double* Q, int64_t K, int32_t r, double* out, void* workspace,
                    size_t workspace_bytes, void* stream);

/* Dense FP64 product of two couplings for a long-range map:
 *   C (M x N) = A (M x K) . B[b_rows] (K x N)
 * row-major with leading dimensions lda >= K, ldb >= N, ldc >= N; row k of the
 * right operand is row b_rows[k] of B (b_rows: K device int64 indices, or NULL
 * for B itself). Replaces np.dot(tmap_0.X, tmap_1[tmap_0.var.index].X) of
 * glue_transport_maps (wot/tmap/util.py:74-94), which chain_transport_maps
 * applies along a path of day pairs (wot/tmap/chaining.py:4-40). */
int wotg_gemm_f64(const double* A, int64_t lda, const double* B, int64_t ldb, const int64_t* b_rows, double* C,
                  int64_t ldc, int64_t M, int64_t N, int64_t K, void* stream);

/* ------------------------------------------------------------------------
 * Batched solves. The reference solves day pairs one after another
 * (OTModel.compute_all_transport_maps, wot/ot/ot_model.py:124-201, one
 * compute_transport_matrix per pair, ot_model.py:318) and a parameter sweep
 * repeats that per parameter set; here every (pair, parameter set) item of a
 * batch advances together: each Sinkhorn half-step is one persistent launch
 * over all pairs that reads a pair's cost once for all of its active items,
 * the reference's control flow (epsilon stages, batches, absorption, stage and
 * duality-gap tests, growth iterations) runs per item on the device, and the
 * iterations are replayed from a captured CUDA graph. Results per item are the
 * reference's (duality-gap solver only), returned as potentials:
 *   tmap_ij = exp((u_bar_i + v_bar_j - cost_scale C_ij) / eps) * scale
 * with eps = stats.final_epsilon and scale = 1/J (or 1 when max_iter was hit).
 * ------------------------------------------------------------------------ */

/* One day pair of a batch: its FP32 cost (as in wotg_problem) and the cost's
 * transpose, both with +INF padding, and the growth G of its source cells. */
typedef struct wotg_pair {
  int64_t I;
  int64_t J;
  const float* C;         /* device, I x ldc */
  int64_t ldc;
  const float* CT;        /* device, J x ldct: C transposed (wotg_transpose_cost) */
  int64_t ldct;
  double cost_scale;
  const double* G;        /* device, I */
} wotg_pair;

/* One transport problem of a batch: a pair, the solver parameters (solver must
 * be WOTG_SOLVER_DUALITY_GAP) and where its outputs go in the batch's
 * concatenated output arrays. */
typedef struct wotg_item {
  int32_t pair;
  int32_t reserved_;
  wotg_params params;
  int64_t row_offset;     /* first entry of this item's I-vectors in u_bar and row_sums */
  int64_t col_offset;     /* first entry of its J-vectors in v_bar */
  int64_t growth_offset;  /* first entry of its growth_iters x I learned growth */
} wotg_item;

/* CT (J x ldct) = C^T for the I x J valid entries of C, +INF in columns
 * [I, ldct). ldct >= I, ldct % 4 == 0. Building block of a batch (no
 * counterpart in the reference). */
int wotg_transpose_cost(const float* C, int64_t I, int64_t J, int64_t ldc, float* CT, int64_t ldct, void* stream);

/* Solves every item of the batch (see above). Outputs (device): u_bar, v_bar,
 * row_sums (tmap.sum(axis=1), the reference's learned growth appended by
 * OTModel, ot_model.py:319) at each item's offsets; learned_growth may be NULL.
 * stats and statuses (wotg_status per item) are HOST arrays of n_items, either
 * may be NULL. Returns WOTG_OK unless a call failed; per-item outcomes
 * (WOTG_MAX_ITER, WOTG_NONFINITE) are in statuses. The iterations run on an
 * internal stream ordered after `stream`; the call returns when all are done. */
size_t wotg_batch_workspace_bytes(const wotg_pair* pairs, int32_t n_pairs, const wotg_item* items, int32_t n_items);
int wotg_solve_batched(const wotg_pair* pairs, int32_t n_pairs, const wotg_item* items, int32_t n_items,
                       double* u_bar, double* v_bar, double* row_sums, double* learned_growth, wotg_stats* stats,
                       int32_t* statuses, void* workspace, size_t workspace_bytes, void* stream);

/* Diagnostic (no counterpart in the reference): the device time of one batched
 * pass over every item of every pair (speculative form, zero weights, no
 * epilogue: the exp-bound core of each half-step) for the configuration the
 * autotuner of the last wotg_solve_batched call in this process chose, as it
 * measured it with CUDA events (best of two launches), per direction: ms_row
 * over the rows of C, ms_col over the rows of CT; kg_rw (4 ints, may be NULL)
 * receives (items per register group, rows per warp) of each. WOTG_BADARG
 * before any batched solve. Host-side, no device work. */
int wotg_batch_pass_timing(float* ms_row, float* ms_col, int32_t* kg_rw);

/* Multi right-hand-side half-step on one materialised cost (row form of
 * wotg_lse_matvec for K weight vectors at once; each cost element is read once):
 *   L[k * ldl + i] = ln2 * log2 sum_j 2^(W[k * ldw + j] - kappa2[k] C_ij),  k < K
 * W: K rows of ldw >= roundup(J, 4) floats (16-byte aligned), finite or -INF
 * (entries [J, ldw) finite: they meet the cost's +INF padding);
 * kappa2: HOST array of K positive values. The K.dot(b * dy) of
 * optimal_transport.py:133 for several b, and the pull-back p @ tmap.T of
 * transport_map_model.py:356 for several populations on a coupling held as
 * potentials. */
size_t wotg_lse_matvec_multi_workspace_bytes(int64_t I, int32_t K);
int wotg_lse_matvec_multi(const float* C, int64_t I, int64_t J, int64_t ldc, const float* W, int64_t ldw,
                          const float* kappa2, int32_t K, double* L, int64_t ldl, void* workspace,
                          size_t workspace_bytes, void* stream);

/* Dense FP64 coupling from potentials (a batch item's map, or any solve's):
 *   out[i * J + j] = exp((u_bar_i + v_bar_j - cost_scale C_ij) / eps + log_scale)
 * (log_scale = -log J for the reference's return value R / J). */
int wotg_coupling_from_potentials(const float* C, int64_t I, int64_t J, int64_t ldc, double cost_scale, double eps,
                                  const double* u_bar, const double* v_bar, double log_scale, double* out,
                                  void* stream);

/* Gradient of the converged unbalanced entropic OT objective (no counterpart in
 * the reference, which has no derivatives): the objective is the reference's
 * dual at the optimum (optimal_transport.py:56-62, which its duality-gap test
 * drives to the primal, :146-152),
 *   D = -lambda1 dx sum_i p_i (e^(-u_bar_i/lambda1) - 1) - lambda2 dy q sum_j (e^(-v_bar_j/lambda2) - 1)
 *       - eps/(I J) sum_ij (R_ij - K0_ij),
 *   R_ij = exp((u_bar_i + v_bar_j - C_ij)/eps), K0_ij = exp(-C_ij/eps), C_ij = cost_scale |x_i - y_j|^2,
 *   dx = 1/I, dy = 1/J, q = mean(p),
 * differentiated by the envelope theorem at the converged potentials (u_bar,
 * v_bar from a solve with the same cost, e.g. wotg_compute_transport_matrix):
 * grad_x (I x d), grad_y (J x d, may be NULL), grad_p (I, may be NULL; the
 * derivative through q = mean(p) included) FP64 on the device; *objective
 * (HOST, may be NULL) = D. X, Y: FP32 points (row strides ldx, ldy), d <= 64;
 * the cost is recomputed from them tile by tile, never stored. */
size_t wotg_ot_adjoint_workspace_bytes(int64_t I, int64_t J);
int wotg_ot_adjoint(const float* X, int64_t I, int64_t ldx, const float* Y, int64_t J, int64_t ldy, int32_t d,
                    double cost_scale, double epsilon, double lambda1, double lambda2, const double* u_bar,
                    const double* v_bar, const double* p, double* grad_x, double* grad_y, double* grad_p,
                    double* objective, void* workspace, size_t workspace_bytes, void* stream);

/* Diagnostic (no counterpart in the reference): the replay profile of the last
 * wotg_solve_batched call on this host thread, one record per graph replay
 * (8 iterations of the whole batch): the number of items still active after
 * the previous replay and the host milliseconds between the waits on
 * successive replays (one replay's device time once the GPU is the bound).
 * Writes min(cap, n) records (either array may be NULL), returns n. */
int32_t wotg_batch_replay_profile(int32_t* active, float* ms, int32_t cap);

/* Diagnostic (no counterpart in the reference): this GPU's measured throughput
 * of ex2.approx.ftz.f32 (exp2 per second, a register-only kernel timed with CUDA
 * events on `stream`, best of 3). Every half-step form spends one exp2 per cost
 * element, so this is their ceiling; allocates nothing; synchronises the stream. */
int wotg_exp2_rate(double* exp2_per_s, void* stream);

/* Diagnostic (no counterpart in the reference): out[i] = 2^z[i] (n FP32 values
 * on the device) by the FMA-pipe exponential that the tensor-core epilogue
 * uses for a share of its elements (range reduction to [-1/2, 1/2], a degree-5
 * minimax polynomial, the exponent bits; z clamped to [-125, 126], NaN kept).
 * Lets a test hold it to its error bound against FP64 2^z. Asynchronous. */
int wotg_exp2_fma(const float* z, float* out, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WOTG_H */
