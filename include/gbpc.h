/*
 * gbpc.h — C ABI of the GB300-native preconditioned-Krylov library (libgbpc.so).
 *
 * Drop-in boundary for the hot path of alecjacobson/warp-preconditioners:
 * adaptive FSAI setup and application, cooperative sparse products, the
 * factored squared-Laplacian (biharmonic) operator, block Jacobi, block
 * ILU(0), block FSAI, scalar Jacobi, and the CG / CR loops that the reference
 * runs through warp.optim.linear.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer (cudaMalloc, torch, or any
 *     allocator on the current device) unless its name ends in `_host`.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream).
 *   - Index arrays are int32, CSR/BSR rows sorted with unique columns; BSR
 *     blocks are b x b, row-major, stored contiguously per block.
 *   - dtype codes: GBPC_F64, GBPC_F32, GBPC_BF16 (storage only).
 *   - Every function returns 0 (GBPC_OK) or a positive GBPC_ERR_* code;
 *     gbpc_last_error() gives a message for the calling thread.
 *   - Setup entry points synchronise `stream` to read validation counters
 *     (as the reference does); apply and solve entry points are
 *     stream-ordered, never synchronise and never allocate.
 *   - Linear operators follow the reference's LinearOperator.matvec contract
 *     z = alpha * Op * x + beta * y: x, y, z may alias each other, beta == 0
 *     never reads y and alpha == 0 never reads x.
 *   - An operator owns scratch memory: do not apply one operator concurrently
 *     on independent streams.
 */
#ifndef GBPC_H
#define GBPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gbpc_status {
  GBPC_OK = 0,
  GBPC_ERR_ARG = 1,          /* invalid argument (message says which) */
  GBPC_ERR_CUDA = 2,         /* CUDA runtime error */
  GBPC_ERR_DIAGONAL = 3,     /* FSAI: non-finite or non-positive diagonal ("positive diagonals") */
  GBPC_ERR_FACTOR = 4,       /* FSAI: factor lost finite entries or a positive diagonal */
  GBPC_ERR_CONVERSION = 5,   /* FSAI: factor dtype conversion lost finite entries or a positive diagonal */
  GBPC_ERR_PIVOT = 6,        /* block Jacobi / ILU(0): missing, non-finite or singular block pivot */
  GBPC_ERR_FREE_INDEX = 7,   /* squared Laplacian: free indices not distinct or out of bounds */
  GBPC_ERR_MASS = 8,         /* mass entries not finite and positive */
  GBPC_ERR_TIMEOUT = 9,      /* a bounded device wait gave up */
  GBPC_ERR_NOMEM = 10,       /* device allocation failed */
  GBPC_ERR_UNSUPPORTED = 11, /* input outside what this build implements (message says what) */
  GBPC_ERR_BLOCK_PIVOT = 12  /* block FSAI: non-positive local pivot */
};

enum gbpc_dtype { GBPC_F64 = 0, GBPC_F32 = 1, GBPC_BF16 = 2 };

/* Vector dtype code of a preconditioner applied in float32 behind a float64
 * interface: x, y, z are float64, the operator converts x to float32, runs
 * its products with float32 arithmetic on float32 or bfloat16 storage, and
 * widens the result (the precision option of the preconditioner only; the
 * Krylov method and the system operator stay float64).  Inside gbpc_solver
 * (CG) the conversions are fused into the loop's own vector kernels. */
enum { GBPC_F32_APPLY = 3 };

enum gbpc_method { GBPC_CG = 0, GBPC_CR = 1 };

/* Message of the last failing call on this thread (never NULL). */
const char* gbpc_last_error(void);
/* ABI version, currently 1. */
int gbpc_version(void);
/* Device bytes held by every live allocation of the library (operators,
 * solvers and their scratch; the fixed array of gbpc_fsai_apply_noalloc is
 * not counted).  No reference counterpart: serving admission control. */
int gbpc_device_bytes(size_t* live_host);

/* ------------------------------------------------------------------------ */
/* FSAI setup stages                                                         */
/* ------------------------------------------------------------------------ */

/* Adaptive FSAI factor rows.  Replaces the `diagonal` and `build` kernels and
 * their launches, warp_preconditioners/fsai.py:44-176 and :305-339, fused with
 * `sort_rows` (warp_preconditioners/fsai_pack.py:15-39).
 * Input: canonical scalar CSR A (n x n, dtype F64 or F32, arithmetic in that
 * type), width = max_row_size in [1, 64], step = max_step_size in [1, 64].
 * Output (device): ell_cols[n*width], ell_vals[n*width] (columns ascending,
 * the diagonal last, unused slots -1 / 0), row_counts[n], scale[n] = a_ii^-1/2.
 * status_host[3] receives the reference's counters: [0] invalid diagonals,
 * [1] truncated rows (pivot guard), [2] rows that lost finiteness or a
 * positive diagonal.  Returns GBPC_ERR_DIAGONAL / GBPC_ERR_FACTOR when the
 * reference raises.  Synchronises `stream`.  Temporary device memory, freed
 * before returning: the equilibrated entries (2 nnz values) and, for the rows
 * being built at once, each row's local factor, vectors and gathered entries
 * ((width (width + 1) / 2 + (2 + min(step, width)) width) values and
 * 2 width + min(step, width) + 5 ints per row; at most a quarter of the free
 * memory and 8 GB, rows taken in chunks beyond that). */
int gbpc_fsai_setup(int n, const int32_t* offsets, const int32_t* columns, const void* values,
                    int dtype, int width, int step, double kap_tolerance, double pivot_floor,
                    int32_t* ell_cols, void* ell_vals, int32_t* row_counts, void* scale,
                    int32_t* status_host, void* stream);

/* Compact sorted ELL rows to CSR.  Replaces `array_scan` + `pack`
 * (warp_preconditioners/fsai_pack.py:42-71).  With columns_out == NULL only
 * offsets_out[n+1] is written and *nnz_host returned (synchronises); call
 * again with the arrays sized *nnz_host. */
int gbpc_fsai_pack(int n, int width, const int32_t* ell_cols, const void* ell_vals,
                   const int32_t* row_counts, int dtype, int32_t* offsets_out,
                   int32_t* columns_out, void* values_out, int64_t* nnz_host, void* stream);

/* Explicit transpose of canonical CSR (rows of the result ascending).
 * Replaces warp.sparse.bsr_transposed as called at
 * warp_preconditioners/fsai.py:356.  t_off[ncol+1], t_col/t_val[nnz]. */
int gbpc_csr_transpose(int nrow, int ncol, const int32_t* offsets, const int32_t* columns,
                       const void* values, int dtype, int32_t* t_off, int32_t* t_col,
                       void* t_val, void* stream);

/* Canonical b x b BSR to scalar CSR keeping stored zeros.  Replaces
 * `scalarize` / `scalarize_compact` (warp_preconditioners/fsai_pack.py:74-130).
 * out_off[nrow_blocks*b+1], out_col/out_val[nnzb*b*b]. */
int gbpc_scalarize(int nrow_blocks, int b, const int32_t* offsets, const int32_t* columns,
                   const void* values, int dtype, int32_t* out_off, int32_t* out_col,
                   void* out_val, void* stream);

/* Factor storage conversion with validation.  Replaces the bsr_copy to a
 * narrower scalar type and `_validate_float32_factor`
 * (warp_preconditioners/fsai.py:181-196, :343-355).  *invalid_host receives
 * the number of rows with a non-finite value or a non-positive diagonal;
 * returns GBPC_ERR_CONVERSION when it is non-zero.  Synchronises. */
int gbpc_convert_factor(int n, const int32_t* offsets, const int32_t* columns, const void* src,
                        int src_dtype, void* dst, int dst_dtype, int32_t* invalid_host,
                        void* stream);

/* Fixed-support numeric refit.  Replaces RefitPlan.update's `diagonal` +
 * `refit` launches (warp_preconditioners/fsai_reuse.py:75-149, :189-245):
 * for every row i of G (CSR g_off/g_col, sorted, diagonal last, at most
 * `width` entries) the local Cholesky of the Jacobi-scaled A on G's support
 * is solved for e_i and normalised, written to out[nnz(G)] in factor_dtype
 * (matrix float64 -> factor float64 / float32 / bfloat16; float32 ->
 * float32 / bfloat16).  G itself is not touched.  status_host[0] counts
 * non-finite or non-positive diagonals of A, status_host[1] rows with a
 * pivot <= pivot_floor, a non-finite value or a non-positive diagonal; the
 * caller publishes `out` only when both are zero.  Synchronises.  For width
 * > 16 it allocates temporary device memory for the local factors of the
 * rows refitted at once (width (width + 1) / 2 values per row; at most a
 * quarter of the free memory and 8 GB, rows taken in chunks beyond that). */
int gbpc_fsai_refit(int n, const int32_t* a_off, const int32_t* a_col, const void* a_val,
                    int dtype, const int32_t* g_off, const int32_t* g_col, int width,
                    double pivot_floor, void* out, int factor_dtype, int32_t* status_host,
                    void* stream);

/* C = A diag(col_scale) B + diag(add_diag), float64 scalar CSR (col_scale,
 * add_diag nullable), on the device: the host SciPy assembly of the
 * smoothing operator Q = alpha M + K M^-1 K (results/dirichlet-tuning/
 * README.md:72-77) with SciPy's summation order: with col_scale the
 * contributions to C_ik arrive in decreasing j (SciPy's intermediate
 * A diag(d) holds each row with its columns decreasing), without it in
 * increasing j; then the diagonal term; exact zeros dropped, rows sorted.
 * Two-phase like gbpc_fsai_pack: c_col == NULL fills c_off[nrow+1] and
 * *nnz_host; the second call writes c_col / c_val.  Synchronises. */
int gbpc_spgemm(int nrow, int ncol, const int32_t* a_off, const int32_t* a_col,
                const double* a_val, const double* col_scale, int b_nrow, const int32_t* b_off,
                const int32_t* b_col, const double* b_val, const double* add_diag, int32_t* c_off,
                int32_t* c_col, double* c_val, int64_t* nnz_host, void* stream);

/* map_out[e] = position in the transpose (t_offsets/t_columns) of entry e of
 * the CSR matrix: replaces fsai_reuse.py `transpose_map` (:54-63).
 * GBPC_ERR_ARG if an entry has no transposed counterpart.  Synchronises. */
int gbpc_transpose_map(int nrow, const int32_t* offsets, const int32_t* columns,
                       const int32_t* t_offsets, const int32_t* t_columns, int32_t* map_out,
                       void* stream);

/* dst[map[e]] = src[e] for e < count (map[e] < 0 skipped): fsai_reuse.py
 * `transpose` (:151-155). */
int gbpc_scatter_values(int64_t count, const void* src, const int32_t* map, void* dst, int dtype,
                        void* stream);

/* ------------------------------------------------------------------------ */
/* Linear operators                                                          */
/* ------------------------------------------------------------------------ */

typedef struct gbpc_op gbpc_op;

/* z = alpha * A x + beta * y for square-block BSR A (block 1..4; block 1 is
 * scalar CSR).  Replaces SparseOperator (warp_preconditioners/
 * sparse_operator.py:107-139), its `_matvec` dispatch (:90-104) and
 * warp.sparse.bsr_mv for the A-apply of cg/cr.  value_dtype F64/F32/BF16;
 * vector_dtype F64 or F32.  Copies A into a device SELL-32 layout. */
int gbpc_op_sparse(int nrow, int ncol, int block, const int32_t* offsets,
                   const int32_t* columns, const void* values, int value_dtype,
                   int vector_dtype, void* stream, gbpc_op** out);

/* Preconditioners of the mixed harmonic systems (vectors interleave `order`
 * = 2 or 3 unknowns per vertex, n vertices; K scalar CSR, mass[n], both in
 * `dtype`; hinv an operator of this library approximating H^-1 on n-vectors,
 * referenced, not owned).  MatchingSchur replaces mixed.py:283-334 (block
 * elimination with repeated H^-1), ShiftedBlock mixed.py:388-427 (scale =
 * data_weight^(1/4)). */
int gbpc_op_matching_schur(int order, int n, const int32_t* k_off, const int32_t* k_col,
                           const void* k_val, int dtype, const void* mass, gbpc_op* hinv,
                           void* stream, gbpc_op** out);
int gbpc_op_shifted_block(int order, int n, double scale, int dtype, gbpc_op* hinv, void* stream,
                          gbpc_op** out);

/* Gram-form approximate inverse z = alpha * G^T (G x) + beta * y from
 * explicit G and G^T (scalar CSR, or b x b BSR for block FSAI).  Replaces
 * FSAI._apply (warp_preconditioners/fsai.py:393-400) and BsrBlockFSAI._apply
 * (benchmarks/block_fsai_candidate.py:311-332).  vector_dtype F64 / F32, or
 * GBPC_F32_APPLY (value_dtype F32 or BF16) for float64 vectors with float32
 * arithmetic inside; the reference's float32 factor storage
 * (fsai.py:255-263) accumulates in float64, which is vector_dtype F64. */
int gbpc_op_fsai(int nrow, int block, const int32_t* g_off, const int32_t* g_col,
                 const void* g_val, const int32_t* gt_off, const int32_t* gt_col,
                 const void* gt_val, int value_dtype, int vector_dtype, void* stream,
                 gbpc_op** out);
/* New values of G and G^T (same patterns as at creation) for an FSAI
 * operator, written in place so that captured applies use them (the
 * reference's refit keeps G.values and GT.values pointers). */
int gbpc_op_fsai_refill(gbpc_op* op, const int32_t* g_off, const int32_t* g_col,
                        const void* g_val, const int32_t* gt_off, const int32_t* gt_col,
                        const void* gt_val, int value_dtype, void* stream);

/* Factored (L diag(1/mass) L + mass_weight diag(mass))[free, free].
 * Replaces SquaredLaplacianOperator (warp_preconditioners/
 * squared_laplacian.py:103-198): setup `_index_free` + `mass_inverse`,
 * apply `forward` + `backward`.  L: scalar CSR n x n (F64 or F32),
 * mass[n], free[nfree].  Returns GBPC_ERR_FREE_INDEX / GBPC_ERR_MASS
 * as the reference raises.  Synchronises. */
int gbpc_op_sqlap(int n, const int32_t* offsets, const int32_t* columns, const void* values,
                  int dtype, const void* mass, const int32_t* free_indices, int nfree,
                  double mass_weight, void* stream, gbpc_op** out);

/* Eliminated right-hand side -((L M^-1 L) u_b)[free] of
 * SquaredLaplacianOperator.rhs (warp_preconditioners/squared_laplacian.py:
 * 200-218).  boundary_values[n], out[nfree]. */
int gbpc_sqlap_rhs(gbpc_op* op, const void* boundary_values, void* out, void* stream);

/* Scalar Jacobi z = alpha * x / diag(A) + beta * y on the scalar diagonal of
 * a BSR matrix.  Replaces warp.optim.linear.preconditioner(A, "diag") as used
 * at benchmarks/block_challenge.py:259-261 and benchmarks/synthetic.py:37. */
int gbpc_op_diagonal(int nrow, int block, const int32_t* offsets, const int32_t* columns,
                     const void* values, int dtype, void* stream, gbpc_op** out);

/* Block Jacobi: inverse diagonal blocks (1..4) with the scaled-determinant
 * guard.  Replaces BlockJacobi (warp_preconditioners/block_ilu.py:225-345):
 * `diagonal_only` + `safe_inverse` (:17-43, :76-104), `diagonal_apply`
 * (:188-202).  inverse_out[nrow*b*b] (optional, may be NULL) receives the
 * inverse blocks.  Returns GBPC_ERR_PIVOT when a pivot is missing, non-finite
 * or singular.  Synchronises. */
int gbpc_op_block_jacobi(int nrow, int block, const int32_t* offsets, const int32_t* columns,
                         const void* values, int dtype, double pivot_tolerance,
                         void* inverse_out, void* stream, gbpc_op** out);
/* New values for a BlockJacobi operator, in place (BlockJacobi.update,
 * warp_preconditioners/block_ilu.py:282-317): inverses are formed in a
 * candidate buffer and copied over the operator's (and inverse_out) only
 * when every pivot is valid; otherwise GBPC_ERR_PIVOT and nothing changes.
 * Captured applies see the new inverse.  Synchronises. */
int gbpc_op_block_jacobi_update(gbpc_op* op, int nrow, int block, const int32_t* offsets,
                                const int32_t* columns, const void* values, int dtype,
                                double pivot_tolerance, void* inverse_out, void* stream);

/* Synchronous block ILU(0) with Jacobi triangular sweeps.  Replaces BlockILU0
 * (warp_preconditioners/block_ilu.py:347-450): `topology`, `invert`,
 * `initialize`, `sweep`, `validate_factors` for setup and `triangular` +
 * `combine` for apply.  factors_out[nnzb*b*b] and inverse_out[nrow*b*b]
 * optional.  Synchronises. */
int gbpc_op_bilu0(int nrow, int block, const int32_t* offsets, const int32_t* columns,
                  const void* values, int dtype, int factor_sweeps, int solve_sweeps,
                  double relaxation, double pivot_tolerance, void* factors_out,
                  void* inverse_out, void* stream, gbpc_op** out);

/* Block-row adaptive FSAI rows (benchmarks/block_fsai_candidate.py:45-178,
 * `diagonal` + `build`): input b x b BSR (F64, b in 2..4, b*max_blocks <= 16),
 * output scalar ELL rows of width b*max_blocks (ell_cols/ell_vals
 * [nrow*b*b*max_blocks]), sorted by column like fsai_pack.py:15-39, with
 * row_counts[nrow*b], and scale[nrow*b].  refit != 0 reuses the supports
 * already in ell_cols.  Returns GBPC_ERR_BLOCK_PIVOT on a non-positive local
 * pivot.  Synchronises. */
int gbpc_block_fsai_setup(int nrow, int block, int max_blocks, const int32_t* offsets,
                          const int32_t* columns, const void* values, int refit,
                          int32_t* ell_cols, void* ell_vals, int32_t* row_counts, void* scale,
                          void* stream);

/* Scalar CSR whose rows come in groups of `block` to b x b BSR, zero-filling
 * missing entries of a stored block.  Replaces warp.sparse.bsr_copy(G,
 * block_shape=(b, b)) at benchmarks/block_fsai_candidate.py:300.  With
 * b_col == NULL only b_off[nrow_blocks+1] and *nnzb_host are produced
 * (synchronises); call again with b_col[nnzb], b_val[nnzb*b*b]. */
int gbpc_csr_to_bsr(int nrow_blocks, int block, const int32_t* offsets, const int32_t* columns,
                    const void* values, int dtype, int32_t* b_off, int32_t* b_col, void* b_val,
                    int64_t* nnzb_host, void* stream);

/* Explicit transpose of b x b BSR, transposing every block.  Replaces
 * warp.sparse.bsr_transposed at benchmarks/block_fsai_candidate.py:301 and
 * warp_preconditioners/biharmonic.py:98.  Synchronises. */
int gbpc_bsr_transpose(int nrow, int ncol, int block, const int32_t* offsets,
                       const int32_t* columns, const void* values, int dtype, int32_t* t_off,
                       int32_t* t_col, void* t_val, void* stream);

/* Apply an operator: z = alpha * Op * x + beta * y (vectors of the
 * operator's vector dtype, length = scalar rows).  Stream-ordered.  The
 * LinearOperator `_apply(x, y, z, alpha, beta)` protocol of the reference's
 * operators (warp_preconditioners/fsai.py:339, :374-381;
 * sparse_operator.py:90-104; block_ilu.py:188-202). */
int gbpc_op_apply(gbpc_op* op, const void* x, const void* y, void* z, double alpha, double beta,
                  void* stream);

/* Scalar length of the operator's vectors. */
int gbpc_op_rows(const gbpc_op* op, int64_t* rows_host);

/* Device bytes the operator holds (matrices, factors, scratch). */
int gbpc_op_device_bytes(const gbpc_op* op, size_t* bytes_host);

/* Release an operator and its device memory (synchronises the device). */
int gbpc_op_destroy(gbpc_op* op);

/* ------------------------------------------------------------------------ */
/* Krylov solvers                                                            */
/* ------------------------------------------------------------------------ */

/* Preconditioned CG (method GBPC_CG) or CR (GBPC_CR) on float64 vectors,
 * replacing warp.optim.linear.cg / cr as called at
 * benchmarks/block_challenge.py:131-139 and visualization/solve_fields.py:
 * 121-124.  Stops when the recursive r.r <= max(atol, tol |b|)^2 or after
 * maxiter iterations (maxiter <= 0 means n).  The whole loop runs on the
 * device inside one CUDA graph with a conditional while-node (use_graph != 0)
 * or as a host loop of the same kernels (use_graph == 0).  M may be NULL.
 * Device outputs (any may be NULL): nit_dev[1] int32, rr_dev[1] and
 * atol_sq_dev[1] float64 — stream-ordered, no synchronisation.  When any
 * *_host output is non-NULL the call synchronises and fills it. */
int gbpc_krylov(int method, gbpc_op* A, gbpc_op* M, const double* b, double* x, double tol,
                double atol, int maxiter, int use_graph, int32_t* nit_dev, double* rr_dev,
                double* atol_sq_dev, int32_t* nit_host, double* rr_host, double* atol_sq_host,
                void* stream);

/* FSAI application that allocates no device memory:
 * z = alpha * G^T (G x) + beta * y from the CSR arrays of G and G^T
 * (n x n, value_dtype F64 or F32; x, y, z float64 and device-resident).
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc: hosts that hand the library a fixed pool of
 * device memory and forbid further allocation, code paths that must stay
 * free of allocation calls (device memory is exhausted or reserved by the
 * host application, or allocation would synchronise or fail mid-pipeline).
 * The intermediate G x lives in a static array inside libgbpc.so of
 * gbpc_fsai_apply_noalloc_max_rows() = 524,288 float64 values (4 MiB);
 * larger n is rejected with GBPC_ERR_ARG.  CUDA loads the code holding that
 * array lazily: the first call on each device loads it and reserves the
 * 4 MiB there (kept until the process exits), and looks up the array's
 * device address (cudaGetSymbolAddress).  A call with n == 0 does only this,
 * so a host that later hands its free memory to a fixed pool makes one such
 * call per device first; make it, too, before any stream capture.  All calls
 * share the one array:
 * calls that overlap on the GPU (different streams, no ordering) race and
 * must be avoided.  x, y and z may alias; beta == 0 never reads y and
 * alpha == 0 never reads x.  No cudaMalloc, cudaFree or allocating library
 * routine is called. */
int gbpc_fsai_apply_noalloc(int n, const int32_t* g_off, const int32_t* g_col, const void* g_val,
                            const int32_t* gt_off, const int32_t* gt_col, const void* gt_val,
                            int value_dtype, const double* x, const double* y, double* z,
                            double alpha, double beta, void* stream);
/* Row limit of gbpc_fsai_apply_noalloc. */
int gbpc_fsai_apply_noalloc_max_rows(void);

/* Reusable solver: owns the work vectors and a cached CUDA graph for the
 * last (b, x) pair, so repeated solves cost one graph launch each.
 * `unroll` iterations (1..64, <= 0 selects the default 8) form one pass of
 * the device loop; the stopping test still runs after every iteration.
 * gbpc_solver_run is stream-ordered and never synchronises; outputs as for
 * gbpc_krylov.  Same reference call sites as gbpc_krylov. */
typedef struct gbpc_solver gbpc_solver;
int gbpc_solver_create(int method, gbpc_op* A, gbpc_op* M, int use_graph, int unroll,
                       void* stream, gbpc_solver** out);
int gbpc_solver_run(gbpc_solver* solver, const double* b, double* x, double tol, double atol,
                    int maxiter, int32_t* nit_dev, double* rr_dev, double* atol_sq_dev,
                    void* stream);

/* Residual history of the solver's next runs: hist[k] = |r_k|_2 (the
 * recursive residual the stopping test reads) for every iteration k <
 * hist_len, hist[0] the initial residual; hist_len = 0 turns it off.  The
 * iterates do not change.  Replaces the reference's diagnostic patch of
 * Warp's loop driver (benchmarks/residual_history.py:22-46). */
int gbpc_solver_set_history(gbpc_solver* solver, double* hist, int hist_len);

/* CTAs of the thread-block cluster that runs this solver's whole CG solve
 * as one kernel (small systems: at most ~600k multiply-adds per iteration,
 * a float64 scalar sparse or factored operator, an FSAI or no
 * preconditioner), or 0 when it runs the graph loop of separate kernels.
 * No reference counterpart. */
int gbpc_solver_cluster(const gbpc_solver* solver, int* cluster_host);
int gbpc_solver_destroy(gbpc_solver* solver);
/* Device bytes of the solver's Krylov state (work vectors, scalars). */
int gbpc_solver_device_bytes(const gbpc_solver* solver, size_t* bytes_host);

/* Restarted right-preconditioned GMRES(restart), restart <= 64: replaces
 * warp.optim.linear.gmres at the reference's call sites
 * (tests/test_biharmonic.py:32, tests/test_indefinite.py:130,
 * benchmarks/indefinite.py:192-225).  Arnoldi on A M with classical
 * Gram-Schmidt applied twice, Givens rotations, stop when the residual norm
 * |b - A x| (the Givens estimate) <= max(atol, tol |b|) or after maxiter
 * Arnoldi steps (maxiter <= 0: the vector length).  One CUDA graph per
 * (b, x) pair when use_graph != 0.  nit_dev / res_dev / target_dev
 * (optional) receive the steps, the final residual norm and the target. */
typedef struct gbpc_gmres gbpc_gmres;
int gbpc_gmres_create(gbpc_op* A, gbpc_op* M, int restart, void* stream, gbpc_gmres** out);
int gbpc_gmres_run(gbpc_gmres* solver, const double* b, double* x, double tol, double atol,
                   int maxiter, int use_graph, int32_t* nit_dev, double* res_dev,
                   double* target_dev, void* stream);
int gbpc_gmres_device_bytes(const gbpc_gmres* solver, size_t* bytes_host);
int gbpc_gmres_destroy(gbpc_gmres* solver);

/* ------------------------------------------------------------------------ */
/* Many right-hand sides: batched operators, batched PCG, mixed-precision     */
/* iterative refinement (no reference counterpart: the reference solves one   */
/* right-hand side per call; these serve its repeated-solve call sites        */
/* benchmarks/dragon.py:149-152 and visualization/solve_fields.py:121-124).   */
/* ------------------------------------------------------------------------ */

/* k <= 32 right-hand sides are stored row-major: row i of X is X[i*k..i*k+k).
 * value_dtype is the storage of the matrix values (F64, F32 or BF16, converted
 * on the device from in_dtype F64/F32 input); vector_dtype F64 or F32. */
typedef struct gbpc_bop gbpc_bop;
int gbpc_bop_sparse(int n, const int32_t* offsets, const int32_t* columns, const void* values,
                    int in_dtype, int value_dtype, int vector_dtype, void* stream, gbpc_bop** out);
/* max_rhs (1..32) sizes the operator's scratch: applies take k <= max_rhs. */
int gbpc_bop_fsai(int n, const int32_t* g_off, const int32_t* g_col, const void* g_val,
                  const int32_t* gt_off, const int32_t* gt_col, const void* gt_val, int in_dtype,
                  int value_dtype, int vector_dtype, int max_rhs, void* stream, gbpc_bop** out);
/* Factored alpha M + L M^-1 L with every vertex free (L float64 input). */
int gbpc_bop_sqlap(int n, const int32_t* offsets, const int32_t* columns, const void* values,
                   int in_dtype, int value_dtype, int vector_dtype, const double* mass,
                   double mass_weight, int max_rhs, void* stream, gbpc_bop** out);
/* Z = alpha * Op X + beta * Y for k right-hand sides (X must not alias Z). */
int gbpc_bop_apply(gbpc_bop* op, int k, const void* X, const void* Y, void* Z, double alpha,
                   double beta, void* stream);
int gbpc_bop_device_bytes(const gbpc_bop* op, size_t* bytes_host);
int gbpc_bop_destroy(gbpc_bop* op);

/* Batched preconditioned CG: k independent recurrences over the same
 * operator with per-right-hand-side scalars and stopping tests
 * (r_j.r_j <= max(atol, tol |b_j|)^2 or maxiter), float64 dots, whole loop
 * in one CUDA graph.  nit_dev[k], rr_dev[k] optional device outputs. */
typedef struct gbpc_bsolver gbpc_bsolver;
int gbpc_bsolver_create(gbpc_bop* A, gbpc_bop* M, int unroll, int max_rhs, void* stream,
                        gbpc_bsolver** out);
int gbpc_bsolver_run(gbpc_bsolver* solver, int k, const void* B, void* X, double tol,
                     double atol, int maxiter, int32_t* nit_dev, double* rr_dev, void* stream);
int gbpc_bsolver_device_bytes(const gbpc_bsolver* solver, size_t* bytes_host);
int gbpc_bsolver_destroy(gbpc_bsolver* solver);

/* Mixed-precision iterative refinement: residual b - A64 x in float64 (A64
 * a float64 batched operator), correction from `inner` (a batched solver,
 * typically float32 operator and float32 / bfloat16 FSAI) to relative
 * tolerance tol_inner, x += d in float64; right-hand side j stops once
 * max|d_j| <= tol_outer * max|x_j|.  B, X float64 [n*k].  Synchronises once
 * per outer step; outer_host[k] / inner_host[k] receive the counts. */
int gbpc_refine(gbpc_bop* A64, gbpc_bsolver* inner, int k, const double* B, double* X,
                double tol_outer, double tol_inner, int max_outer, int max_inner,
                int32_t* outer_host, int32_t* inner_host, void* stream);

/* Many independent systems of uneven size in one solve: preconditioned CG
 * on a block-diagonal A (and M) whose diagonal blocks are the systems,
 * system s owning rows [seg_rows_host[s], seg_rows_host[s + 1]).  Each
 * product is one launch for all systems; alpha, beta, the dot products,
 * the stopping test (r_s.r_s <= max(atol, tol |b_s|)^2 or maxiter, maxiter
 * <= 0 meaning the system's size) and the iteration count are per system,
 * and a system's iterates do not depend on the others in the solve.  Whole
 * loop in one CUDA graph (use_graph != 0) or a host loop of the same
 * kernels.  nit_dev / rr_dev / atol_sq_dev: nseg entries each (any may be
 * NULL).  No reference counterpart (the reference solves one system per
 * warp.optim.linear.cg call, benchmarks/block_challenge.py:131-139). */
typedef struct gbpc_msolver gbpc_msolver;
int gbpc_msolver_create(gbpc_op* A, gbpc_op* M, int nseg, const int64_t* seg_rows_host,
                        int use_graph, int unroll, void* stream, gbpc_msolver** out);
int gbpc_msolver_run(gbpc_msolver* solver, const double* b, double* x, double tol, double atol,
                     int maxiter, int32_t* nit_dev, double* rr_dev, double* atol_sq_dev,
                     void* stream);
int gbpc_msolver_device_bytes(const gbpc_msolver* solver, size_t* bytes_host);
int gbpc_msolver_destroy(gbpc_msolver* solver);

/* Many independent small systems in one launch, each solved by its own
 * thread-block cluster of 16 CTAs (8 where 16 cannot be scheduled): system s
 * is A[s] (a float64 scalar sparse operator, or a factored squared
 * Laplacian with every vertex free) preconditioned by M[s] (a float64
 * scalar FSAI, or NULL).  Nothing is concatenated; each cluster stops when
 * its own system passes the stopping test (r.r <= max(atol, tol |b_s|)^2,
 * or maxiter; maxiter <= 0 means the system's size).  A run solves systems
 * 0 .. count-1 (count <= nsys); b_host / x_host are host arrays of count
 * device pointers; nit_dev / rr_dev / atol_sq_dev hold count entries (any
 * may be NULL).  A system's iterates equal those of the
 * single-system cluster kernel that gbpc_solver uses for CG below 32,768
 * rows.  Stream-ordered.  No reference counterpart. */
typedef struct gbpc_csolver gbpc_csolver;
int gbpc_csolver_create(int nsys, gbpc_op* const* A, gbpc_op* const* M, void* stream,
                        gbpc_csolver** out);
int gbpc_csolver_run(gbpc_csolver* solver, int count, const double* const* b_host,
                     double* const* x_host, double tol, double atol, int maxiter,
                     int32_t* nit_dev, double* rr_dev, double* atol_sq_dev, void* stream);
int gbpc_csolver_cluster_size(const gbpc_csolver* solver, int* cluster_host);
int gbpc_csolver_device_bytes(const gbpc_csolver* solver, size_t* bytes_host);
int gbpc_csolver_destroy(gbpc_csolver* solver);

/* ------------------------------------------------------------------------ */
/* Vector utilities (dtype GBPC_F64 or GBPC_F32; stream-ordered, no
 * allocation, no synchronisation).                                          */
/* ------------------------------------------------------------------------ */

/* out[i] = 2 randi(rand_init(seed, i), 0, 2) - 1: the seeded Rademacher probe
 * of FSAI.quality (warp_preconditioners/fsai_reuse.py:143-147, the `probe`
 * kernel), drawn from Warp's PCG-hash stream. */
int gbpc_rademacher(int64_t n, int seed, int dtype, void* out, void* stream);

/* z = alpha x + beta y (alpha == 0 never reads x, beta == 0 never reads y;
 * z may alias x or y).  The vector update warp.optim.linear's loops and
 * fsai_reuse.py:149-152 (`subtract`) perform with Warp array ops. */
int gbpc_vec_axpby(int64_t n, int dtype, double alpha, const void* x, double beta,
                   const void* y, void* z, void* stream);

/* *result (device float64) = x . y accumulated in float64 in a fixed order
 * (the same value on every run), replacing warp.utils.array_inner
 * (fsai_reuse.py:277).  `work`: gbpc_vec_dot_work_size() device doubles. */
int gbpc_vec_dot_work_size(void);
int gbpc_vec_dot(int64_t n, int dtype, const void* x, const void* y, double* work,
                 double* result, void* stream);

/* FP64 FMA throughput probe: `ctas` CTAs of 256 threads, each thread 8
 * independent FMA chains of `iters` steps (8 * iters FMAs).  `out` holds 2
 * device doubles.  No reference counterpart: the benchmark times it to
 * measure the FP64 peak it divides by. */
int gbpc_fma_probe(int64_t iters, int ctas, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBPC_H */
