/*
 * rbg_gb300.h -- C ABI of the GB300 (sm_103a) AVOS transitive-closure library.
 *
 * One shared library, librbg_gb300.so, exports every entry point below.  Conventions:
 *   - plain pointers and sizes only; device buffers are owned by the caller;
 *   - every entry point that needs scratch takes a caller-provided `workspace` whose size
 *     the matching *_workspace_bytes query returns; no entry point allocates device memory
 *     behind the caller (rbg_fw_dense_noalloc uses a fixed array compiled into the library);
 *   - each call is ordered on the caller's CUDA stream (`stream`, a cudaStream_t; 0 is the
 *     legacy default stream); calls that report a status synchronise that stream before
 *     they return;
 *   - every entry point returns an int32 status (RBG_OK or an RBG_ERR_* code) and never
 *     throws across the ABI.
 *
 * Reference behaviour replaced (paths are within rappdw/redblackgraph):
 *   AVOS algebra       redblackgraph/core/src/redblackgraph/rbg_math.c.in:30-121
 *   dense closure      redblackgraph/core/src/redblackgraph/warshall.c.in:51-135
 *                      redblackgraph/sparse/csgraph/_shortest_path.pyx:213-389
 *   component closure  redblackgraph/sparse/csgraph/transitive_closure.py:85-195,
 *                      redblackgraph/sparse/csgraph/_components.pyx:86-344
 *   DAG closure        redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:168-351
 *   dense product      redblackgraph/core/src/redblackgraph/redblack.c.src:554-594
 *   sparse product     redblackgraph/sparse/sparsetools/rbm_math.h:117-222,
 *                      redblackgraph/gpu/spgemm.py:32-119
 *   squaring closure   redblackgraph/sparse/csgraph/transitive_closure.py:198-380,
 *                      redblackgraph/gpu/transitive_closure.py:26-184
 */
#ifndef RBG_GB300_H
#define RBG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void *rbg_stream_t; /* a cudaStream_t */

/* storage types, in the order of the reference's per-type loops (warshall.c.in:32-43) */
#define RBG_DTYPE_INT8 0
#define RBG_DTYPE_UINT8 1
#define RBG_DTYPE_INT16 2
#define RBG_DTYPE_UINT16 3
#define RBG_DTYPE_INT32 4
#define RBG_DTYPE_UINT32 5
#define RBG_DTYPE_INT64 6
#define RBG_DTYPE_UINT64 7

/* status codes */
#define RBG_OK 0
#define RBG_ERR_OVERFLOW 1 /* Python: OverflowError (rbg_math.c.in:103-118)           */
#define RBG_ERR_CYCLE 2    /* Python: ValueError / CycleError (warshall.c.in:82-86)    */
#define RBG_ERR_CAPACITY 3 /* Python: RuntimeError (capacity of a fixed buffer)       */
#define RBG_ERR_NOMEM 4    /* workspace too small or HBM budget exceeded              */
#define RBG_ERR_TIMEOUT 5  /* a bounded device wait gave up                           */
#define RBG_ERR_INVALID 6  /* bad argument                                            */
#define RBG_ERR_CUDA (-1)  /* a CUDA runtime call failed                              */

/* event bits reported in rbg_result_t.flags */
#define RBG_EV_OVF_SIZE 1u  /* msb(x)+msb(y) >= bits                                 */
#define RBG_EV_OVF_ONES 2u  /* product equals RED_ONE (all ones)                     */
#define RBG_EV_HANG 4u      /* the reference's MSB loop would never return here      */
#define RBG_EV_CYCLE 8u     /* a vertex reaches itself                               */
#define RBG_EV_RISK 16u     /* internal: clean-lane product reached the top bit      */
#define RBG_EV_UNCLEAN 32u  /* internal: input outside the clean regime              */
#define RBG_EV_WIDE 64u     /* internal: 64-bit values do not fit 32-bit lanes       */
#define RBG_EV_TIMEOUT 128u /* a bounded wait gave up                                */

/* mode bits for the dense closure */
#define RBG_MODE_CYTHON 1u      /* Cython floyd_warshall semantics (int32 only)          */
#define RBG_MODE_TRIANGULAR 2u  /* assume_upper_triangular loop (_shortest_path.pyx:365) */
#define RBG_MODE_FORCE_EXACT 4u /* always run the sequential-order kernel                */
#define RBG_MODE_FORCE_WIDE 8u  /* 64-bit storage: skip the 32-bit lane attempt          */
#define RBG_MODE_GRAPH 16u      /* rbg_fw_batch, rbg_fw_dense: record the launch sequence as
                                   a CUDA graph and replay it on later calls with the same
                                   sizes, offsets, buffers and workspace (small LRU cache);
                                   the DAG path's level loop is a while node the device ends,
                                   so a call is one graph launch and one read of results   */
#define RBG_MODE_TILE_NARROW 32u /* rbg_fw_batch: 128 x 64 phase-3 tiles in every round   */
#define RBG_MODE_AUTOTUNE 64u   /* rbg_fw_batch: per-round tile shape chosen by timing both
                                   shapes on the first call for a batch layout (the first
                                   call closes the batch twice; not when in == out)      */
#define RBG_MODE_NO_DAG 128u    /* rbg_fw_batch, rbg_fw_dense: no DAG path; every matrix
                                   takes the blocked (or exact) kernels                   */

/* which kernel path produced a result */
#define RBG_PATH_BLOCKED32 1
#define RBG_PATH_BLOCKED64 2
#define RBG_PATH_EXACT 3
#define RBG_PATH_DAG 4   /* int32 / int64 acyclic matrix in the clean regime, closed by the
                            DAG closure by levels                                          */

typedef struct rbg_result {
    int32_t status;   /* RBG_OK or RBG_ERR_*                                         */
    uint32_t flags;   /* RBG_EV_* bits seen                                          */
    int64_t diameter; /* MSB of the largest value written (warshall.c.in:89,106)     */
    int64_t k, i, j;  /* loop position of the event that decided `status`, else -1   */
    int32_t path;     /* RBG_PATH_* that produced the result                         */
    int32_t reserved;
    int64_t executed; /* relaxations the blocked kernels executed (skipped tiles excluded) */
} rbg_result_t;

/* Library version (major*10000 + minor*100 + patch). */
int32_t rbg_version(void);

/* Number of kernel launches this library has issued since it was loaded (no reference
 * counterpart: instrumentation for benchmarks). */
int64_t rbg_launch_count(void);

/* Start timing the blocked closure kernels with CUDA events recorded on the launching stream
 * (no reference counterpart: benchmark instrumentation; one process-wide timer). */
int32_t rbg_profile_begin(void);

/* Stop timing; ms[k] and launches[k] (k = 0 tile, 1 panel, 2 diagonal, 3 convert/finalize)
 * receive the summed kernel time and launch count since rbg_profile_begin. */
int32_t rbg_profile_end(double *ms, int64_t *launches);

/* rbg_profile_end for the first `slots` (1..9) timer slots: 0-3 as above, then the DAG path of
 * rbg_fw_batch / rbg_fw_dense: 4 scan, 5 closure by levels (with its CSR), 6 statistics, 7 write,
 * 8 the replay of matrices in any numbering (pattern, triples, replay). */
int32_t rbg_profile_end_slots(double *ms, int64_t *launches, int32_t slots);

/* Scratch bytes rbg_fw_dense needs for an n x n matrix of `dtype` under `mode`. */
int32_t rbg_fw_dense_workspace_bytes(int32_t dtype, int64_t n, uint32_t mode, int64_t *bytes);

/*
 * Dense AVOS transitive closure of one n x n matrix (row-major, leading dimensions in
 * elements).  Replaces the `warshall` gufunc loop {T}_warshall
 * (redblackgraph/core/src/redblackgraph/warshall.c.in:51-107, reached from
 * redblackgraph/core/redblack.py:49-50) and, with RBG_MODE_CYTHON, _floyd_warshall_avos
 * (redblackgraph/sparse/csgraph/_shortest_path.pyx:340-389).  `in` and `out` are device
 * pointers and may be equal.  Results (W, diameter and the error the reference raises) are
 * bit-exact with the reference; `result` (host memory) receives status, diameter and the
 * location of the deciding event.  Synchronises `stream`.
 */
int32_t rbg_fw_dense(int32_t dtype, int64_t n, const void *in, int64_t ld_in, void *out,
                     int64_t ld_out, uint32_t mode, void *workspace, int64_t workspace_bytes,
                     rbg_result_t *result, rbg_stream_t stream);

/* Largest n, and the size of the fixed device scratch array, of rbg_fw_dense_noalloc. */
#define RBG_NOALLOC_MAX_N 1024
#define RBG_NOALLOC_SCRATCH_BYTES (12u << 20)

/*
 * Dense AVOS closure that allocates nothing: same arguments, results and errors as
 * rbg_fw_dense, but without a workspace.  This entry point has no counterpart in the
 * reference.  It serves callers that cannot call cudaMalloc (allocation forbidden or unsafe
 * where they run, or a host program that owns only its input and output buffers): the
 * scratch is a 12 MiB array in the library's device image, which every GPU that loads the
 * library holds until the process exits.  n must be at most RBG_NOALLOC_MAX_N, otherwise the
 * call returns RBG_ERR_CAPACITY without touching the GPU.  The first call on a device looks up
 * the array's device address; make that first call before any stream capture (later calls
 * look it up again, so the address stays right after cudaDeviceReset).  All calls share the
 * one array: calls that overlap on the GPU race on it and must be serialised by the caller.
 * RBG_MODE_GRAPH is ignored here (instantiating a graph may take driver memory).
 * Synchronises `stream`.
 */
int32_t rbg_fw_dense_noalloc(int32_t dtype, int64_t n, const void *in, int64_t ld_in, void *out,
                             int64_t ld_out, uint32_t mode, rbg_result_t *result,
                             rbg_stream_t stream);

/* Scratch bytes rbg_fw_batch needs for `count` matrices of sizes `sizes` (host array). */
int32_t rbg_fw_batch_workspace_bytes(int32_t dtype, int64_t count, const int64_t *sizes,
                                     uint32_t mode, int64_t *bytes);

/*
 * Dense AVOS closure of `count` independent matrices in one batched run: matrix i is
 * sizes[i] x sizes[i], row-major and contiguous at element offset offsets[i] of the device
 * buffers `in` / `out` (which may be equal).  Every round of every matrix is issued as one
 * launch per kernel over all matrices still active, largest first.  Replaces the serial
 * per-component loop of component_wise_closure
 * (redblackgraph/sparse/csgraph/transitive_closure.py:161-190) and the gufunc batch loop
 * {T}_gufunc_warshall (redblackgraph/core/src/redblackgraph/warshall.c.in:110-135); each
 * matrix's W, diameter and error are those of rbg_fw_dense.  `results` (host, count entries)
 * receives one rbg_result_t per matrix.  Synchronises `stream`.
 */
int32_t rbg_fw_batch(int32_t dtype, int64_t count, const int64_t *sizes, const int64_t *offsets,
                     const void *in, void *out, uint32_t mode, void *workspace,
                     int64_t workspace_bytes, rbg_result_t *results, rbg_stream_t stream);
/*
 * DAG path of rbg_fw_batch and rbg_fw_dense (RBG_DTYPE_INT32 and RBG_DTYPE_INT64, unless
 * RBG_MODE_NO_DAG, RBG_MODE_TRIANGULAR, RBG_MODE_FORCE_EXACT or RBG_MODE_FORCE_WIDE is given): a
 * matrix in the clean regime (off-diagonal values 0 or in [2, 2^31), diagonal in {-1, 0, 1}),
 * with at most 16 off-diagonal entries per row and at most 8192 rows, whose graph is acyclic, is
 * closed through the DAG closure by levels.  With its vertices in a topological order (every
 * off-diagonal entry below, or every one above, the diagonal) the sequential loop's step k only
 * pushes row k into the rows of k's children (below) or pulls k's parents into the rows that
 * reach k (above), so the values are the DAG recurrence's and the diameter comes from each
 * cell's first product in step order.  In any other numbering the loop is replayed on the
 * closure's pattern (the triples (i, k, j) of each step with both cells in the pattern), which
 * gives the same diameter and overflow decision.  A matrix whose loop computes a product
 * reaching bit 31 continues without the 32-bit lanes: on 64-bit lanes (int64) or on the exact
 * kernel (int32).  The path's scratch (row slots, the candidates' CSR, the closure's row pool,
 * the replay's pattern and triples) is carved from `workspace`; a closure that does not fit
 * leaves its matrices to the blocked kernels.  Every accept / reject decision is made on the
 * device and the results are read back once per call.
 */

/* Destroy the CUDA graphs RBG_MODE_GRAPH keeps for the DAG path (waits for the device first);
 * the next call in that mode records again.  No reference counterpart. */
int32_t rbg_release_scratch(void);

/*
 * Row statistics rbg_fw_batch_rows records while it writes the closed matrices, so that a
 * caller merging them into one CSR matrix (rbg_cc_compact_scan + rbg_cc_compact_fill) need
 * not read them again.  Device arrays:
 *   row_base   [count]: matrix c's row i is output row row_id[row_base[c] + i], or
 *              row_base[c] + i when row_id is NULL
 *   row_count  nonzero values of every output row
 *   chunk_mask (NULL: none) 32-column chunks of every row that hold a nonzero, in the layout of
 *              rbg_cc_compact_count: ceil(sizes[c] / 2048) words per row, matrix c's rows from
 *              word ceil(offsets[c] / 2048) + row_base[c] + c
 *   comp_max   (NULL: none) [count] largest value of each matrix, by atomic max over values
 *              > 0: the caller zeroes it
 */
typedef struct rbg_row_stats {
    const int64_t *row_base;
    const int32_t *row_id;
    int64_t *row_count;
    uint64_t *chunk_mask;
    int32_t *comp_max;
} rbg_row_stats_t;

/*
 * rbg_fw_batch (RBG_DTYPE_INT32 only) that also records `stats` for every matrix whose result
 * comes from the 32-bit blocked pass (results[c].path == RBG_PATH_BLOCKED32 and status
 * RBG_OK); the rows of any other matrix are left unwritten.  Replaces the second read of the
 * closed blocks by merge_component_matrices' row counting (_components.pyx:254-290).
 */
int32_t rbg_fw_batch_rows(int32_t dtype, int64_t count, const int64_t *sizes, const int64_t *offsets,
                          const void *in, void *out, uint32_t mode, void *workspace,
                          int64_t workspace_bytes, const rbg_row_stats_t *stats, rbg_result_t *results,
                          rbg_stream_t stream);

/* ---------------------------------------------------------------------- sparse product */

/* A CSR matrix in device memory: int64 row pointers, int32 column indices (sorted, no
 * duplicates within a row), values of the call's dtype. */
typedef struct rbg_csr {
    int64_t n_rows, n_cols;
    const int64_t *indptr;
    const int32_t *indices;
    const void *data;
} rbg_csr_t;

/* scalar semantics of the sparse product */
#define RBG_SEM_C64 0  /* rb_matrix @: C core algebra on values widened to 64 bits, result cast
                          back to the storage type (redblackgraph/sparse/rbm.py:83-121)        */
#define RBG_SEM_CY32 1 /* redblackgraph.gpu: int32 values, Cython algebra, silent wrap
                          (redblackgraph/gpu/spgemm_numeric.py:61-88)                          */

/* Bytes of the workspace that lives from rbg_spgemm_count to rbg_spgemm_gather ("head"). */
int32_t rbg_spgemm_head_bytes(int64_t n_rows, int64_t *bytes);

/*
 * Step 1 of C = A (x) B, optionally merged with R as one squaring step R (+) R^2 (R = A = B,
 * R's value kept on magnitude ties, result int32: redblackgraph/sparse/csgraph/
 * transitive_closure.py:272-357, redblackgraph/gpu/transitive_closure.py:77-156): counts the
 * candidate products per row (replaces rbm_matmat_pass1, redblackgraph/sparse/sparsetools/
 * rbm_math.h:117-156, and the symbolic phase, redblackgraph/gpu/spgemm_symbolic.py:250-353).
 * `upper` keeps only columns j >= i (redblackgraph/gpu/spgemm.py:32-119).  Returns the total
 * candidates and the number of rows that need the dense accumulator.  Synchronises `stream`.
 */
int32_t rbg_spgemm_count(const rbg_csr_t *A, const rbg_csr_t *B, const rbg_csr_t *R, int32_t upper,
                         void *head, int64_t head_bytes, int64_t *total_candidates,
                         int64_t *dense_rows, rbg_stream_t stream);

/* Bytes of the second workspace ("tail") for the counts rbg_spgemm_count returned. */
int32_t rbg_spgemm_tail_bytes(int64_t n_rows, int64_t n_cols, int64_t total_candidates,
                              int64_t dense_rows, int64_t *bytes);

/*
 * Step 2: numeric product (replaces rbm_matmat_pass2, redblackgraph/sparse/sparsetools/
 * rbm_math.h:165-222, and the numeric phase, redblackgraph/gpu/spgemm_numeric.py:104-327).
 * Each row's columns come out sorted; zero sums are dropped.  Returns nnz(C) and the event
 * flags (RBG_ERR_OVERFLOW when a RBG_SEM_C64 product overflows).  Synchronises `stream`.
 */
int32_t rbg_spgemm_numeric(int32_t sem, int32_t dtype, const rbg_csr_t *A, const rbg_csr_t *B,
                           const rbg_csr_t *R, int32_t upper, void *head, void *tail,
                           int64_t tail_bytes, int64_t total_candidates, int64_t dense_rows,
                           int64_t *nnz, uint32_t *flags, rbg_stream_t stream);

/* Step 3: write C into caller buffers: indptr (n_rows + 1, int64), indices (nnz, int32),
 * data (nnz, dtype).  Ordered on `stream`, no synchronisation. */
int32_t rbg_spgemm_gather(int32_t dtype, int64_t n_rows, int64_t n_cols, const void *head,
                          const void *tail, int64_t total_candidates, int64_t dense_rows,
                          int64_t *indptr, int32_t *indices, void *data, rbg_stream_t stream);

/*
 * Z = X (+) Y cell by cell with the squaring merge's magnitude rule (the value of smaller
 * |value|, X's on a tie, zero results dropped; int32 values, sorted rows).  Replaces
 * sparse_avos_sum_gpu (redblackgraph/gpu/transitive_closure.py:77-156).  Count step (head sized
 * by rbg_spgemm_head_bytes; synchronises `stream`), then fill step into caller buffers.
 */
int32_t rbg_csr_merge_count(const rbg_csr_t *X, const rbg_csr_t *Y, void *head, int64_t head_bytes,
                            int64_t *nnz, rbg_stream_t stream);
int32_t rbg_csr_merge_fill(const rbg_csr_t *X, const rbg_csr_t *Y, const void *head, int64_t *indptr,
                           int32_t *indices, int32_t *data, rbg_stream_t stream);

/*
 * The entries of X that Y does not hold with the same value: Z = {(i, j, X[i][j]) : (i, j) not
 * stored in Y, or Y[i][j] != X[i][j]} (values compared as integers; X and Y of any RBG_DTYPE_*,
 * rows sorted, no duplicates).  The squaring closure's step difference: with Z = R_t minus R_(t-1),
 * R_(t+1) = R_t (+) R_t^2 equals R_t (+) Z R_t (+) R_t Z, because every product of two entries
 * that did not change was already folded into R_t (the semi-naive form of the squaring loop of
 * redblackgraph/sparse/csgraph/transitive_closure.py:198-380 and
 * redblackgraph/gpu/transitive_closure.py:26-72).  Count step (head sized by
 * rbg_spgemm_head_bytes; *nnz on the host; synchronises `stream`), then fill step into caller
 * buffers (Z's values in X's storage type).
 */
int32_t rbg_csr_diff_count(int32_t x_dtype, const rbg_csr_t *X, int32_t y_dtype, const rbg_csr_t *Y, void *head,
                           int64_t head_bytes, int64_t *nnz, rbg_stream_t stream);
int32_t rbg_csr_diff_fill(int32_t x_dtype, const rbg_csr_t *X, int32_t y_dtype, const rbg_csr_t *Y,
                          const void *head, int64_t *indptr, int32_t *indices, void *data, rbg_stream_t stream);

/*
 * Operands of one semi-naive squaring step as a single product: A' = [D R] (n x 2n: row i is D's
 * row i, then R's row i with its columns moved by n) and B' = [R ; D] (2n x n: R's rows, then
 * D's), so that A' B' = D R (+) R D, and rbg_spgemm_* on (A', B') with R merged forms
 * R (+) D R (+) R D in one pass.  D and R: n x n, values of `dtype` (4 or 8 bytes), rows sorted.
 * Caller buffers: a_indptr n + 1, b_indptr 2n + 1, indices and data nnz(D) + nnz(R) each.
 * Reads nnz(D) and nnz(R) back (synchronises `stream`), then enqueues the copies.
 */
int32_t rbg_spgemm_seminaive_operands(int32_t dtype, const rbg_csr_t *D, const rbg_csr_t *R, int64_t *a_indptr,
                                      int32_t *a_indices, void *a_data, int64_t *b_indptr, int32_t *b_indices,
                                      void *b_data, rbg_stream_t stream);

/*
 * Diameter source of the sparse DAG closure: the largest magnitude among the stored entries of A
 * and the candidates A[v][w] (x) C[w][x] (w != v, x over row w of the closure C, Cython int32
 * product), as redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:262-305 keeps it
 * (candidates that lose the (+) included).  int32 values; `workspace` needs 8 bytes; *max_abs
 * (host) receives the maximum.  Synchronises `stream`.
 */
int32_t rbg_dag_candidate_max(const rbg_csr_t *A, const rbg_csr_t *C, void *workspace,
                              int64_t workspace_bytes, int64_t *max_abs, rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Closure of a DAG by topological levels (replaces transitive_closure_dag_sparse_cython,
 * redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:168-351, and the level-parallel
 * transitive_closure_dag_gpu, redblackgraph/gpu/transitive_closure.py:474-652).
 * ---------------------------------------------------------------------------------------- */

/* Scratch bytes rbg_dag_closure needs for n vertices and nnz stored entries. */
int32_t rbg_dag_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes);

/*
 * Row v of the closure = v's stored entries (+) A[v][w] (x) C[w][.] over v's parents w != v
 * (Cython int32 product and sum), computed level by level into a caller-provided row pool
 * (pool_cols / pool_vals, pool_capacity entries; row v at row_off[v], row_len[v] entries,
 * columns ascending; row_off / row_len are device arrays of n).  A is CSR with int32 values.
 * Returns RBG_OK with *nnz (host) = entries used and *max_abs = the largest magnitude of any
 * stored entry or candidate (the reference's diameter source); RBG_ERR_CAPACITY when the pool
 * is too small (*nnz = a size to retry with) or a row has more than 8192 distinct columns
 * (*nnz = -1); RBG_ERR_CYCLE when the graph has a cycle.  *levels (host) = topological
 * levels.  Synchronises `stream` once per eight levels.
 */
int32_t rbg_dag_closure(const rbg_csr_t *A, void *workspace, int64_t workspace_bytes, int32_t *pool_cols,
                        int32_t *pool_vals, int64_t pool_capacity, int64_t *row_off, int32_t *row_len,
                        int64_t *nnz, int64_t *max_abs, int64_t *levels, rbg_stream_t stream);

/* Scratch bytes rbg_dag_gather needs. */
int32_t rbg_dag_gather_workspace_bytes(int64_t n, int64_t *bytes);

/* The pooled rows of rbg_dag_closure as CSR: indptr (n + 1, int64), indices and data (int32).
 * Ordered on `stream`. */
int32_t rbg_dag_gather(int64_t n, const int32_t *pool_cols, const int32_t *pool_vals, const int64_t *row_off,
                       const int32_t *row_len, void *workspace, int64_t workspace_bytes, int64_t *indptr,
                       int32_t *indices, int32_t *data, rbg_stream_t stream);

/* Scratch bytes rbg_avos_matmul needs. */
int32_t rbg_avos_matmul_workspace_bytes(int32_t dtype, int64_t m, int64_t q, int64_t p,
                                        int64_t *bytes);

/*
 * Dense AVOS product C[m,p] = A[m,q] (x) B[q,p] (row-major device buffers) under the C core
 * scalar semantics.  Replaces the AVOS einsum inner loop
 * {T}_sum_of_products_contig_contig_outstride0_two (redblackgraph/core/src/redblackgraph/
 * redblack.c.src:554-594) behind rb.array @ (redblackgraph/core/redblack.py:14-38).
 * Returns RBG_ERR_OVERFLOW when any product overflows (OverflowError in the reference);
 * `flags` (host) receives the RBG_EV_* bits.  Synchronises `stream`.
 */
int32_t rbg_avos_matmul(int32_t dtype, int64_t m, int64_t q, int64_t p, const void *A, int64_t lda,
                        const void *B, int64_t ldb, void *C, int64_t ldc, void *workspace,
                        int64_t workspace_bytes, uint32_t *flags, rbg_stream_t stream);

/*
 * Element-wise AVOS sum (op 0) or product (op 1) of two device arrays of n elements:
 * z[i] = x[i] (+) y[i] or x[i] (x) y[i] (the product's bits are the unsigned result the C core
 * returns).  Replaces c_avos_sum / c_avos_product (redblackgraph/core/src/redblackgraph/
 * redblackgraphmodule.c:491-533) and avos_sum_kernel / avos_product_kernel
 * (redblackgraph/gpu/avos_kernels.py:150-176).  Returns RBG_ERR_OVERFLOW when a product
 * overflows.  `workspace` needs 256 bytes.  Synchronises `stream`.
 */
int32_t rbg_avos_elementwise(int32_t op, int32_t dtype, int64_t n, const void *x, const void *y,
                             void *z, void *workspace, int64_t workspace_bytes, uint32_t *flags,
                             rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Component-wise closure (redblackgraph/sparse/csgraph/transitive_closure.py:85-195): split a
 * CSR graph (n vertices; int64 indptr, int32 indices, int32 values, all device buffers) into its
 * connected components, densify each into the rbg_fw_batch layout, close them in one batch,
 * and compact the closed blocks back into one CSR matrix with global indices.
 * ---------------------------------------------------------------------------------------- */

/* Scratch bytes the rbg_cc_* calls need for an n-vertex graph (one workspace serves all). */
int32_t rbg_cc_workspace_bytes(int64_t n, int64_t *bytes);

/*
 * Connected components with edges taken in both directions, numbered by their least vertex
 * (replaces find_components_sparse, redblackgraph/sparse/csgraph/_components.pyx:86-177, and
 * get_component_vertices, :326-344).  Outputs (device, caller-allocated):
 *   label[n]          component of each vertex
 *   sorted_vertex[n]  vertices grouped by component, ascending inside each component
 *   local[n]          index of each vertex inside its component (extract_submatrix's renumbering,
 *                     _components.pyx:180-252)
 *   start[n + 1]      component c holds sorted_vertex[start[c] .. start[c + 1])
 * and *ncomp (host).  The union-find loop is bounded (log2 n + 64 hooking passes); reaching
 * the bound returns RBG_ERR_TIMEOUT.  Synchronises `stream`.
 */
int32_t rbg_cc_label(int64_t n, const int64_t *indptr, const int32_t *indices, void *workspace,
                     int64_t workspace_bytes, int32_t *label, int32_t *sorted_vertex,
                     int32_t *local, int64_t *start, int64_t *ncomp, rbg_stream_t stream);

/*
 * Write each component's dense block into `flat` (elements of `dtype`, RBG_DTYPE_INT32 or
 * RBG_DTYPE_INT64): component c is the start[c+1]-start[c] square at element offset
 * dense_off[c] (device array); its rows are zeroed and every stored int32 value
 * (sign-extended for int64) is scattered in.  Replaces extract_submatrix + toarray
 * (_components.pyx:180-252, transitive_closure.py:172-176).  Only the blocks are written, so
 * they may sit anywhere in a larger buffer (flat_elems bounds them; a block past it is
 * skipped).  Any grouping of the vertices into blocks works, not only connected components;
 * entries joining two blocks are dropped.  Ordered on `stream`.
 */
int32_t rbg_cc_densify(int32_t dtype, int64_t n, const int64_t *indptr, const int32_t *indices,
                       const int32_t *data, const int32_t *label, const int32_t *local,
                       const int64_t *start, const int64_t *dense_off, void *flat,
                       int64_t flat_elems, rbg_stream_t stream);

/* 64-bit words of the optional chunk mask of rbg_cc_compact_count / _fill for a batch of
 * flat_elems dense elements. */
int32_t rbg_cc_chunk_mask_words(int64_t n, int64_t ncomp, int64_t flat_elems, int64_t *words);

/*
 * Count the nonzeros of the closed blocks per global row and scan them; *nnz (host) is the
 * merged matrix's nnz.  When comp_max (device, ncomp int32) is not NULL it receives the largest
 * value of each closed component, floored at 0 (the final-value diameter of the 'D' method,
 * redblackgraph/sparse/csgraph/_shortest_path.pyx:842-845).  When chunk_mask (device,
 * rbg_cc_chunk_mask_words words) is not NULL it records which 32-column chunks of every row
 * hold a nonzero, and rbg_cc_compact_fill then reads only those.  Synchronises `stream`.
 */
int32_t rbg_cc_compact_count(int64_t n, int64_t ncomp, const int32_t *label, const int32_t *local,
                             const int64_t *start, const int64_t *dense_off, const int32_t *flat,
                             void *workspace, int64_t workspace_bytes, int64_t *nnz,
                             int32_t *comp_max, uint64_t *chunk_mask, rbg_stream_t stream);

/*
 * rbg_cc_compact_count for counts already known (row_count, device, n int64: the
 * rbg_fw_batch_rows statistics): scans them into the workspace for rbg_cc_compact_fill;
 * *nnz (host) is the merged matrix's nnz.  Synchronises `stream`.
 */
int32_t rbg_cc_compact_scan(int64_t n, const int64_t *row_count, void *workspace, int64_t workspace_bytes,
                            int64_t *nnz, rbg_stream_t stream);

/*
 * Write the merged CSR matrix (replaces merge_component_matrices, _components.pyx:254-324):
 * indptr (n + 1, int64), indices (nnz, int32, ascending in each row), data (nnz, int32).  Uses
 * the counts (and the chunk mask, when not NULL) rbg_cc_compact_count left.  Ordered on `stream`.
 */
int32_t rbg_cc_compact_fill(int64_t n, const int32_t *label, const int32_t *local,
                            const int64_t *start, const int64_t *dense_off, const int32_t *flat,
                            const int32_t *sorted_vertex, const void *workspace, int64_t *indptr,
                            int32_t *indices, int32_t *data, const uint64_t *chunk_mask, rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Component-wise closure straight from the CSR graph (no dense blocks) when every component is
 * numbered in a topological order (its off-diagonal entries all below, or all above, the
 * diagonal) and in the clean regime: the DAG path of rbg_fw_batch applied to the graph.  The
 * sequence is rbg_cc_dag_classify -> rbg_cc_dag_edges -> rbg_dag_closure on the edges (its row
 * pool is read as it is) -> rbg_cc_dag_stats -> rbg_cc_dag_merge_count / _fill; values and diameters are
 * those of merge_component_matrices over the reference's per-component closures
 * (redblackgraph/sparse/csgraph/transitive_closure.py:85-195).  Components come from
 * rbg_cc_label; `workspace` is its workspace.
 * ---------------------------------------------------------------------------------------- */

/* comp_flags[c] (device, ncomp): bit 0 outside the clean regime, bit 1 an entry below the
 * diagonal, bit 2 an entry above it; diag (device, n): each row's diagonal value (0 when not
 * stored); edge_ptr (device, n + 1): row pointers of the off-diagonal nonzeros, *edges (host)
 * their number.  sorted_vertex and start (ncomp + 1 entries, start[ncomp] = n) as rbg_cc_label
 * writes them; a graph of n > 0 vertices without components is RBG_ERR_INVALID.  Synchronises
 * `stream`. */
int32_t rbg_cc_dag_classify(int64_t n, const int64_t *indptr, const int32_t *indices, const int32_t *data,
                            const int32_t *sorted_vertex, const int64_t *start, int64_t ncomp,
                            void *workspace, int64_t workspace_bytes, uint32_t *comp_flags, int32_t *diag,
                            int64_t *edge_ptr, int64_t *edges, rbg_stream_t stream);

/* The off-diagonal nonzeros (columns ascending) at edge_ptr.  Ordered on `stream`. */
int32_t rbg_cc_dag_edges(int64_t n, const int64_t *indptr, const int32_t *indices, const int32_t *data,
                         const int64_t *edge_ptr, int32_t *edge_col, int32_t *edge_val, rbg_stream_t stream);

/* Per component c (comp_kind[c]: 1 entries below the diagonal, 2 above, 0 skip): top_msb[c] =
 * the largest MSB of the products the sequential loop performs (a component with top_msb >= 31
 * may overflow and must take the dense path), first_msb[c] = the largest MSB of any cell's
 * first value (the Floyd-Warshall diameter; -1 when there is none), comp_max[c] = the largest
 * final value, floored at 0 (the 'D' method's diameter source).  `edges` is a device CSR matrix
 * of n rows (int32 values); the closure rows are rbg_dag_closure's row pool as it left it
 * (row_off, row_len, pool_cols, pool_vals).  Ordered on `stream`. */
int32_t rbg_cc_dag_stats(int64_t n, int64_t ncomp, const int32_t *label, const int32_t *local,
                         const int64_t *start, const int32_t *sorted_vertex, const int32_t *comp_kind,
                         const rbg_csr_t *edges, const int64_t *row_off, const int32_t *row_len,
                         const int32_t *pool_cols, const int32_t *pool_vals, const int32_t *diag,
                         int32_t *top_msb, int32_t *first_msb, int32_t *comp_max, rbg_stream_t stream);

/* Row pointers (device, n + 1) of the merged matrix: each closure row (row_len from the row
 * pool) plus its diagonal value when nonzero; *nnz (host) its size.  Synchronises `stream`. */
int32_t rbg_cc_dag_merge_count(int64_t n, const int32_t *row_len, const int32_t *diag, void *workspace,
                               int64_t workspace_bytes, int64_t *out_indptr, int64_t *nnz, rbg_stream_t stream);

/* The merged matrix's columns (ascending) and values, from the row pool.  Ordered on `stream`. */
int32_t rbg_cc_dag_merge_fill(int64_t n, const int64_t *row_off, const int32_t *row_len,
                              const int32_t *pool_cols, const int32_t *pool_vals, const int32_t *diag,
                              const int64_t *out_indptr, int32_t *out_indices, int32_t *out_data,
                              rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Relationship lookups on resident closures (redblackgraph/reference/calc_relationship.py:54-71).
 * ---------------------------------------------------------------------------------------- */
typedef struct rbg_lookup_t {
    const void *W;     /* device: closed matrix, row-major, leading dimension ld (elements) */
    int64_t ld;
    int64_t rows;      /* rows of W (u and v must be below) */
    int64_t n;         /* row length (columns searched) */
    int64_t u, v;      /* the two vertices (rows) */
    int32_t dtype;     /* RBG_DTYPE_* of W */
    int32_t reserved;
} rbg_lookup_t;

/*
 * For every query (a device array of `count` rbg_lookup_t), the common ancestor of u and v:
 * the first j minimising W[u][j] + W[v][j] over the j where both are non-zero, the sum wrapping
 * in W's type as numpy scalar arithmetic does on the reference's rows.  out (device, 3 int64
 * per query) receives j (-1: no relationship; -2: invalid query), W[u][j], W[v][j] (the value
 * bits, to be read back in the matrix's dtype).  The relationship name is formed from the two
 * values on the host (lookup_relationship, calc_relationship.py:23-51).  Ordered on `stream`,
 * no synchronisation.
 */
int32_t rbg_relationship_lookup(int64_t count, const rbg_lookup_t *queries, int64_t *out,
                                rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Relational composition: the closure of a closed graph after adding one vertex or one edge,
 * without recomputing the closure (replaces the C core gufuncs vertex_relational_composition
 * and edge_relational_composition, redblackgraph/core/src/redblackgraph/
 * relational_composition.c.in:72-262, and with RBG_MODE_CYTHON their Cython counterparts,
 * redblackgraph/sparse/csgraph/_relational_composition.pyx:10-113, int32 only).
 * ---------------------------------------------------------------------------------------- */
typedef struct rbg_compose_result {
    int32_t status;   /* RBG_OK; RBG_ERR_OVERFLOW (a product overflowed, or would make the
                         reference's MSB loop run forever: RBG_EV_HANG in `event`);
                         RBG_ERR_CYCLE (vertex composition: the new vertex closes a cycle)    */
    uint32_t flags;   /* RBG_EV_* over every product                                        */
    uint32_t event;   /* RBG_EV_* of the deciding product (RBG_ERR_OVERFLOW)                */
    int32_t reserved;
    int64_t step;     /* reference loop of the deciding event: 1 (u (x) R), 2 (R (x) v; edge:
                         the update), 3 (the cycle check), 4 (vertex update); -1 when OK     */
    int64_t i, j;     /* its row and column (step 3: i = the vertex index k)                */
    int64_t lhs, rhs; /* its operands (step 3: u_k, v_k), value bits widened from the type  */
    int64_t updated;  /* entries in the updated rectangle                                   */
} rbg_compose_result_t;

/* Scratch bytes rbg_vertex_compose / rbg_edge_compose need for an n x n closure. */
int32_t rbg_compose_workspace_bytes(int32_t dtype, int64_t n, int64_t *bytes);

/*
 * R_lambda = the closure of closed R (n x n, leading dimension ldr, `dtype`) with a new vertex:
 * u (its row, n values), v (its column, n values), colour `color`.  out is (n + 1) x (n + 1)
 * with leading dimension ldo >= n + 1; out == R (same ld) updates in place, touching only the
 * rows reaching the new vertex x the columns it reaches, plus row and column n (the buffer must
 * have n + 1 rows).  res->status is what the reference raises: OverflowError for
 * RBG_ERR_OVERFLOW, ValueError ("would result in a cycle", index res->i, values res->lhs /
 * res->rhs) for RBG_ERR_CYCLE.  Synchronises `stream`.
 */
int32_t rbg_vertex_compose(int32_t dtype, int64_t n, const void *R, int64_t ldr, const void *u, const void *v,
                           int64_t color, void *out, int64_t ldo, uint32_t mode, void *workspace,
                           int64_t workspace_bytes, rbg_compose_result_t *res, rbg_stream_t stream);

/*
 * R' = the closure of closed R (n x n) with the edge alpha -> beta of value `relationship`: row
 * alpha becomes (row alpha with column beta replaced) (x) R, and every row reaching alpha takes
 * the update.  out (n x n, ldo) may be R (in place).  The caller checks R[beta][alpha] == 0
 * first (a cycle), as the reference's Python layer does.  Synchronises `stream`.
 */
int32_t rbg_edge_compose(int32_t dtype, int64_t n, const void *R, int64_t ldr, int64_t alpha, int64_t beta,
                         int64_t relationship, void *out, int64_t ldo, uint32_t mode, void *workspace,
                         int64_t workspace_bytes, rbg_compose_result_t *res, rbg_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Orderings of closed graphs (replace _ordering.pyx:15-177, _permutation.pyx:11-205 and
 * _topological_sort.pyx:30-265 of redblackgraph/sparse/csgraph).  int32 values, int32 indices.
 * ---------------------------------------------------------------------------------------- */

/* Per vertex: anc = sum of the Cython MSB of the row's non-zero values, maxrel = the largest
 * value in the vertex's column (starting from 0), diag = the diagonal value (the row's last
 * diagonal entry, 0 when none).  Device arrays of n.  Ordered on `stream`. */
int32_t rbg_ordering_metrics_csr(int64_t n, const int64_t *indptr, const int32_t *indices, const int32_t *data,
                                 int64_t *anc, int32_t *maxrel, int32_t *diag, rbg_stream_t stream);
int32_t rbg_ordering_metrics_dense(int64_t n, const int32_t *A, int64_t lda, int64_t *anc, int32_t *maxrel,
                                   int32_t *diag, rbg_stream_t stream);

int32_t rbg_canonical_permutation_workspace_bytes(int64_t n, int64_t *bytes);

/* The canonical permutation perm (perm[new] = old): vertices sorted by (size of their component
 * descending, component id ascending, anc descending, maxrel ascending, diag descending, vertex
 * id ascending).  label[v] = component of v, comp_start[c + 1] - comp_start[c] = its size
 * (rbg_cc_label's outputs).  Ordered on `stream`. */
int32_t rbg_canonical_permutation(int64_t n, const int32_t *label, const int64_t *comp_start, const int64_t *anc,
                                  const int32_t *maxrel, const int32_t *diag, int32_t *perm, void *workspace,
                                  int64_t workspace_bytes, rbg_stream_t stream);

/* B[i][j] = A[perm[i]][perm[j]] (upper != 0: only j >= i, zeros below).  A != B. */
int32_t rbg_permute_dense(int32_t dtype, int64_t n, const void *A, int64_t lda, const int32_t *perm, void *B,
                          int64_t ldb, int32_t upper, rbg_stream_t stream);

int32_t rbg_permute_csr_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes);
/* Row i of the result = row perm[i] of A with columns mapped through the inverse permutation
 * (upper != 0 keeps new columns >= i), columns ascending.  count writes indptr_out (n + 1) and
 * *nnz_out (host); fill writes indices and data (int32).  Same workspace for both calls. */
int32_t rbg_permute_csr_count(const rbg_csr_t *A, const int32_t *perm, int32_t upper, int64_t *indptr_out,
                              void *workspace, int64_t workspace_bytes, int64_t *nnz_out, rbg_stream_t stream);
int32_t rbg_permute_csr_fill(const rbg_csr_t *A, const int32_t *perm, int32_t upper, const int64_t *indptr_out,
                             int32_t *indices_out, int32_t *data_out, void *workspace, int64_t workspace_bytes,
                             rbg_stream_t stream);

int32_t rbg_topological_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes);
/* A topological permutation (perm[new] = old) after which every stored entry (v, w), w != v,
 * lies above the diagonal: vertices by Kahn level, deepest first, vertex id ascending within a
 * level.  *levels = number of levels.  RBG_ERR_CYCLE with *cycle_vertex = a vertex on a cycle.
 * Synchronises `stream`. */
int32_t rbg_topological_order(const rbg_csr_t *A, void *workspace, int64_t workspace_bytes, int32_t *perm,
                              int64_t *levels, int64_t *cycle_vertex, rbg_stream_t stream);

/* *result = 1 when no stored entry lies below the diagonal (strict: on or below).  workspace >=
 * 4 bytes.  Synchronises `stream`. */
int32_t rbg_is_upper_triangular_csr(const rbg_csr_t *A, int32_t strict, int32_t *result, void *workspace,
                                    int64_t workspace_bytes, rbg_stream_t stream);

/* Row/column remap of an int32 CSR (replaces extract_submatrix and merge_component_matrices,
 * redblackgraph/sparse/csgraph/_components.pyx:178-323): output row row_map[k] (-1: dropped)
 * receives input row k, its columns mapped through col_map (-1: dropped), columns ascending;
 * each output row receives at most one input row.  Writes indptr_out (n_out + 1) and *nnz_out;
 * RBG_ERR_CAPACITY when *nnz_out > capacity (indices/data untouched: call again with room).
 * Synchronises `stream`. */
int32_t rbg_csr_remap_workspace_bytes(int64_t n_out, int64_t nnz, int64_t *bytes);
int32_t rbg_csr_remap(const rbg_csr_t *A, const int32_t *row_map, const int32_t *col_map, int64_t n_out,
                      int64_t *indptr_out, int32_t *indices_out, int32_t *data_out, int64_t capacity, void *workspace,
                      int64_t workspace_bytes, int64_t *nnz_out, rbg_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* RBG_GB300_H */
