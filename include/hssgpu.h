/*
 * hssgpu.h -- C ABI of the GB300 (sm_103a) HSS hot path.
 *
 * The library holds an HSS matrix's generator tree (D, U, V, R, W, B) on one
 * GPU as packed FP64 arrays with level-ordered task lists, and runs:
 *   - the HSS x dense product      (reference: src/matmul.jl:13-62,
 *                                   `*(hssA, B)` :13, `mul!(C, hssA, B, a, b)` :18),
 *   - the implicit ULV factorization and solve, split into a resident
 *     factorization and a solve      (reference: src/ulvfactor.jl:10-107,
 *                                   `ulvfactsolve` :10, reached by `hssA \ B`,
 *                                   src/hssmatrix.jl:234; factor-only
 *                                   reduction src/ulvdivide.jl:58-85),
 *   - FP32 factorization + FP64 iterative refinement (new; same API),
 *   - batched forests of independent matrices, and the sampling products of
 *     randomized compression (reference: src/compression.jl:278-430).
 *
 * Conventions (mirroring the Julia reference): matrices are column-major
 * with an explicit leading dimension; indices are 0-based here.  Every entry
 * point returns an hss_status; hss_last_error() gives a message.  Device
 * pointers ("d" prefix) must live on the handle's device; "_host" variants
 * take host memory and synchronise.  A handle must not be used from two host
 * threads or two streams at the same time.
 */
#ifndef HSSGPU_H
#define HSSGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  HSS_OK = 0,
  HSS_ERR_BAD_DIMS = 1,       /* DimensionMismatch / ArgumentError in the reference */
  HSS_ERR_OOM = 2,
  HSS_ERR_SINGULAR = 3,       /* root LU hit an exact zero pivot (reference: SingularException) */
  HSS_ERR_NO_CONVERGENCE = 4, /* refinement did not reach the tolerance in maxit steps */
  HSS_ERR_TIMEOUT = 5,
  HSS_ERR_CUDA = 6,
  HSS_ERR_INVALID = 7         /* null handle, bad argument */
} hss_status;

typedef enum { HSS_PREC_FP64 = 0, HSS_PREC_FP32 = 1 } hss_precision;

typedef struct hss_plan_s* hss_handle;
typedef struct hss_factor_s* hss_factor;

/* Node table: one row of HSS_NODE_FIELDS int64 per node, node 0 = root,
 * children after their parent (any order otherwise).  Field meaning:
 *   [0] left child (-1 for a leaf)   [1] right child (-1 for a leaf)
 *   [2] leaf rows m  (branch: 0)     [3] leaf cols n (branch: 0)
 *   [4] ku: columns of U (leaf) or of R1/R2 (branch); 0 at the root
 *   [5] kv: columns of V (leaf) or of W1/W2 (branch); 0 at the root
 *   [6] D  [7] U  [8] V       element offsets into `packed` (leaf)
 *   [9] B12 [10] B21 [11] R1 [12] R2 [13] W1 [14] W2   (branch; -1 if empty)
 *   [15] reserved (0)
 * Block shapes follow the reference's HssMatrix fields (src/hssmatrix.jl:11-67):
 *   D m x n, U m x ku, V n x kv; B12 ku(left) x kv(right), B21 ku(right) x kv(left),
 *   R1 ku(left) x ku, R2 ku(right) x ku, W1 kv(left) x kv, W2 kv(right) x kv.  */
#define HSS_NODE_FIELDS 16

/* Replaces the construction of `HssMatrix` (src/hssmatrix.jl:36-67): uploads a
 * packed generator tree.  Checks the same dimensions as `checkdims`
 * (src/hssmatrix.jl:308-322) and returns HSS_ERR_BAD_DIMS otherwise. */
int hss_create(int64_t nnodes, const int64_t* nodes, const double* packed,
               int64_t npacked, hss_handle* out);

/* A forest of `count` independent matrices sharing one plan (batched form).
 * nnodes[i], nodes[i], packed[i], npacked[i] describe matrix i as above. */
int hss_create_batch(int32_t count, const int64_t* nnodes, const int64_t* const* nodes,
                     const double* const* packed, const int64_t* npacked, hss_handle* out);

/* Host-only validation of one node table (no GPU needed): the same checks as
 * hss_create, and on success the per-node bookkeeping of hss_node_info for
 * every node into info[nnodes * HSS_INFO_FIELDS] (nullable).  Lets a caller
 * validate a tree before uploading it (reference: `checkdims`,
 * src/hssmatrix.jl:308-322). */
int hss_inspect(int64_t nnodes, const int64_t* nodes, int64_t npacked, int64_t* info);

int hss_destroy(hss_handle h);

/* size(hssA) (src/hssmatrix.jl:94) of matrix `tree` of the forest. */
int hss_size(hss_handle h, int32_t tree, int64_t* m, int64_t* n);
int hss_ntrees(hss_handle h, int32_t* count);

/* Per-node bookkeeping for bit-exact checks: fields
 * [0] depth [1] height [2] row0 [3] col0 [4] m [5] n [6] ku [7] kv
 * [8] k [9] mk [10] nk [11] leaf [12] tree  (ULV reduce-problem sizes). */
#define HSS_INFO_FIELDS 13
int hss_node_info(hss_handle h, int64_t node, int64_t* fields);

/* `cols` of node `node` in `_ulvfactsolve!` (src/ulvfactor.jl:62,76), 0-based.
 * Writes at most cap entries, returns the length in *len. */
int hss_ulv_cols(hss_handle h, int64_t node, int64_t* cols, int64_t cap, int64_t* len);

/* mul!(C, hssA, B, alpha, beta) (src/matmul.jl:18-28) on the device.
 * B is n x r (ldb), C is m x r (ldc); stream is a cudaStream_t (NULL = default). */
int hss_matmul(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC,
               int64_t ldc, double alpha, double beta, void* stream);

/* Same, with host B and C; copies in, computes, copies out, synchronises. */
int hss_matmul_host(hss_handle h, const double* B, int64_t ldb, int64_t r, double* C,
                    int64_t ldc, double alpha, double beta);

/* hss_matmul without any memory allocation; no counterpart in the reference.
 * For callers that cannot call cudaMalloc during a call (host callbacks,
 * pre-allocated real-time loops, runtimes that forbid allocation after
 * start-up).  The per-node workspace and the argument table live in fixed
 * file-scope device arrays (8 MiB + one argument slot, held by every GPU that
 * loads the library until the process exits): at most 2^20 doubles of workspace (workspace rows
 * x r; e.g. n = 65536 at rank 32 allows r <= 16), larger calls return
 * HSS_ERR_BAD_DIMS.  The arrays are shared by all calls on a device: calls
 * that overlap on the GPU race; calls on one stream are ordered.  The call
 * makes the handle's device current; the first call on a device resolves the
 * arrays' addresses there (make it before any stream capture).  Same
 * arguments and result as hss_matmul. */
int hss_matmul_noalloc(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC,
                       int64_t ldc, double alpha, double beta, void* stream);

/* Batched product over a forest: matrix i uses dB[i], dC[i], r[i] (device). */
int hss_matmul_batch(hss_handle h, const double* const* dB, const int64_t* ldb,
                     const int64_t* r, double* const* dC, const int64_t* ldc,
                     double alpha, double beta, void* stream);

/* ULV factorization (new entry point: the reference only has the fused
 * `ulvfactsolve`, src/ulvfactor.jl:10; its factor-only reduction is
 * src/ulvdivide.jl:58-85).  precision = HSS_PREC_FP64 or HSS_PREC_FP32.
 * Asynchronous on `stream`; errors surface at the next synchronising call. */
int hss_ulvfactor(hss_handle h, int32_t precision, hss_factor* out, void* stream);
int hss_factor_destroy(hss_factor f);

/* Recompute an existing factorization in place (same plan and precision),
 * e.g. after the generators changed or to re-run without allocating. */
int hss_ulvrefactor(hss_factor f, void* stream);

typedef struct {
  int32_t iterations;      /* refinement steps taken (0 for a plain solve) */
  int32_t converged;       /* 1 if every column reached tol */
  double residual;         /* max over columns of ||b - A x|| / ||b|| (when computed) */
} hss_solve_stats;

/* x = A \ b with the resident factorization (reference semantics of
 * `ulvfactsolve`, src/ulvfactor.jl:10-107).  For an FP32 factor the solve is
 * refined with FP64 HSS products until max_j ||b_j - A x_j|| / ||b_j|| <= tol
 * or maxit steps (HSS_ERR_NO_CONVERGENCE).  For an FP64 factor tol = 0 skips
 * the residual; tol > 0 refines in FP64 the same way.  tol < 0 is a single
 * solve in the factor's precision without any residual.  Device pointers. */
int hss_ulvsolve(hss_factor f, const double* dB, int64_t ldb, int64_t r, double* dX,
                 int64_t ldx, double tol, int32_t maxit, hss_solve_stats* stats,
                 void* stream);
/* Refactor f's plan (its generators may have changed) and solve, in one call:
 * `hssA \ B` (src/hssmatrix.jl:234) as hss_ulvrefactor + hss_ulvsolve, with the
 * first solve's upward sweep of level h started as soon as level h is factored
 * (a second stream, one event per level), so it runs behind the factorization
 * instead of after it.  Same arguments and results as hss_ulvsolve. */
int hss_ulvfactsolve(hss_factor f, const double* dB, int64_t ldb, int64_t r, double* dX, int64_t ldx, double tol,
                     int32_t maxit, hss_solve_stats* stats, void* stream);
int hss_ulvsolve_host(hss_factor f, const double* B, int64_t ldb, int64_t r, double* X,
                      int64_t ldx, double tol, int32_t maxit, hss_solve_stats* stats);

/* Batched solve over a forest factor: matrix i uses dB[i], dX[i], r[i]. */
int hss_ulvsolve_batch(hss_factor f, const double* const* dB, const int64_t* ldb,
                       const int64_t* r, double* const* dX, const int64_t* ldx,
                       double tol, int32_t maxit, hss_solve_stats* stats, void* stream);

/* `hssA \ B` (src/hssmatrix.jl:234 -> src/ulvfactor.jl:10): factor + solve in
 * one call with host buffers. */
int hss_ulvfactsolve_host(hss_handle h, int32_t precision, const double* B, int64_t ldb,
                          int64_t r, double* X, int64_t ldx, double tol, int32_t maxit,
                          hss_solve_stats* stats);

/* Batches over independently created single-tree plans (the serving form):
 * one launch per tree level covers every matrix of the batch.  A batcher owns
 * the merged task lists and per-call buffers; use one batcher per stream. */
typedef struct hss_batcher_s* hss_batcher;
int hss_batcher_create(hss_batcher* out);
int hss_batcher_destroy(hss_batcher b);
/* Factor `count` plans in one set of launches; out[i] receives a new
 * factorization of hs[i] (release with hss_factor_destroy). */
int hss_batcher_factor(hss_batcher b, int32_t count, const hss_handle* hs, int32_t precision,
                       hss_factor* out, void* stream);
/* Solve (and refine, as hss_ulvsolve) distinct factorizations fs[i] of one
 * precision with right-hand sides dB[i] (r[i] columns) into dX[i]. */
int hss_batcher_solve(hss_batcher b, int32_t count, const hss_factor* fs, const double* const* dB,
                      const int64_t* ldb, const int64_t* r, double* const* dX, const int64_t* ldx,
                      double tol, int32_t maxit, hss_solve_stats* stats, void* stream);

/* Device memory held by a factorization (bytes). */
int hss_factor_bytes(hss_factor f, int64_t* bytes);
/* Device memory held now by a handle and / or a factorization (either may be
 * null): generators and their derived copies, node and task tables, factor
 * storage and the workspaces grown by earlier calls (bytes). */
int hss_device_bytes(hss_handle h, hss_factor f, int64_t* bytes);

/* Autotuner (new; the reference has no GPU kernels to choose between).  Times,
 * on scratch right-hand sides with r columns, the two solve kernels of every
 * tree level of this factorization -- a warp per right-hand side ("register")
 * and a block per 32 right-hand sides with GEMM steps ("blocked", FP32 factors)
 * -- and the two refinement residual products (one persistent launch, one
 * launch per level), and keeps the faster per level in the factorization for
 * its later solves (hss_ulvsolve*; a batcher's merged solves use the built-in
 * rule).  Synchronises the stream.  hss_autotune_info reads the choices back:
 * per level 1 blocked, 0 register, -1 not tuned; product 1 persistent, 0 per
 * level, -1 not tuned (arrays of *nup / *ndown entries; null to query sizes). */
int hss_autotune(hss_factor f, int64_t r, void* stream);
int hss_autotune_info(hss_factor f, int32_t* nup, int8_t* up, int32_t* ndown, int8_t* down, int32_t* pmv);

/* Profiling aid: bracket every launch of one kernel kind with CUDA events on
 * its stream (-1 disables), then read the summed device time and the number
 * of launches (hss_trace_end synchronises on the recorded events). */
enum {
  HSS_TRACE_MV_LEAF = 0,      /* leaf D*B and V^T*B          (src/matmul.jl:34,46) */
  HSS_TRACE_MV_UP = 1,        /* W1^T Z1 + W2^T Z2           (src/matmul.jl:39) */
  HSS_TRACE_MV_DOWN = 2,      /* B12 Z2 + R1 F, B21 Z1 + R2 F (src/matmul.jl:50-56) */
  HSS_TRACE_MV_FINAL = 3,     /* leaf C += U F               (src/matmul.jl:47) */
  HSS_TRACE_FACTOR_LEAF = 4,  /* ULV reduction of the leaves (src/ulvfactor.jl:22-57) */
  HSS_TRACE_FACTOR_MERGE = 5, /* merge + reduction per level (src/ulvfactor.jl:74-89) */
  HSS_TRACE_SOLVE_UP = 6,     /* upward solve per level */
  HSS_TRACE_SOLVE_DOWN = 7,   /* Q^T back-application per level (src/ulvfactor.jl:98-107) */
  HSS_TRACE_MV_DX = 8,        /* tensor-core leaf products D X of the refinement residual (src/matmul.jl:46) */
  HSS_TRACE_KINDS = 9
};
int hss_trace_begin(int32_t kind);
int hss_trace_end(double* total_ms, int64_t* launches);
/* Like hss_trace_end, and the device time of every traced launch in launch
 * order (ms[i] for i < cap; *launches is the count, which may exceed cap):
 * per tree level for the level kinds. */
int hss_trace_times(double* ms, int64_t cap, int64_t* launches);

/* Entries of a single-tree handle: out(i, j) = A(rows[i], cols[j]) into the
 * nr x nc device matrix dOut (column-major, ld ldo >= nr), 0-based indices in
 * any order, repeats allowed: `getindex(hssA, i::Vector, j::Vector)`
 * (src/hssmatrix.jl:108-128).  The restricted bases of every node are formed
 * level by level and the off-diagonal blocks in 64 x 64 FP64 tiles.
 * hss_full is `full(hssA)` (:270-305) = all rows and columns. */
int hss_getindex(hss_handle h, const int64_t* rows, int64_t nr, const int64_t* cols, int64_t nc, double* dOut,
                 int64_t ldo, void* stream);
int hss_full(hss_handle h, double* dOut, int64_t ldo, void* stream);

/* C = A * B for two single-tree handles on matching cluster trees (A's column
 * clusters = B's row clusters): `*(hssA::HssMatrix, hssB::HssMatrix)`
 * (src/matmul.jl:65-117), a new handle whose ranks are the sums of the
 * operands' (no recompression).  Upsweep, downsweep and generator assembly
 * run as lists of small FP64 products on the device; the call synchronises
 * `stream`. */
int hss_hssmul(hss_handle a, hss_handle b, hss_handle* out, void* stream);

/* `recompress!(hssA; atol, rtol)` (src/compression.jl:148-260) on the device:
 * orthonormalize the generators (src/generators.jl:64-114), then truncate
 * the couplings top-down, every rank decision a column-pivoted QR on the GPU
 * with `_compress_block!`'s rule (keep |R_ii| > max(atol, rtol |R_11|)).  The
 * result is a new handle; the input is not modified.  hss_orthonormalize is
 * the first half alone.  Both synchronise `stream` once per tree level. */
int hss_recompress(hss_handle h, double atol, double rtol, hss_handle* out, void* stream);
int hss_orthonormalize(hss_handle h, hss_handle* out, void* stream);

/* `adjoint(hssA)` / `transpose(hssA)` for real generators (src/hssmatrix.jl:
 * 165-178) on the device: D^T, U and V exchanged, B12 and B21 exchanged and
 * transposed, R and W exchanged; a new handle with the same node numbering.
 * Synchronises `stream`. */
int hss_transpose(hss_handle h, hss_handle* out, void* stream);

/* C = alpha A^T B + beta C (dense B, C on the device): the product with the
 * adjoint, for `*(A::AbstractMatrix, hssB)` (src/matmul.jl:14, as
 * (hssB' * A')') and `hssA' * B`.  The adjoint's generators are made on the
 * device at the first call and kept with the handle (twice the generator
 * memory from then on); otherwise as hss_matmul. */
int hss_matmul_t(hss_handle h, const double* dB, int64_t ldb, int64_t r, double* dC, int64_t ldc, double alpha,
                 double beta, void* stream);

/* HSS-valued division (src/ulvdivide.jl:13-252): X = hssA \ hssB (hss_ldiv,
 * `ldiv!`, src/hssmatrix.jl:235) and X = hssB / hssA (hss_rdiv, `rdiv!` =
 * adjoint(hssA' \ hssB'), :237), new handles on B's column (ldiv) or row
 * (rdiv) clusters.  The reference's recursion on the generators: A's leaves
 * reduced by its FP64 ULV factorization, the same transforms applied to B's
 * leaf rows, the remainder B - L Y0 recompressed (atol, rtol) and pruned one
 * level per step, the root block solved, and the solution unpacked back up
 * with recompression at every level.  Memory is O(n k) per level, no dense
 * n x n block is formed.  hssA must be square on matching row and column
 * clusters with square leaves of at most 512 rows; hssB on A's cluster tree.
 * Synchronises `stream` several times per level. */
int hss_ldiv(hss_handle hA, hss_handle hB, double atol, double rtol, hss_handle* out, void* stream);
int hss_rdiv(hss_handle hB, hss_handle hA, double atol, double rtol, hss_handle* out, void* stream);

/* Number of kernels this library has launched in the process so far. */
int64_t hss_launch_counter(void);

/* Process-wide switches.  HSS_OPT_GENERIC_FACTOR = 1 routes every ULV
 * factorization level to the global-memory kernel (used to test the on-chip
 * kernel against it); 0 (default) picks the on-chip kernel where it fits.
 * HSS_OPT_RESIDUAL_FP64 = 1 forms the refinement residual of an FP32 factor
 * with the native FP64 product instead of the default double-float product
 * on the FP32 pipe (~48-bit, made for GB300's low FP64 rate).
 * HSS_OPT_LEVEL_PRODUCT = 1 runs every product with one kernel launch per
 * tree level instead of the default single persistent launch (leaves up to
 * 512 columns, ranks up to 64); used to test the two against each other.
 * HSS_OPT_GRAPHS = 1 replays the per-level launch sequences of factorizations
 * and solve passes issued on a non-default stream as CUDA graphs: the second
 * call with unchanged task lists, buffers and sizes is captured, later ones
 * replay the graph (no capture on the legacy default stream).  A solve with
 * refinement (maxit <= 64) is then one graph: the convergence check runs on
 * the device and sets the condition of a while node around the refinement
 * step, and the host reads the loop's status once.  The "_host" solves run on
 * the plan's own non-blocking stream, ordered after the legacy default stream.
 * HSS_OPT_SAMPLE_DF = 1 computes hss_sample's products in double-float
 * arithmetic on the FP32 pipe (~2^-47 relative per operation instead of
 * FP64's 2^-53, several times faster on GB300; entries of A and X must lie
 * within float's exponent range): the mixed-precision form of the sampling
 * in randcompress.  0 (default): FP64.
 * HSS_OPT_FLAT_PRODUCT = 0 turns off the flat form of the persistent FP64
 * product (1, default: FP64 products of at most 4 columns run it, with every
 * leaf carrying its own chain of translator products and two grid barriers
 * in place of the tree's dependency chain); used to test the two forms
 * against each other.
 * HSS_OPT_POLL_LIMIT = p sets how many times a block of the persistent
 * products polls for ready work before it gives up, records a device status
 * and exits (0: the default, 2^22 polls, i.e. seconds).  The next
 * synchronising call on the plan (hss_matmul_host, hss_ulvsolve* with
 * refinement) returns HSS_ERR_TIMEOUT and clears the plan's counters; the
 * product's result is then undefined, the plan stays usable.  A small value
 * makes the waits run out on purpose (failure-detection tests).  Launch
 * sequences already captured as CUDA graphs keep the limit they were
 * captured with.
 * HSS_OPT_TENSOR_RESIDUAL = 0 turns off the tensor-core leaf products of the
 * double-float refinement residual (1, default: for leaves up to 128 x 128
 * the products D X run as exact bf16 slice products on tcgen05, with FP32
 * accumulation in tensor memory, about 48 significant bits like the rest of
 * the residual; 0: on the FP32 pipe in double-float arithmetic).
 * HSS_OPT_FAIL_ALLOC = k > 0 makes the k-th device allocation of this library
 * from now on fail as out of memory, on the host, before the CUDA driver is
 * called (0 disarms): fault injection for the HSS_ERR_OOM paths.  The call
 * that hits it returns HSS_ERR_OOM and leaves no partial object behind. */
enum {
  HSS_OPT_GENERIC_FACTOR = 1,
  HSS_OPT_RESIDUAL_FP64 = 2,
  HSS_OPT_LEVEL_PRODUCT = 3,
  HSS_OPT_GRAPHS = 4,
  HSS_OPT_SAMPLE_DF = 5,
  HSS_OPT_FLAT_PRODUCT = 6,
  HSS_OPT_POLL_LIMIT = 7,
  HSS_OPT_FAIL_ALLOC = 8,
  HSS_OPT_TENSOR_RESIDUAL = 9
};
int hss_set_option(int32_t option, int64_t value);

const char* hss_last_error(void);
int32_t hss_version(void);

/* ---- randomized compression (reference src/compression.jl:278-444) ----
 *
 * The dense matrix A (m x n, column-major, lda) lives on the device.  The
 * reference's `randcompress(A, rcl, ccl, kest)` (:278) and
 * `randcompress_adaptive(A, rcl, ccl; kest)` (:312) become, on the host:
 * draw Omega_col (n x s), Omega_row (m x s); S_col = A * Omega_col and
 * S_row = A^T * Omega_row with hss_sample; hss_rc_compress; for the adaptive
 * form, test with fresh samples through hss_sample, hss_matmul and hss_sumsq
 * and repeat with more columns (the loop of :330-352). */

/* S = alpha * op(A) * X + beta * S (op(A) = A if trans == 0, A^T if 1):
 * A * Omega and A' * Omega of src/compression.jl:290-291, :326-327, :336-337.
 * X has n (trans 0) or m (trans 1) rows and r columns.  FP64. */
int hss_sample(const double* dA, int64_t lda, int64_t m, int64_t n, int32_t trans, const double* dX, int64_t ldx,
               int64_t r, double* dY, int64_t ldy, double alpha, double beta, void* stream);

/* *out = sum of squares of the m x r device matrix B (the `norm(...)^2` of
 * src/compression.jl:340-341); synchronises `stream`. */
int hss_sumsq(const double* dB, int64_t ldb, int64_t m, int64_t r, double* out, void* stream);

/* Row and column cluster trees, which must be compatible (`compatible`,
 * src/clustertree.jl): one table of nnodes rows of 6 int64 -- left child,
 * right child (-1 for leaves), row range [rlo, rhi), column range [clo, chi),
 * 0-based -- with the root in row 0 covering [0, m) x [0, n). */
typedef struct hss_rc_s* hss_rc;
#define HSS_CLUSTER_FIELDS 6
int hss_rc_create(int64_t nnodes, const int64_t* clusters, hss_rc* out);
int hss_rc_destroy(hss_rc rc);
int hss_rc_size(hss_rc rc, int64_t* m, int64_t* n);

/* `_randcompress!(hss_blkdiag(A, rcl, ccl), A, Scol, Srow, Ocol, Orow, 0, 0,
 * atol, rtol; rootnode = true)` (src/compression.jl:358-430, `_interpolate`
 * :433-444): from the s samples S_col = A * Omega_col (m x s) and
 * S_row = A^T * Omega_row (n x s), builds the HSS approximation of A as a new
 * handle (node numbering = the cluster table's, generators on the device).
 * Rank decisions (QR with column pivoting) are FP64 on the GPU; the call
 * synchronises `stream` once to read the ranks.  Samples are not modified. */
int hss_rc_compress(hss_rc rc, const double* dA, int64_t lda, const double* dScol, int64_t ldscol,
                    const double* dSrow, int64_t ldsrow, const double* dOcol, int64_t ldocol, const double* dOrow,
                    int64_t ldorow, int64_t s, double atol, double rtol, hss_handle* out, void* stream);
/* Ranks of the last hss_rc_compress: 2 per cluster node (column side = U/R
 * rank, row side = V/W rank); 0 for the root. */
int hss_rc_ranks(hss_rc rc, int32_t* ranks);

/* S = op(A) * X for the m x n matrix of rc's clusters (new; the sample
 * products of src/compression.jl:290-291, :336-337 for the mixed-precision
 * form).  With HSS_OPT_SAMPLE_DF set, the part of A outside the diagonal leaf
 * blocks is multiplied in double-float arithmetic and the leaf blocks' part
 * D * X is added in FP64, so that the corrected sample S - D * X that
 * hss_rc_compress forms keeps double-float accuracy relative to itself (the
 * near-diagonal entries of kernel matrices dominate S).  Without the option:
 * hss_sample in FP64. */
int hss_rc_sample(hss_rc rc, const double* dA, int64_t lda, int32_t trans, const double* dX, int64_t ldx, int64_t r,
                  double* dY, int64_t ldy, void* stream);

/* Node table (nnodes x HSS_NODE_FIELDS, the hss_create format) and packed
 * generators of a single-tree handle, e.g. to rebuild the host HssMatrix. */
int hss_export_size(hss_handle h, int64_t* nnodes, int64_t* npacked);
int hss_export(hss_handle h, int64_t* nodes, double* packed);

#ifdef __cplusplus
}
#endif
#endif /* HSSGPU_H */
