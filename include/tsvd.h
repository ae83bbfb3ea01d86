/*
 * tsvd.h — C-ABI of the GB300-native Tree-SVD per-snapshot refresh.
 *
 * One process, one GPU (sm_103a). Every device buffer is owned by the
 * session (or allocated inside a call and freed before it returns); callers
 * pass plain host pointers and sizes, except for the *_device entry points,
 * which take device pointers that stay owned by the caller.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   frPCA(mat_csr*, mat**, mat**, mat**, int k, int q) ............ Code/frpca.c:239,
 *                                                                    Code/matrix_vector_functions_intel_mkl_ext.h:75
 *   mat / mat_csr layouts ........................................ Code/matrix_vector_functions_intel_mkl.h:20-23,
 *                                                                    Code/matrix_vector_functions_intel_mkl_ext.h:22-33
 *   UGraph::inputDynamicGraph / Graph::inputDirectedDynamicGraph .. Code/Graph_dynamic.h:530-605 / :119-238
 *   nodegree_Dense{Undirected,Directed}_Refresh_PPR_initialization  Code/ppr_computation_store_dynamic.h:2035-2121,
 *     (+ _Transpose)                                                 :3811-3898, :4133-4228
 *   nodegree_DenseDynamicForwardPush / ...Directed...(Transpose) .. Code/ppr_computation_store_dynamic.h:1394-1498,
 *                                                                    :2945-3030, :3356-3437
 *   Log_sparse_matrix_entries[_with_norm_computation][_LP] ......... Code/ppr_computation_store_dynamic.h:2527-2561,
 *                                                                    :2598-2638, :2649-2732, :2742-2826
 *   sparse_sub_svd_function_with_norm_computation ................ Code/Tree_u_NC.cpp:75-226
 *   tree merge (dense_sub_svd_function, root U*sqrt(S)) ........... Code/Tree_u_NC.cpp:723-850, :238-262
 *   Tree_{u,d}_{NC,LP} main snapshot loop + CSV output ............ Code/Tree_u_NC.cpp:296-911, Code/Tree_d_NC.cpp:400-1171
 *
 * Conventions: every call returns tsvd_status; a failing call leaves a
 * message readable through tsvd_last_error() (thread-local). A session is
 * not thread-safe: one caller at a time.
 */
#ifndef TSVD_H
#define TSVD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tsvd_status {
  TSVD_OK = 0,
  TSVD_ERR_INVALID = 1,   /* bad argument or size */
  TSVD_ERR_OOM = 2,       /* device or pinned-host allocation failed */
  TSVD_ERR_DEVICE = 3,    /* CUDA runtime error (message in tsvd_last_error) */
  TSVD_ERR_TIMEOUT = 4,   /* a bounded device loop gave up (status flag set by a kernel) */
  TSVD_ERR_STATE = 5,     /* call out of order (e.g. embedding before the first step) */
  TSVD_ERR_IO = 6,        /* file could not be read or written */
  TSVD_ERR_NUMERIC = 7    /* non-finite value detected in a factor */
} tsvd_status;

const char *tsvd_status_string(tsvd_status s);
const char *tsvd_last_error(void);
/* Build identification string ("tsvd-gb300 sm_103a ..."). */
const char *tsvd_version(void);
/* Number of kernels this library has launched in the process so far. */
int64_t tsvd_launch_count(void);

/* ------------------------------------------------------------------------- */
/* Legacy drop-in types and frPCA (same memory layout as the reference).      */
/* ------------------------------------------------------------------------- */
#ifndef TSVD_NO_LEGACY
/* Column-major dense matrix. Code/matrix_vector_functions_intel_mkl.h:20-23 */
typedef struct {
  int nrows, ncols;
  double *d;
} mat;

/* 1-based CSR with begin/end row pointers.
 * Code/matrix_vector_functions_intel_mkl_ext.h:22-33 */
typedef struct {
  int nnz;
  int nrows, ncols;
  double *values;
  int *cols;
  int *pointerB, *pointerE;
} mat_csr;

/* Drop-in for frPCA (Code/frpca.c:239-326): randomized SVD of A with
 * oversampling 5 and q passes over A. *U (nrows x k), *S (k x 1) and
 * *V (ncols x k) are preallocated by the caller as in
 * Code/Tree_u_NC.cpp:139-142 and are overwritten. Singular values come
 * back in ascending order, like the reference (dsyevd order, frpca.c:298-310).
 * The Gaussian test matrix comes from the counter-based generator seeded by
 * tsvd_set_frpca_seed() (the reference seeds MKL VSL with time(NULL)). The
 * caller's double values are rounded to float and both products run as FP32
 * SpMM on the GPU (tsvd_frpca_fp32); the small solves are fp32 with fp64
 * Grams and an fp64-refined eigen-solve, so results match the reference's
 * FP64 frPCA to about 1e-6 relative in the leading singular values, not to
 * double precision.
 * Errors are reported through tsvd_last_error(); the legacy signature has no
 * return value, and on error the outputs are left zero-filled. */
void frPCA(mat_csr *A, mat **U, mat **S, mat **V, int k, int q);
#endif

void tsvd_set_frpca_seed(uint64_t seed);

/* Status-returning frPCA over a host CSR (0- or 1-based, int64 row_ptr of
 * nrows+1 entries). U: nrows x k, V: ncols x k (both column-major, like
 * `mat`), S: k values in DESCENDING order. Any of U, S, V may be NULL.
 * Replaces Code/frpca.c:239 for callers that want status codes and a seed. */
tsvd_status tsvd_frpca(int32_t nrows, int32_t ncols, int64_t nnz,
                       const int64_t *row_ptr, const int32_t *col_idx,
                       const double *values, int32_t index_base, int32_t k,
                       int32_t q, uint64_t seed, double *U, double *S,
                       double *V);

/* Same arguments and outputs as tsvd_frpca, with the matrix kept in FP32 (a
 * CSR / CSC pair of the non-empty columns, values rounded from double to
 * float) and both products of every pass run as FP32 SpMM, as in the plain
 * GPU form. tsvd_frpca rounds the values to half precision (relative 2^-11)
 * for the tensor-core products. The legacy frPCA symbol uses this path.
 * Replaces Code/frpca.c:239 (products: csr_matrix_{,transpose_}matrix_mult,
 * Code/matrix_vector_functions_intel_mkl_ext.c:364-398). */
tsvd_status tsvd_frpca_fp32(int32_t nrows, int32_t ncols, int64_t nnz,
                            const int64_t *row_ptr, const int32_t *col_idx,
                            const double *values, int32_t index_base, int32_t k,
                            int32_t q, uint64_t seed, double *U, double *S,
                            double *V);

/* Same computation and arguments as tsvd_frpca, but it allocates nothing.
 * No counterpart in the reference. For callers that cannot call cudaMalloc:
 * plug-ins inside a host application that reserves the device memory pool
 * for its own allocator, and latency-bound host loops that must stay off the
 * allocator (cudaMalloc/cudaFree can synchronize the device). All device
 * scratch is one static array of about 11 MB that every GPU loading this
 * library keeps until process exit; host staging is static too. Limits:
 * nrows <= 512, ncols <= 16384, <= 2048 non-empty columns, nnz <= 262144,
 * k <= 64, |values| <= FLT_MAX; larger inputs return TSVD_ERR_INVALID. The
 * call is synchronous: it runs on the legacy default stream (ordered with
 * the caller's blocking streams), reads a count back to the host midway and
 * returns with the results in U, S, V. The first call on a device resolves
 * the array's address (make it before any stream capture). Calls share the
 * array, so calls that overlap on the GPU race. */
tsvd_status tsvd_frpca_noalloc(int32_t nrows, int32_t ncols, int64_t nnz,
                               const int64_t *row_ptr, const int32_t *col_idx,
                               const double *values, int32_t index_base,
                               int32_t k, int32_t q, uint64_t seed, double *U,
                               double *S, double *V);

/* The tree merge's SVD on one dense matrix: replaces dense_sub_svd_function
 * (Code/Tree_u_NC.cpp:238-262) over truncated_singular_value_decomposition
 * (Code/matrix_vector_functions_intel_mkl.c:1259-1300). M: rows x cols,
 * column-major (the reference's mat); US (rows x d, column-major) = U_d
 * diag(s_d), sigma: s_d descending. d <= min(rows, cols, 144), cols <= 2048.
 * Host pointers; device memory is allocated and freed inside the call. */
tsvd_status tsvd_merge_svd(int32_t rows, int32_t cols, const double *M, int32_t d, double *US,
                           double *sigma);

/* ------------------------------------------------------------------------- */
/* Session: device graph store + PPR store + block factors + merge tree.      */
/* ------------------------------------------------------------------------- */
typedef struct tsvd_session tsvd_session;

enum {
  /* Log transform of the proximity x (Code/ppr_computation_store_dynamic.h): */
  TSVD_TRANSFORM_LOG10_NC = 0, /* x > rmin ? log10(x/rmin) : 0      (:2549-2556) */
  TSVD_TRANSFORM_LOG10_LP = 1, /* log10(1 + x/rmin) on stored x     (:2621-2632) */
  TSVD_TRANSFORM_LN_N = 2      /* max(0, ln(x * N))                                */
};

enum {
  /* Block-recompute rule once iter >= lazy_update_start_iter. */
  TSVD_DIRTY_REFERENCE = 0, /* resid + ||A-A_old||_F >= sqrt(2)*delta*||A||_F   (:2707-2711) */
  TSVD_DIRTY_FROBENIUS = 1, /* ||A-A_old||_F > dirty_frac * ||A||_F                           */
  TSVD_DIRTY_ALL = 2        /* every block, every snapshot                                  */
};

enum {
  TSVD_ROOT_SQRT_SIGMA = 0, /* U * sqrt(|S|)  (Tree_u_NC.cpp:765-772)  */
  TSVD_ROOT_U = 1           /* U              (Tree_u_LP.cpp root)    */
};

enum {
  /* Refresh arithmetic for a new adjacency slot j of vertex u. */
  TSVD_REFRESH_EXACT = 0, /* p *= (j+1)/j in double (ppr:6520-6522, the sparse path)        */
  TSVD_REFRESH_INTDIV = 1 /* p *= (j+1)/j in int   (ppr:2102, 3875, 4203, the dense path)  */
};

enum {
  /* How tsvd_session_step computes a snapshot. Both give the same results
   * within the parity tolerances and leave the same state behind, so a
   * session may switch between them (tsvd_session_set_form). */
  TSVD_FORM_MIXED = 0, /* 64-source residue runs (one 256-byte vector atomic per       */
                       /* neighbour), dirty blocks batched per stage, products on the  */
                       /* tensor cores with half-precision A^T and hi+lo skinny        */
                       /* operands                                                     */
  TSVD_FORM_PLAIN = 1  /* the plain GPU form: one frontier entry and one scalar atomic */
                       /* per (vertex, source) cell with fp64 push arithmetic; every   */
                       /* dirty block factorized on its own with FP32 CSR SpMM; one    */
                       /* merge launch sequence per tree node                          */
};

enum {
  /* Product path of the mixed form's block frPCA (the plain form always uses
   * FP32 CSR SpMM, one block at a time). */
  TSVD_BLOCKS_DENSE = 0,  /* half-precision A^T of the block's non-empty columns,     */
                          /* tensor-core products, all dirty blocks in one batch      */
  TSVD_BLOCKS_SPARSE = 1, /* FP32 CSR / CSC of every dirty block, SpMM products in    */
                          /* one batch                                                */
  TSVD_BLOCKS_AUTO = 2    /* per block, by density: at the first factorization both   */
                          /* paths are timed on sample blocks of different density    */
                          /* and a cost model (dense: per stored cell; sparse: per    */
                          /* non-zero and per stored cell of the build) gives the     */
                          /* density below which a block takes the SpMM path; each    */
                          /* snapshot then runs one dense and one sparse batch        */
};

typedef struct tsvd_config {
  int32_t n_vertices;       /* N (argv[9] of the reference drivers)                  */
  int32_t directed;         /* 0: UGraph (Tree_u_*), 1: Graph + transpose (Tree_d_*)  */
  int32_t n_sources;        /* |S|                                                   */
  const int32_t *sources;   /* |S| vertex ids, row order of the embedding            */
  double alpha;             /* argv[3]                                               */
  double rmax;              /* argv[5]: residuemax == reservemin                     */
  int32_t n_parts;          /* argv[7]: column blocks                                */
  int32_t hierarchy_n;      /* argv[8]: merge arity h (n_parts must be a power of h) */
  int32_t rank_d;           /* d (128 in the reference, Tree_u_NC.cpp:357)           */
  int32_t oversample;       /* s (5 in the reference, frpca.c:242)                   */
  int32_t passes_q;         /* argv[4]: q                                            */
  int32_t dynamic_ppr_start_iter; /* argv[10]                                        */
  int32_t lazy_update_start_iter; /* argv[11]                                        */
  double delta;             /* argv[12]                                              */
  int32_t transform;        /* TSVD_TRANSFORM_*                                      */
  int32_t dirty_rule;       /* TSVD_DIRTY_*                                          */
  double dirty_frac;        /* for TSVD_DIRTY_FROBENIUS                              */
  int32_t root_scaling;     /* TSVD_ROOT_*                                           */
  int32_t refresh_mode;     /* TSVD_REFRESH_*                                        */
  uint64_t seed;            /* Gaussian test matrices                                */
  int32_t device;           /* CUDA device ordinal                                   */
  int32_t max_push_rounds;  /* bound on frontier rounds per push (0 = default)       */
  int32_t push_levels;      /* threshold schedule: push r > rmax*ratio^k, k = L-1..0  */
  double push_ratio;        /* (1 level = the plain rmax test)                      */
  double push_cofrac;       /* co-push residues > rmax*cofrac on runs being pushed   */
                            /* (default 0.85; 1 = plain rmax test only)              */
  int32_t lp_right_factor;  /* 1: after every snapshot, V_b = A_b^T U for each block  */
                            /* refreshed in it (LP drivers; needs TSVD_ROOT_U)        */
  int32_t ppr_host_reserve; /* 1: the reserve p (half of the PPR state) lives in     */
                            /* pinned host memory, read and written by the kernels    */
                            /* over NVLink-C2C; the residues stay in HBM. For graphs  */
                            /* whose 16 N Sp bytes of state exceed HBM (N 6.2M,       */
                            /* |S| 3000: 305 GB)                                      */
  int32_t form;             /* TSVD_FORM_*: how a snapshot is computed (see below)   */
  int32_t block_path;       /* TSVD_BLOCKS_*: product path of the mixed form's frPCA */
  int32_t plain_frontier_cap; /* plain form: entries of its frontier list (0: 2^26);  */
                            /* cells beyond it wait in the touched bitset for the    */
                            /* next round                                            */
  int32_t push_hub_degree;  /* > 0: the push_levels schedule holds back only         */
                            /* vertices of at least this degree (a hub waits until   */
                            /* its residue reaches rmax*ratio^k, while the rest push */
                            /* at rmax); 0: it applies to every vertex               */
} tsvd_config;

/* Fills the reference's defaults (Tree_u_NC, run.sh: alpha .5, q 12, ...). */
void tsvd_config_default(tsvd_config *cfg);

tsvd_status tsvd_session_create(const tsvd_config *cfg, tsvd_session **out);
/* Estimated device bytes of a session with this configuration once
 * expected_edges pairs are inserted (no counterpart in the reference; the
 * serving layer admits tenants by it). */
tsvd_status tsvd_session_footprint(const tsvd_config *cfg, int64_t expected_edges,
                                   int64_t *bytes);
tsvd_status tsvd_session_destroy(tsvd_session *s);

/* One snapshot (one iteration of the driver loop, Tree_u_NC.cpp:507-866):
 * insert the edges (a delta file's worth), refresh + push PPR, log-transform
 * and test every block, factorize dirty blocks, merge dirty ancestors.
 * `edges` holds m (from, to) pairs of int32, host memory. */
tsvd_status tsvd_session_step(tsvd_session *s, const int32_t *edges, int64_t m);
/* Same, with the pairs already in device memory (owned by the caller). */
tsvd_status tsvd_session_step_device(tsvd_session *s, const int32_t *edges_dev,
                                     int64_t m);
/* Current embedding, |S| x d, row-major doubles (row i = sources[i]). */
tsvd_status tsvd_session_embedding(tsvd_session *s, double *out);
/* Device pointer to the current embedding (|S| x d row-major float), valid
 * until the next step. */
tsvd_status tsvd_session_embedding_device(tsvd_session *s, const float **out);

/* Switches the form of the following snapshots (TSVD_FORM_*). The plain form
 * runs one snapshot per call: tsvd_session_run refuses it. */
tsvd_status tsvd_session_set_form(tsvd_session *s, int32_t form);

/* The session's CUDA stream (cudaStream_t), for callers that order their own
 * work or timing events against the session's kernels. */
tsvd_status tsvd_session_stream(tsvd_session *s, void **stream);

typedef struct tsvd_step_stats {
  int32_t iter;
  int32_t skipped;          /* 1 when the driver's lazy skip rule fired          */
  int64_t edges_inserted;
  int64_t push_rounds;      /* frontier rounds (both directions)                */
  int64_t pushes;           /* (vertex, source) pushes executed                 */
  int64_t push_edge_updates;/* sum of deg(v) over pushes                        */
  int32_t dirty_blocks;
  int32_t factorized_blocks;
  int32_t merged_nodes;
  double ms_insert, ms_refresh, ms_push, ms_log, ms_frpca, ms_merge, ms_total;
  int64_t push_items;       /* (vertex, 64-source chunk) items pushed             */
  double ms_push_kernels;   /* device time of the push scatter kernels            */
  double ms_materialize_kernel; /* device time of the block materialization      */
  int64_t push_item_edges;  /* sum of deg(v) over pushed items (neighbour-list reads) */
  double ms_lp;             /* LP right factor of the refreshed blocks            */
  int32_t eig_sweeps_frpca; /* Jacobi sweeps of the blocks' eigSVD (max)          */
  int32_t eig_sweeps_merge; /* Jacobi sweeps of the merges (max over levels)      */
  int32_t merge_subspace_iters; /* subspace iterations of merges wider than 256  */
                            /* columns (max over levels; 0 for narrow merges)    */
  int32_t eig_refine_sweeps;/* sweeps of the fp64 refinement Jacobi (max, all     */
                            /* eigen-solves of the snapshot)                     */
  int32_t sparse_blocks;    /* blocks factorized through FP32 CSR SpMM            */
  double tune_density;      /* TSVD_BLOCKS_AUTO: density below which a block takes */
                            /* the SpMM path (0 before the first factorization)  */
} tsvd_step_stats;
tsvd_status tsvd_session_last_stats(tsvd_session *s, tsvd_step_stats *out);

/* The driver loop over `count` snapshots (Tree_u_NC.cpp:507-911 without the
 * file reads): snapshot k is the pairs [offsets[k], offsets[k+1]) of `edges`
 * (offsets: count + 1 pair indices, host memory). Each snapshot does what
 * tsvd_session_step does, but the factor stage of snapshot k (frPCA of the
 * dirty blocks, merge, LP right factor) runs on a second thread and stream
 * while snapshot k+1 is inserted, refreshed, pushed and materialized.
 * embeddings (optional, host): count x |S| x d doubles, snapshot k's
 * embedding at k * |S| * d (zeros before the first one). stats (optional):
 * count entries; ms_total is the snapshot's latency, from the start of its
 * insert to the end of its factor stage. Returns after the last snapshot is
 * complete; tsvd_session_last_stats then reports the last snapshot. */
tsvd_status tsvd_session_run(tsvd_session *s, const int32_t *edges, const int64_t *offsets,
                             int32_t count, double *embeddings, tsvd_step_stats *stats);
/* Same, with `edges` in device memory (owned by the caller). */
tsvd_status tsvd_session_run_device(tsvd_session *s, const int32_t *edges_dev,
                                    const int64_t *offsets, int32_t count, double *embeddings,
                                    tsvd_step_stats *stats);

/* ---- link prediction (LP drivers) ---------------------------------------
 * Replaces mkl_right_matrix_multiplication_without_norm
 * (Code/Tree_u_LP.cpp:291-407; Tree_d_LP.cpp) and the scoring loop of the LP
 * drivers (Tree_u_LP.cpp:1046-1122; degree-scaled variant
 * ppr_computation_store_dynamic.h:7600-7779). With cfg.lp_right_factor, every
 * snapshot computes V_b = A_b^T U for each block refreshed in it, with U the
 * root factor of that snapshot, and keeps that U beside V_b; blocks that are
 * not refreshed keep both (the reference's left_matrix_U_cache). */

/* V: n_vertices x rank_d row-major (host). Rows of vertices whose block was
 * never refreshed, or whose column never held a non-zero, are zero. */
tsvd_status tsvd_lp_right_factor(tsvd_session *s, float *v_out);
/* score[k] = U_b[row(i)] . V[j] for the pair (i, j) = (pairs[2k], pairs[2k+1]),
 * i a source, b the block of j, U_b the root factor V_b was computed with;
 * times outdeg(i) * indeg(j) (deg(i) * deg(j) undirected) if degree_scaled. */
tsvd_status tsvd_lp_scores(tsvd_session *s, const int32_t *pairs, int64_t m,
                           int32_t degree_scaled, double *scores);
/* Fraction of positives among the k highest scores (ties: lower index first);
 * Tree_u_LP.cpp:1104-1122 with k = sample_m. */
tsvd_status tsvd_lp_precision(const double *scores, const uint8_t *positive, int64_t m,
                              int64_t k, double *precision);

/* ---- granular PPR-store interface (the reference's thread entry points) --- */
/* a1: append edges to the device adjacency (both directions for undirected,
 * out- and in-lists for directed); records former degrees. */
tsvd_status tsvd_graph_insert(tsvd_session *s, const int32_t *edges, int64_t m);
/* a3: refresh for snapshot `iter` (from scratch when iter <
 * dynamic_ppr_start_iter, else the residual perturbation of the new slots).
 * `transpose` selects the in-edge (reverse) PPR of a directed graph. */
tsvd_status tsvd_ppr_refresh(tsvd_session *s, int32_t iter, int32_t transpose);
/* a4: frontier push until every eligible residual is <= rmax. */
tsvd_status tsvd_ppr_push(tsvd_session *s, int32_t transpose);
/* a5/a6: log transform, norms and dirty test for every block; dirty[b] = 1
 * for blocks to refactorize (host array of n_parts bytes, may be NULL). */
tsvd_status tsvd_blocks_materialize(tsvd_session *s, int32_t iter,
                                    uint8_t *dirty);
/* a7/a8: frPCA of the dirty blocks, leaf factors B = U*diag(S), residuals. */
tsvd_status tsvd_blocks_factorize(tsvd_session *s, int32_t iter);
/* a9: merge the ancestors of refactorized leaves; writes the embedding. */
tsvd_status tsvd_tree_merge(tsvd_session *s);

/* ---- inspection (host copies; for tests and tools) ---- */
/* Degrees (n_vertices int32 each; former = before the last insert). dir: 0 out/undirected, 1 in. */
tsvd_status tsvd_graph_degrees(tsvd_session *s, int32_t dir, int32_t *deg,
                               int32_t *former_deg);
/* Adjacency in insertion order: offsets (N+1, int64) and neighbours. */
tsvd_status tsvd_graph_adjacency(tsvd_session *s, int32_t dir, int64_t *offsets,
                                 int32_t *nbrs, int64_t nbrs_capacity);
/* PPR state as |S| x N row-major float: which = 0 residue, 1 reserve. */
tsvd_status tsvd_ppr_state(tsvd_session *s, int32_t transpose, int32_t which,
                           float *out);
/* The same for the listed source rows only (count x N row-major float; row i
 * = source index rows[i]), for sampled checks of large sessions. */
tsvd_status tsvd_ppr_state_rows(tsvd_session *s, int32_t transpose, int32_t which,
                                const int32_t *rows, int32_t count, float *out);
/* Per-block numbers: ||A||_F, ||A-A_old||_F, residual, nnz(A), dirty flag. */
tsvd_status tsvd_block_info(tsvd_session *s, double *norm_a, double *norm_diff,
                            double *resid, int64_t *nnz, uint8_t *dirty);
/* Tree node factor (|S| x d row-major doubles) and its singular values (d). */
tsvd_status tsvd_tree_factor(tsvd_session *s, int32_t node, double *out,
                             double *sigma);
/* Dense log-transformed block b as |S| x n_b row-major float (tests). */
tsvd_status tsvd_block_dense(tsvd_session *s, int32_t b, float *out);

/* ------------------------------------------------------------------------- */
/* Serving: many tenants on one GPU, requests taken as they arrive.            */
/* No counterpart in the reference (its drivers refresh one graph from a list  */
/* of delta files). A tenant is one session; it is admitted when its          */
/* estimated footprint fits in the HBM budget left, and charged the larger of */
/* that estimate and the device memory its creation took. `slots` worker      */
/* threads each take the oldest waiting request whose tenant is idle, so      */
/* requests start as soon as a slot and their tenant are free and different   */
/* tenants' snapshots overlap on the device (one stream per session).         */
/* Thread-safe: any thread may submit or wait.                                */
/* ------------------------------------------------------------------------- */
typedef struct tsvd_server tsvd_server;
typedef struct tsvd_server_stats_t {
  int64_t updates;       /* completed edge-update requests                 */
  int64_t edges;         /* edges they applied                             */
  double p50_ms, p99_ms; /* update latency, submission to completion       */
  double edges_per_s;    /* edges over first submission .. last completion */
  int64_t hbm_budget, hbm_charged;
  int32_t tenants;
} tsvd_server_stats_t;

/* hbm_budget_bytes <= 0: the free device memory now, less 4 GB. */
tsvd_status tsvd_server_create(int32_t device, int64_t hbm_budget_bytes, int32_t slots,
                               tsvd_server **out);
/* TSVD_ERR_OOM when the tenant does not fit in the budget left (nothing is
 * allocated then). expected_edges sizes the footprint estimate. */
tsvd_status tsvd_server_add_tenant(tsvd_server *sv, const tsvd_config *cfg,
                                   int64_t expected_edges, int32_t *tenant);
/* Waits for the tenant's queued requests, then frees its session and budget. */
tsvd_status tsvd_server_remove_tenant(tsvd_server *sv, int32_t tenant);
/* One snapshot of m (from, to) pairs (copied at submission). */
tsvd_status tsvd_server_submit_update(tsvd_server *sv, int32_t tenant, const int32_t *edges,
                                      int64_t m, int64_t *request);
/* The tenant's embedding (|S| x d doubles into out, which must stay valid
 * until the request completes) after every update submitted before it. */
tsvd_status tsvd_server_submit_query(tsvd_server *sv, int32_t tenant, double *out,
                                     int64_t *request);
/* Blocks until the request completes; its status, latency (submission to
 * completion) and service time (start to completion). */
tsvd_status tsvd_server_wait(tsvd_server *sv, int64_t request, double *latency_ms,
                             double *service_ms);
tsvd_status tsvd_server_drain(tsvd_server *sv);
tsvd_status tsvd_server_stats(tsvd_server *sv, tsvd_server_stats_t *out);
/* The tenant's session (inspection; do not step it while requests run). */
tsvd_status tsvd_server_session(tsvd_server *sv, int32_t tenant, tsvd_session **out);
tsvd_status tsvd_server_destroy(tsvd_server *sv);

/* ------------------------------------------------------------------------- */
/* Synthetic inputs (seeded; stand in for the reference's datasets).           */
/* ------------------------------------------------------------------------- */
/* R-MAT edges (a,b,c,d) with self-loops and duplicates dropped (undirected
 * duplicates are unordered pairs), vertex ids permuted by a seeded random
 * permutation, then shuffled into uniform-random timestamp order.
 * edges_out: 2*m int32. */
tsvd_status tsvd_rmat_edges(int32_t n, int64_t m, double a, double b, double c,
                            int32_t directed, uint64_t seed,
                            int32_t *edges_out);
/* Snapshot sizes: first gets round(first_frac*m), the rest split evenly. */
tsvd_status tsvd_snapshot_sizes(int64_t m, int32_t n_snapshots,
                                double first_frac, int64_t *sizes_out);
/* |S| distinct vertices drawn uniformly from those touched by `edges`
 * (the reference samples among first-snapshot nodes,
 * Random_Sample_Points_NC.cpp), returned sorted ascending. */
tsvd_status tsvd_sample_sources(int32_t n, const int32_t *edges, int64_t m,
                                int32_t k, uint64_t seed, int32_t *out);
/* Parse a "u v" per line edge file. compat_dup_last = 1 reproduces the
 * reference reader's repeat of the last pair when the file ends in
 * whitespace (Graph_dynamic.h:127-130, 539-542). A path ending in ".bin" is
 * read as raw int32 (from, to) pairs in host byte order instead (no
 * counterpart in the reference: fast ingestion of large deltas). *edges is
 * malloc'ed; free with tsvd_free. */
tsvd_status tsvd_read_edge_file(const char *path, int32_t compat_dup_last,
                                int32_t **edges, int64_t *m);
/* Writes m pairs as a ".bin" edge file (no counterpart in the reference). */
tsvd_status tsvd_write_edge_file_binary(const char *path, const int32_t *edges, int64_t m);
void tsvd_free(void *p);

/* Gaussian test-matrix entry used by frPCA (Philox4x32-10 + Box-Muller in
 * float, rounded to half precision); identical on host and device. */
float tsvd_gaussian(uint64_t seed, uint32_t stream, uint32_t row, uint32_t col);

#ifdef __cplusplus
}
#endif
#endif /* TSVD_H */
