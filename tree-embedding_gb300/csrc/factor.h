// Batched frPCA of column blocks and batched tree merges.
#pragma once
#include "internal.h"

namespace tsvd {

struct FrpcaWork {
  int nmax = 0;           // problems (blocks or merge parents) per batch
  int64_t rows_max = 0;   // max block width (rows of A^T)
  int sp = 0, l = 0, d = 0;
  __half *xhi = nullptr, *xlo = nullptr;  // [nmax][rows_max][kLp]
  float *z = nullptr;                      // [nmax][rows_max][kLp]
  float *y = nullptr;                      // [nmax][sp][kLp]
  __half *qhi = nullptr, *qlo = nullptr;  // [nmax][sp][kLp]
  double *g = nullptr;                     // [nmax][256*256]
  float *t = nullptr;                      // [nmax][kLp*kLp]
  float *lambda = nullptr;                 // [nmax][256]
  float *v = nullptr;                      // [nmax][256*256]
  float *colscale = nullptr;               // [nmax][512]: scale, inverse scale
  double *sums = nullptr;                  // [nmax] sum of kept sigma^2
  double *gram_work = nullptr;
  size_t gram_bytes = 0;
  void *jac_work = nullptr;
  size_t jac_bytes = 0;
  void **dptr = nullptr;   // device pointer-array area
  void **hptr = nullptr;   // pinned staging for the pointer arrays
  size_t ptr_slots = 0;
  int32_t *dint = nullptr; // device int area (row counts, block ids)
  int32_t *hint = nullptr;
  CUtensorMap *tmap_dev = nullptr;   // tensor maps of the products: 6 per problem
  CUtensorMap *tmap_host = nullptr;  // pinned staging for them
  size_t tmap_slots = 0;
  int last_sweeps = 0;
  double *dv = nullptr, *dt = nullptr, *dh = nullptr;  // [nmax][256*256] eigen refinement
  double **dh_ptrs = nullptr;  // device: dh + i 256^2 for each problem i
  int last_refine_sweeps = 0;
  // merges wider than 256 columns (allocated on first use)
  float *wm = nullptr;      // [nprob][|S|][n] the concatenated children
  float *wv = nullptr;      // [nprob][n][256] basis of the right singular subspace
  float *ww = nullptr;      // [nprob][n][256] M^T Y before normalization
  float *wy = nullptr;      // [nprob][|S|][256] M V, then its orthonormal basis
  float *wy2 = nullptr;
  double *wchol = nullptr;  // [nprob][2][256][256] Cholesky factors
  float *wk = nullptr;      // [nprob][256*256 + 256*257/2] fp32 Gram + packed factor
  float *wnorm = nullptr;   // [nprob][n] column norms of M
  size_t wide_cap = 0;      // problems x n x |S| the buffers hold
  int wide_nprob = 0, wide_n = 0;
  int wide_iters = 0;       // subspace iterations of the last wide merge level
};

tsvd_status frpca_work_alloc(FrpcaWork &W, int nmax, int64_t rows_max, int sp, int l, int d);
void frpca_work_free(FrpcaWork &W);

struct SparseBlock;

struct FrpcaProblem {
  int32_t block;            // Gaussian stream id
  const __half *at;         // A^T [ncols][sp]
  int32_t ncols;
  const int32_t *colmap;    // device: compacted column -> global column id
  int32_t col_base;         // global id of the block's first column
  float *b_out;             // |S| x d (ld d): U * diag(sigma), or null
  float *sigma_out;         // d, or null
  float *u_out;             // sp x d (ld d): U, or null
  float *v_out;             // ncols x d (ld d): V, or null
  const SparseBlock *sparse = nullptr;  // FP32 CSR/CSC of the block (plain form): both
                                        // products as SpMM instead of tensor-core GEMMs
};

// Runs frPCA (k = d, oversampling l - d, q passes) on every problem. sum_sigma2
// (host, nprob) receives the sum of the kept squared singular values. Either
// every problem carries a SparseBlock (FP32 SpMM products) or none does
// (half-precision A^T on the tensor cores).
tsvd_status frpca_batch(FrpcaWork &W, const FrpcaProblem *probs, int nprob, int q,
                        uint64_t seed, int nsrc, cudaStream_t st, double *sum_sigma2);

struct MergeProblem {
  const float *children[16];  // h child factors, |S| x d (ld d)
  float *out;                 // |S| x d (ld d)
  float *sigma_out;           // d
};

// Truncated SVD of [B_1 ... B_h] for every problem; out = U_d * diag(s_d) * f(s_d)
// with f = 1 (inner node), s^-1/2 (root, U sqrt(S)) or s^-1 (root, U).
// The merge of one ready matrix: m_host (rows x cols row-major fp32, host);
// out (rows x d, device) = U_d diag(s_d), sigma_out (d, device) = s_d. W
// sized by frpca_work_alloc with sp >= rows.
tsvd_status merge_matrix(FrpcaWork &W, const float *m_host, int rows, int cols, float *out,
                         float *sigma_out, cudaStream_t st);

tsvd_status merge_batch(FrpcaWork &W, const MergeProblem *probs, int nprob, int h, int nsrc,
                        int root_mode, cudaStream_t st);

struct LpProblem {
  const __half *at;  // A^T of the block, [ncols][sp]
  int32_t ncols;
  float *v_out;      // [ncols][kLp]: row c = A[:, c]^T U (columns >= d are zero)
};

// LP right factor of every listed block: V_b = A_b^T U with U the |S| x d root
// factor (orthonormal columns), on the tensor cores (the transposed product of
// the frPCA passes). Tree_u_LP.cpp:291-407 (csr_matrix_transpose_matrix_mult
// per updated block).
tsvd_status lp_right_batch(FrpcaWork &W, const LpProblem *probs, int nprob, const float *u,
                           int nsrc, int d, cudaStream_t st);

}  // namespace tsvd
