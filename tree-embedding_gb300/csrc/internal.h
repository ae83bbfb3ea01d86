// Internal declarations shared by the CUDA translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (the encoder is resolved at run time; no libcuda link)
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "status.h"

#define TSVD_CUDA(call)                                                      \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess)                                                   \
      return tsvd::fail(_e == cudaErrorMemoryAllocation ? TSVD_ERR_OOM       \
                                                        : TSVD_ERR_DEVICE,   \
                        "%s:%d %s: %s", __FILE__, __LINE__, #call,           \
                        cudaGetErrorString(_e));                             \
  } while (0)

namespace tsvd {
void count_launch();
}

#define TSVD_LAUNCH_CHECK()                                                  \
  do {                                                                       \
    tsvd::count_launch();                                                    \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess)                                                   \
      return tsvd::fail(TSVD_ERR_DEVICE, "%s:%d launch: %s", __FILE__,       \
                        __LINE__, cudaGetErrorString(_e));                   \
  } while (0)

namespace tsvd {

constexpr int kWarp = 32;
constexpr int kRowPad = 128;  // |S| is padded to a multiple of this (GEMM M tile)
constexpr int kLp = 144;      // padded width of the l = d + s skinny matrices

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// Grid size for grid-stride kernels: a multiple of the SM count.
int grid_for(int64_t work_items, int threads_per_block, int blocks_per_sm = 8);
int sm_count();

// ---------------------------------------------------------------- scan/sort
// Exclusive prefix sum of n int32 counts into int64 offsets (out has n+1
// entries; out[n] = total). `tmp` must hold scan_tmp_bytes(n) bytes.
size_t scan_tmp_bytes(int64_t n);
tsvd_status scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n,
                            void *tmp, cudaStream_t st);
// Stable LSD radix sort of (key, value) pairs by key (key < 2^key_bits).
size_t sort_tmp_bytes(int64_t n);
tsvd_status stable_sort_pairs(uint32_t *keys, uint32_t *vals,
                              uint32_t *keys_alt, uint32_t *vals_alt, int64_t n,
                              int key_bits, void *tmp, cudaStream_t st,
                              bool *result_in_alt);

// ---------------------------------------------------------------- adjacency
struct Adjacency {
  int32_t n = 0;
  int64_t cap_total = 0;
  int64_t m = 0;           // stored entries
  int64_t *off = nullptr;  // n+1 row starts (capacity-based)
  int32_t *deg = nullptr;
  int32_t *former = nullptr;
  int32_t *nbr = nullptr;
};

struct InsertScratch {
  void *buf = nullptr;
  size_t bytes = 0;
};

// Appends `count` (vertex, neighbour) entries given in insertion order.
tsvd_status adjacency_append(Adjacency &A, const uint32_t *keys,
                             const uint32_t *vals, int64_t count,
                             InsertScratch &scr, cudaStream_t st);
void adjacency_free(Adjacency &A);

// ---------------------------------------------------------------- dense ops
struct GemmBatch {
  // Per problem (device arrays of length nprob):
  const int32_t *ncols;      // n_c of each block (the K of fwd / M of bwd)
  int lda;                   // = Sp
  int nprob;
  // device, 3 per problem (gemm_encode_maps): A^T, skinny hi, skinny lo
  const CUtensorMap *maps;
};

// Tensor maps of one batch of products, written to out[3 i .. 3 i + 2] for
// problem i: the block A^T (at[i], nc[i] rows of pitch lda, fp16) as the
// forward (fwd = 1) or backward product's A operand, and the skinny hi / lo
// halves (kLp columns; nc[i] rows in the forward product, lda in the
// backward one; lo may be null). Host pointers; out is host memory.
tsvd_status gemm_encode_maps(int fwd, int nprob, const __half *const *at, const int32_t *nc,
                             int lda, const __half *const *hi, const __half *const *lo,
                             CUtensorMap *out);

// Y[b] (Sp x Lp fp32) = A_b (Sp x n_c) * (Xhi + Xlo)[b] (n_c x Lp) * scale.
// y_base/y_bytes: the contiguous allocation behind y (zeroed for split-K).
tsvd_status gemm_fwd(const GemmBatch &gb, bool has_lo, float *const *y, float *y_base,
                     size_t y_bytes, int sp, int max_nc, float inv_xscale, cudaStream_t st);
// Z[b] (n_c x Lp fp32) = A_b^T (n_c x Sp) * (Yhi + Ylo)[b] (Sp x Lp) * scale
tsvd_status gemm_bwd(const GemmBatch &gb, bool has_lo, float *const *z, int sp, int max_nc,
                     float inv_yscale, cudaStream_t st);
// Non-zero if a tensor-core GEMM gave up waiting for its MMAs since the last
// check (a bounded wait ran out); synchronizes the stream.
tsvd_status gemm_check(cudaStream_t st);

// C[z] = op(A[z]) B[z] in fp32, row-major (op(A) = A^T when trans_a: A is
// K x M), problem z at z * stride of each operand; fixed-order sums.
tsvd_status sgemm_batched(bool trans_a, int M, int N, int K, const float *A, int lda, int64_t sa,
                          const float *B, int ldb, int64_t sb, float *C, int ldc, int64_t sc,
                          int nprob, cudaStream_t st);

// G[b] (l x l fp64) = X[b]^T X[b], X row-major [rows_b][ld] fp32.
tsvd_status gram_batched(const float *const *x, const int32_t *rows, int max_rows,
                         int l, int ld, double *const *g, double *work,
                         size_t work_bytes, int nprob, cudaStream_t st);
size_t gram_work_bytes(int max_rows, int l, int nprob);

// CholeskyQR step: T[b] = R^{-1} from G[b] (upper triangular, l x kLp fp32).
tsvd_status chol_inverse_batched(double *const *g, float *const *t, int l,
                                 int nprob, cudaStream_t st);
// CholeskyQR step for l <= 256: factor G[b] = L L^T in fp64 (work: nprob x
// (l*l + l) doubles), then y_b = x_b L^{-T} row by row (x, y: rows x l fp32,
// ld l, problem b at offset b * stride). Directions whose pivot falls below
// 1e-13 of the largest diagonal entry give zero columns.
tsvd_status chol_solve_wide_batched(double *const *g, double *work, const float *x, float *y,
                                    int rows, int l, int64_t stride, int nprob, cudaStream_t st);
// Cheap step of a subspace iteration (l <= 256): K[b] (l x l fp32, at b l l)
// + shift * trace/l * I = L L^T in fp32, Lpk (packed, nprob x l(l+1)/2) gets
// L, y_b = x_b L^{-T}. Keeps every direction; the basis is well-conditioned,
// not exactly orthonormal.
tsvd_status chol_shift_solve_batched(const float *K, float *Lpk, const float *x, float *y,
                                     int rows, int l, int64_t stride, float shift, int nprob,
                                     cudaStream_t st);
// Y[b] = X[b] * W[b] * diag(colscale[b]); writes fp32 (columns [n_out, ldy)
// zeroed) and, when yhi/ylo are given, the fp16 split of Y * split_scale.
tsvd_status apply_right_batched(const float *const *x, const int32_t *rows,
                                int max_rows, int ldx, const float *const *w,
                                int ldw, int n_in, int n_out,
                                const float *const *colscale, float *const *y,
                                int ldy, __half *const *yhi, __half *const *ylo,
                                float split_scale, int nprob, cudaStream_t st);
// Two-sided cyclic Jacobi on G[b] (n x n fp64 in, fp32 work): eigenvalues
// (descending) and eigenvectors V[b] (n x n row-major fp32, column j is the
// eigenvector of lambda[j]).
// refine = 1: g[b] = V^T G V for approximate eigenvectors V (nearly
// diagonal); the diagonal is carried in fp64 (see jacobi_kernel) and the
// rotations are replayed onto vinit[b] (V, n x n row-major), so v[b] = V R.
// v may alias vinit.
tsvd_status jacobi_eig_batched(double *const *g, int n, float *const *lambda,
                               float *const *v, int nprob, void *work,
                               size_t work_bytes, cudaStream_t st,
                               int *sweeps_out, int refine = 0,
                               const float *const *vinit = nullptr);
size_t jacobi_work_bytes(int n, int nprob);

}  // namespace tsvd
