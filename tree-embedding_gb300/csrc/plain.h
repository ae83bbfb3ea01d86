// The plain GPU form of the snapshot refresh: the straightforward port that
// the mixed-precision batched form is measured against.
//
//  * push: one frontier entry per (vertex, source) cell, one warp per entry
//    (lanes over the neighbour list), one scalar atomic per neighbour and
//    source; push arithmetic in fp64, stored in the shared fp32 state (the
//    reference's dense path: float arrays, double expressions);
//  * frPCA: every dirty block factorized on its own (one launch sequence per
//    block) with FP32 CSR SpMM for both products (A X over the rows, A^T Q
//    over the columns) instead of the half-precision tensor-core products;
//  * merge: one launch sequence per tree node.
//
// It shares the graph store, the PPR state arrays, the block materialization
// (log transform, norms, lazy test) and the small dense solves with the
// mixed form, so a session can switch forms between snapshots and both
// leave the same invariants behind.
#pragma once
#include "internal.h"
#include "ppr.h"

namespace tsvd {

struct PlainPpr {
  uint32_t *cbits = nullptr;  // touched cells, bit ppr_cell(v, s, n)
  int64_t nwords = 0;
  int2 *front[2] = {nullptr, nullptr};  // (vertex, source) entries
  int64_t cap = 0;
  int cur = 0;
  bool seeded = false;
  bool primed = false;                // frontier 0 written by the from-scratch refresh
  unsigned long long *counters = nullptr;  // [0],[1] frontier counts (attempted entries:
                                           // above cap, the rest waits in the bitset)
  unsigned long long *host_counters = nullptr;  // pinned
  unsigned long long *stats = nullptr;  // [2]: pushes, edge updates
  cudaEvent_t kev[16] = {};
};

tsvd_status plain_alloc(PlainPpr &Q, int32_t n, int32_t sp, int64_t cap);
void plain_free(PlainPpr &Q);
// Refresh of every source (from scratch: r = e_s) on the cell frontier.
tsvd_status plain_refresh(PlainPpr &Q, PprState &P, const Adjacency &A,
                          const int32_t *sources_dev, bool from_scratch, const PprParams &prm,
                          cudaStream_t st);
// Rounds until no cell with a residue above rmax (and a non-zero degree) is left.
tsvd_status plain_push(PlainPpr &Q, PprState &P, const Adjacency &A, const PprParams &prm,
                       uint8_t *vmark, cudaStream_t st, PushStats *out);

// One block of the log-transformed matrix in FP32, both ways round: CSR over
// the sources (rows 0..sp, rows >= |S| empty) and CSC over the block's
// compacted columns, entries in ascending order within every row / column.
struct SparseBlock {
  int32_t rows = 0, cols = 0;
  int64_t nnz = 0;
  int64_t *rowptr = nullptr;  // rows + 1
  int32_t *colidx = nullptr;  // nnz
  float *rval = nullptr;      // nnz
  int64_t *colptr = nullptr;  // cols + 1
  int32_t *rowidx = nullptr;  // nnz
  float *cval = nullptr;      // nnz
};

struct PlainBlockWork {
  SparseBlock blk;
  int64_t nnz_cap = 0, cols_cap = 0, rows_cap = 0;
  int32_t *cnt = nullptr;      // per column / per row counts
  uint32_t *keys = nullptr, *vals = nullptr, *keys_alt = nullptr, *vals_alt = nullptr;
  int32_t *ecol = nullptr;     // column of every CSC entry
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
};

// Where a block's values come from: the log transform of the reserve in fp32
// (plain form), or the accepted half-precision A^T of the mixed form (then
// the sparse and the tensor-core paths multiply exactly the same values).
struct BlockSource {
  const float *p1 = nullptr, *p2 = nullptr;  // reserve (forward, reverse or null), chunk-major
  const int32_t *colmap = nullptr;           // compacted column -> vertex, for this block
  const __half *at = nullptr;                // or: A^T [ncols][sp] (then p1, p2 unused)
  int32_t ncols = 0, n = 0, sp = 0, nsrc = 0, transform = 0;
  float rmin_f = 0.f, inv_rmin_f = 0.f, n_f = 0.f;
};

tsvd_status plain_block_build(PlainBlockWork &W, const BlockSource &src, int64_t nnz_hint,
                              cudaStream_t st);
void plain_block_free(PlainBlockWork &W);

// Y[b] (rows_out x kLp fp32) = scale * S_b (rows_out x K, CSR) * (hi + lo)[b]
// (K x kLp half, lo optional): the FP32 SpMM of the plain form, one warp per
// output row, entries of a row summed in their stored order.
tsvd_status spmm_batched(const int64_t *const *ptr, const int32_t *const *idx,
                         const float *const *val, const int32_t *rows_out, int max_rows,
                         const __half *const *hi, const __half *const *lo, float *const *y,
                         float scale, int nprob, cudaStream_t st);

}  // namespace tsvd
