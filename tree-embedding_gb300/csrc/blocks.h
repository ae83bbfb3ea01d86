// Column-block materialization interface.
#pragma once
#include <algorithm>

#include "internal.h"

namespace tsvd {

struct MaterializeArgs {
  const float *p1;        // reserve, chunk-major (ppr_cell) (forward / undirected)
  const float *p2;        // reserve of the reverse push (directed) or null
  const int32_t *colmap;  // compacted vertex ids, block b at [b*col_dim, ...)
  const int32_t *ncols;   // current column counts
  const int32_t *ncols_old;
  const __half *const *at_old;  // accepted A^T of each block
  __half *const *at_new;        // output A^T of each block
  int32_t n, sp, nsrc, col_dim;
  int transform;
  float rmin_f, inv_rmin_f, n_f;
  double *norm2, *diff2;
  unsigned long long *nnz, *stored;
};

tsvd_status colmap_update(uint8_t *vmark, int32_t *colmap, int32_t *colpos, int32_t *ncols,
                          int32_t n, int32_t col_dim, int32_t nparts, cudaStream_t st);
tsvd_status materialize_blocks(const MaterializeArgs &a, int nparts, int32_t max_nc,
                               cudaStream_t st);

}  // namespace tsvd
