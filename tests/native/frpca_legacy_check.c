/* Calls the reference-compatible frPCA(mat_csr *, mat **, mat **, mat **, k, q)
 * exactly as the reference's drivers do (Code/Tree_u_NC.cpp:139-145): a
 * 1-based CSR with begin/end row pointers (pointerB / pointerE), output
 * matrices preallocated by the caller, singular values handed back in
 * ascending order. Built and run by tests/test_gpu_legacy_frpca.py.
 *
 *   frpca_legacy_check IN OUT
 * IN : int32 m, n, nnz, k, q; uint64 seed; int32 pointerB[m], pointerE[m],
 *      cols[nnz] (all 1-based); float64 values[nnz]
 * OUT: float64 U[m*k], S[k], V[n*k] (column-major, as the reference's mat),
 *      then the int32 count of U / S / V entries left unwritten (NaN sentinel)
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tsvd.h"

static mat *matrix_new(int nrows, int ncols) {
  mat *M = (mat *)malloc(sizeof(mat));
  M->nrows = nrows;
  M->ncols = ncols;
  M->d = (double *)malloc(sizeof(double) * (size_t)nrows * ncols);
  for (size_t i = 0; i < (size_t)nrows * ncols; ++i) M->d[i] = NAN;  /* sentinel */
  return M;
}

static int rd(FILE *f, void *p, size_t sz, size_t n) { return fread(p, sz, n, f) == n ? 0 : -1; }

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  int hdr[5];
  unsigned long long seed;
  if (rd(f, hdr, 4, 5) || rd(f, &seed, 8, 1)) return 4;
  const int m = hdr[0], n = hdr[1], nnz = hdr[2], k = hdr[3], q = hdr[4];
  mat_csr A;
  A.nrows = m;
  A.ncols = n;
  A.nnz = nnz;
  A.pointerB = (int *)malloc(sizeof(int) * m);
  A.pointerE = (int *)malloc(sizeof(int) * m);
  A.cols = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  A.values = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  if (rd(f, A.pointerB, 4, m) || rd(f, A.pointerE, 4, m) || rd(f, A.cols, 4, nnz) ||
      rd(f, A.values, 8, nnz))
    return 5;
  fclose(f);
  mat *U = matrix_new(m, k), *S = matrix_new(k, 1), *V = matrix_new(n, k);
  tsvd_set_frpca_seed(seed);
  frPCA(&A, &U, &S, &V, k, q);
  int unset = 0;
  for (size_t i = 0; i < (size_t)m * k; ++i) unset += isnan(U->d[i]);
  for (int i = 0; i < k; ++i) unset += isnan(S->d[i]);
  for (size_t i = 0; i < (size_t)n * k; ++i) unset += isnan(V->d[i]);
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 6;
  fwrite(U->d, 8, (size_t)m * k, o);
  fwrite(S->d, 8, (size_t)k, o);
  fwrite(V->d, 8, (size_t)n * k, o);
  fwrite(&unset, 4, 1, o);
  fclose(o);
  if (strlen(tsvd_last_error()) > 0) fprintf(stderr, "tsvd_last_error: %s\n", tsvd_last_error());
  return 0;
}
