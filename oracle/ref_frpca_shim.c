/* TEST INFRASTRUCTURE ONLY: plain-array entry points around the reference's
 * own frPCA (Code/frpca.c:239-326) and truncated SVD of the tree merge
 * (Code/matrix_vector_functions_intel_mkl.c:1259-1300, called by
 * dense_sub_svd_function, Code/Tree_u_NC.cpp:238-262), compiled from the
 * reference sources where they lie by oracle/build_ref.sh against the MKL
 * stand-in in oracle/mkl_shim/. Used by tests to pin the CPU oracle's
 * restatement of those two algorithms; never linked into the product. */
#include <stdlib.h>
#include <string.h>

#include "matrix_vector_functions_intel_mkl_ext.h"

void frPCA(mat_csr *A, mat **U, mat **S, mat **V, int k, int q);
void truncated_singular_value_decomposition(mat *M, mat *U, mat *S, mat *Vt, int d);

/* A: m x n in 0-based CSR (rowptr[m + 1], cols, vals). Outputs column-major:
 * U m x k, S k (the order frPCA leaves them in), V n x k. */
int tsvd_ref_frpca(int m, int n, const int *rowptr, const int *cols, const double *vals, int k,
                   int q, double *U_out, double *S_out, double *V_out) {
  const int nnz = rowptr[m];
  mat_csr A;
  A.nnz = nnz;
  A.nrows = m;
  A.ncols = n;
  A.values = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  A.cols = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  A.pointerB = (int *)malloc(sizeof(int) * (size_t)m);
  A.pointerE = (int *)malloc(sizeof(int) * (size_t)m);
  for (int p = 0; p < nnz; ++p) {
    A.values[p] = vals[p];
    A.cols[p] = cols[p] + 1;
  }
  for (int i = 0; i < m; ++i) {
    A.pointerB[i] = rowptr[i] + 1;
    A.pointerE[i] = rowptr[i + 1] + 1;
  }
  mat *U = matrix_new(m, k), *S = matrix_new(k, 1), *V = matrix_new(n, k);
  frPCA(&A, &U, &S, &V, k, q);
  memcpy(U_out, U->d, sizeof(double) * (size_t)m * k);
  memcpy(S_out, S->d, sizeof(double) * (size_t)k);
  memcpy(V_out, V->d, sizeof(double) * (size_t)n * k);
  matrix_delete(U);
  matrix_delete(S);
  matrix_delete(V);
  free(A.values);
  free(A.cols);
  free(A.pointerB);
  free(A.pointerE);
  return 0;
}

/* M: m x n column-major. US = U_d S_d (m x d, column-major), the merge node
 * factor of dense_sub_svd_function; sigma: the d leading singular values. */
int tsvd_ref_merge_svd(int m, int n, const double *M_in, int d, double *US_out,
                       double *sigma_out) {
  mat *M = matrix_new(m, n);
  memcpy(M->d, M_in, sizeof(double) * (size_t)m * n);
  mat *U = matrix_new(m, d), *S = matrix_new(d, d), *Vt = matrix_new(d, n);
  truncated_singular_value_decomposition(M, U, S, Vt, d);
  mat *US = matrix_new(m, d);
  matrix_matrix_mult(U, S, US);
  memcpy(US_out, US->d, sizeof(double) * (size_t)m * d);
  for (int i = 0; i < d; ++i) sigma_out[i] = matrix_get_element(S, i, i);
  matrix_delete(M);
  matrix_delete(U);
  matrix_delete(S);
  matrix_delete(Vt);
  matrix_delete(US);
  return 0;
}
