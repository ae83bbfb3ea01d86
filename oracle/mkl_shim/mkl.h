/* TEST INFRASTRUCTURE ONLY. The subset of the Intel MKL C interface that the
 * reference's frpca.c and matrix_vector_functions_intel_mkl{,_ext}.c use,
 * declared so those files compile unchanged without MKL: dense BLAS and
 * LAPACKE come from the OpenBLAS that scipy bundles (LP64, symbols prefixed
 * "scipy_"); the sparse products and the random streams are implemented in
 * oracle/mkl_shim/mkl_shim.c. Built only by oracle/build_ref.sh. */
#ifndef TSVD_MKL_SHIM_H
#define TSVD_MKL_SHIM_H
#include <stddef.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MKL_INT;

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_LAYOUT CBLAS_LAYOUT;
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE;

void scipy_cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n,
                       int k, double alpha, const double *a, int lda, const double *b, int ldb,
                       double beta, double *c, int ldc);
void scipy_cblas_dgemv(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, int m, int n, double alpha,
                       const double *a, int lda, const double *x, int incx, double beta, double *y,
                       int incy);
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dgemv scipy_cblas_dgemv

/* C := alpha op(A) B + beta C; A sparse (CSR / COO), B and C dense column-major
 * with 1-based sparse indices when matdescra[3] == 'F' (the only form used). */
void mkl_dcsrmm(const char *transa, const MKL_INT *m, const MKL_INT *n, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *indx, const MKL_INT *pntrb, const MKL_INT *pntre, const double *b,
                const MKL_INT *ldb, const double *beta, double *c, const MKL_INT *ldc);
void mkl_dcoomm(const char *transa, const MKL_INT *m, const MKL_INT *n, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *rowind, const MKL_INT *colind, const MKL_INT *nnz, const double *b,
                const MKL_INT *ldb, const double *beta, double *c, const MKL_INT *ldc);

void *mkl_calloc(size_t num, size_t size, int alignment);
void *mkl_malloc(size_t size, int alignment);
void mkl_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
