/* TEST INFRASTRUCTURE ONLY: LAPACKE declarations for the MKL stand-in (see
 * mkl.h); the routines come from scipy's bundled OpenBLAS (LP64). */
#ifndef TSVD_MKL_SHIM_LAPACKE_H
#define TSVD_MKL_SHIM_LAPACKE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

lapack_int scipy_LAPACKE_dgeqrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda,
                                double *tau);
lapack_int scipy_LAPACKE_dorgqr(int layout, lapack_int m, lapack_int n, lapack_int k, double *a,
                                lapack_int lda, const double *tau);
lapack_int scipy_LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda,
                                lapack_int *ipiv);
lapack_int scipy_LAPACKE_dgesvd(int layout, char jobu, char jobvt, lapack_int m, lapack_int n,
                                double *a, lapack_int lda, double *s, double *u, lapack_int ldu,
                                double *vt, lapack_int ldvt, double *superb);
lapack_int scipy_LAPACKE_dsyev(int layout, char jobz, char uplo, lapack_int n, double *a,
                               lapack_int lda, double *w);
lapack_int scipy_LAPACKE_dsyevd(int layout, char jobz, char uplo, lapack_int n, double *a,
                                lapack_int lda, double *w);
lapack_int scipy_LAPACKE_dgeqpf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda,
                                lapack_int *jpvt, double *tau);
lapack_int scipy_LAPACKE_dtrtrs(int layout, char uplo, char trans, char diag, lapack_int n,
                                lapack_int nrhs, const double *a, lapack_int lda, double *b,
                                lapack_int ldb);
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_dsyev scipy_LAPACKE_dsyev
#define LAPACKE_dsyevd scipy_LAPACKE_dsyevd
#define LAPACKE_dgeqpf scipy_LAPACKE_dgeqpf
#define LAPACKE_dtrtrs scipy_LAPACKE_dtrtrs
#ifdef __cplusplus
}
#endif
#endif
