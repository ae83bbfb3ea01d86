/* TEST INFRASTRUCTURE ONLY: the VSL random-stream interface used by the
 * reference (time-seeded Gaussian and uniform streams), implemented in
 * mkl_shim.c by a counter-based generator so runs are repeatable and the
 * test can read back the Gaussian matrix frPCA drew (tsvd_ref_last_gaussian). */
#ifndef TSVD_MKL_SHIM_VSL_H
#define TSVD_MKL_SHIM_VSL_H
#ifdef __cplusplus
extern "C" {
#endif
typedef void *VSLStreamStatePtr;
#define VSL_BRNG_MCG31 0x100000
#define VSL_RNG_METHOD_GAUSSIAN_ICDF 2
#define VSL_RNG_METHOD_GAUSSIAN_BOXMULLER 0
#define VSL_RNG_METHOD_UNIFORM_STD 0
int vslNewStream(VSLStreamStatePtr *stream, int brng, unsigned int seed);
int vslDeleteStream(VSLStreamStatePtr *stream);
int vsRngGaussian(int method, VSLStreamStatePtr stream, int n, float *r, float a, float sigma);
int vdRngGaussian(int method, VSLStreamStatePtr stream, int n, double *r, double a, double sigma);
int vdRngUniform(int method, VSLStreamStatePtr stream, int n, double *r, double a, double b);
#ifdef __cplusplus
}
#endif
#endif
