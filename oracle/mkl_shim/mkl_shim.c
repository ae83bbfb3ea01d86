/* TEST INFRASTRUCTURE ONLY: the parts of the MKL interface declared in
 * mkl.h / mkl_vsl.h that OpenBLAS does not provide, so the reference's
 * frpca.c and matrix_vector_functions_intel_mkl{,_ext}.c can be compiled and
 * run here as a check on the CPU oracle. Never linked into the product.
 *
 * mkl_dcsrmm / mkl_dcoomm: C := alpha op(A) B + beta C with A sparse in
 * 1-based CSR (pointerB/pointerE) or COO and B, C dense column-major, the
 * "GXXF" form every reference call uses.
 * VSL streams: a counter-based generator (splitmix64 + Box-Muller, written
 * here) replaces MKL's MCG31; the seed the reference passes (time(NULL) for
 * the Gaussian test matrices) is ignored, so runs repeat, and the last
 * Gaussian draw is kept for tsvd_ref_last_gaussian(). */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <unistd.h>
#include <stdlib.h>
#include <string.h>

#include "mkl.h"
#include "mkl_vsl.h"

static void scale_c(const MKL_INT rows, const MKL_INT n, const double beta, double *c,
                    const MKL_INT ldc) {
  for (MKL_INT j = 0; j < n; ++j)
    for (MKL_INT i = 0; i < rows; ++i) c[i + (size_t)j * ldc] = beta == 0.0 ? 0.0 : beta * c[i + (size_t)j * ldc];
}

/* MKL runs this product on every core; so does the stand-in (threads =
 * TSVD_REF_THREADS, default: all online cores). B is first copied row-major
 * so that each stored entry of A reads one contiguous row of B. Without
 * transpose, threads take contiguous row ranges of C; with it (C = A^T B),
 * each thread accumulates its rows of A into a private k x n buffer and the
 * buffers are summed. */
typedef struct {
  int trans;
  MKL_INT m, n, k, r0, r1;
  double alpha;
  const double *val, *bt;
  const MKL_INT *indx, *pntrb, *pntre;
  double *acc;   /* row-major: m x n (no transpose: rows r0..r1) or k x n (private) */
} csrmm_job;

static void *csrmm_run(void *arg) {
  csrmm_job *J = (csrmm_job *)arg;
  const MKL_INT n = J->n;
  for (MKL_INT i = J->r0; i < J->r1; ++i)
    for (MKL_INT p = J->pntrb[i] - 1; p < J->pntre[i] - 1; ++p) {
      const MKL_INT col = J->indx[p] - 1;
      const double a = J->alpha * J->val[p];
      double *dst = J->trans ? J->acc + (size_t)col * n : J->acc + (size_t)i * n;
      const double *src = J->trans ? J->bt + (size_t)i * n : J->bt + (size_t)col * n;
      for (MKL_INT j = 0; j < n; ++j) dst[j] += a * src[j];
    }
  return NULL;
}

static int shim_threads(void) {
  const char *e = getenv("TSVD_REF_THREADS");
  long t = e ? atol(e) : sysconf(_SC_NPROCESSORS_ONLN);
  return t < 1 ? 1 : (t > 256 ? 256 : (int)t);
}

void mkl_dcsrmm(const char *transa, const MKL_INT *m, const MKL_INT *n, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *indx, const MKL_INT *pntrb, const MKL_INT *pntre, const double *b,
                const MKL_INT *ldb, const double *beta, double *c, const MKL_INT *ldc) {
  (void)matdescra;
  const int trans = transa[0] == 'T' || transa[0] == 't';
  const MKL_INT out_rows = trans ? *k : *m, in_rows = trans ? *m : *k, nc = *n;
  scale_c(out_rows, nc, *beta, c, *ldc);
  double *bt = (double *)malloc(sizeof(double) * (size_t)in_rows * nc + 8);
  for (MKL_INT j = 0; j < nc; ++j)
    for (MKL_INT i = 0; i < in_rows; ++i) bt[(size_t)i * nc + j] = b[i + (size_t)j * *ldb];
  int T = shim_threads();
  if (T > *m) T = *m > 0 ? *m : 1;
  csrmm_job jobs[256];
  pthread_t th[256];
  double *acc = NULL;
  if (!trans) acc = (double *)calloc((size_t)*m * nc + 1, sizeof(double));
  for (int t = 0; t < T; ++t) {
    csrmm_job J = {trans, *m, nc, *k, (MKL_INT)((long long)*m * t / T),
                   (MKL_INT)((long long)*m * (t + 1) / T), *alpha, val, bt, indx, pntrb, pntre,
                   trans ? (double *)calloc((size_t)*k * nc + 1, sizeof(double)) : acc};
    jobs[t] = J;
    pthread_create(&th[t], NULL, csrmm_run, &jobs[t]);
  }
  for (int t = 0; t < T; ++t) pthread_join(th[t], NULL);
  for (MKL_INT i = 0; i < out_rows; ++i)
    for (MKL_INT j = 0; j < nc; ++j) {
      double x = 0.0;
      if (trans)
        for (int t = 0; t < T; ++t) x += jobs[t].acc[(size_t)i * nc + j];
      else
        x = acc[(size_t)i * nc + j];
      c[i + (size_t)j * *ldc] += x;
    }
  if (trans)
    for (int t = 0; t < T; ++t) free(jobs[t].acc);
  free(acc);
  free(bt);
}

void mkl_dcoomm(const char *transa, const MKL_INT *m, const MKL_INT *n, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *rowind, const MKL_INT *colind, const MKL_INT *nnz, const double *b,
                const MKL_INT *ldb, const double *beta, double *c, const MKL_INT *ldc) {
  (void)matdescra;
  const int trans = transa[0] == 'T' || transa[0] == 't';
  const MKL_INT out_rows = trans ? *k : *m;
  scale_c(out_rows, *n, *beta, c, *ldc);
  for (MKL_INT p = 0; p < *nnz; ++p) {
    const MKL_INT r = rowind[p] - 1, col = colind[p] - 1;
    const double a = *alpha * val[p];
    for (MKL_INT j = 0; j < *n; ++j) {
      if (trans)
        c[col + (size_t)j * *ldc] += a * b[r + (size_t)j * *ldb];
      else
        c[r + (size_t)j * *ldc] += a * b[col + (size_t)j * *ldb];
    }
  }
}

void *mkl_calloc(size_t num, size_t size, int alignment) {
  (void)alignment;
  return calloc(num, size);
}
void *mkl_malloc(size_t size, int alignment) {
  (void)alignment;
  return malloc(size);
}
void mkl_free(void *p) { free(p); }

/* ------------------------------------------------------------ random streams */
typedef struct {
  uint64_t key, counter;
} shim_stream;

static uint64_t g_seed = 20231;
static uint64_t g_streams = 0;
static float *g_last = NULL;
static int g_last_n = 0;

static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static double uniform01(shim_stream *s) {  /* in (0, 1) */
  const uint64_t x = splitmix64(s->key ^ splitmix64(s->counter++));
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static double gaussian(shim_stream *s) {  /* Box-Muller, one value per pair of uniforms */
  const double u1 = uniform01(s), u2 = uniform01(s);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

int vslNewStream(VSLStreamStatePtr *stream, int brng, unsigned int seed) {
  (void)brng;
  (void)seed;
  shim_stream *s = (shim_stream *)malloc(sizeof *s);
  s->key = splitmix64(g_seed * 0x100000001B3ull + g_streams++);
  s->counter = 0;
  *stream = s;
  return 0;
}

int vslDeleteStream(VSLStreamStatePtr *stream) {
  free(*stream);
  *stream = NULL;
  return 0;
}

int vsRngGaussian(int method, VSLStreamStatePtr stream, int n, float *r, float a, float sigma) {
  (void)method;
  for (int i = 0; i < n; ++i) r[i] = (float)(a + sigma * gaussian((shim_stream *)stream));
  free(g_last);
  g_last = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  memcpy(g_last, r, sizeof(float) * (size_t)n);
  g_last_n = n;
  return 0;
}

int vdRngGaussian(int method, VSLStreamStatePtr stream, int n, double *r, double a, double sigma) {
  (void)method;
  for (int i = 0; i < n; ++i) r[i] = a + sigma * gaussian((shim_stream *)stream);
  return 0;
}

int vdRngUniform(int method, VSLStreamStatePtr stream, int n, double *r, double a, double b) {
  (void)method;
  for (int i = 0; i < n; ++i) r[i] = a + (b - a) * uniform01((shim_stream *)stream);
  return 0;
}

/* Restart the generator (every later stream derives from this seed). */
void tsvd_ref_set_seed(uint64_t seed) {
  g_seed = seed;
  g_streams = 0;
}

/* Copies the last Gaussian draw (at most n values) into out; returns its length. */
int tsvd_ref_last_gaussian(float *out, int n) {
  const int m = g_last_n < n ? g_last_n : n;
  if (out && m > 0) memcpy(out, g_last, sizeof(float) * (size_t)m);
  return g_last_n;
}
