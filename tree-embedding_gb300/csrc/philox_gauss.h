/*
 * Counter-based Gaussian generator shared by host and device code.
 *
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11) turns (counter, key) into four 32-bit words; two
 * of them feed a Box-Muller transform evaluated in float with explicitly
 * rounded operations (fma / correctly rounded div and sqrt) and polynomial
 * log / sin / cos written from their series, so the host and the GPU produce
 * bit-identical values. The result is rounded to half precision (round to
 * nearest even), the precision at which the test matrix enters the tensor-core
 * products; the CPU oracle consumes the same values.
 *
 * Replaces initialize_random_matrix (Code/matrix_vector_functions_intel_mkl.c:
 * 479-505), which draws N(0,1) floats from MKL VSL seeded with time(NULL).
 */
#ifndef TSVD_PHILOX_GAUSS_H
#define TSVD_PHILOX_GAUSS_H

#include <stdint.h>
#include <string.h>
#ifndef __CUDACC__
#include <math.h>
#endif

#if defined(__CUDACC__)
#define TSVD_HD __host__ __device__ __forceinline__
#else
#define TSVD_HD static inline
#endif

/* Exactly rounded primitives: on the device the _rn intrinsics keep nvcc from
 * contracting a*b+c; the host side is compiled with -ffp-contract=off. */
#if defined(__CUDA_ARCH__)
#define TSVD_FMUL(a, b) __fmul_rn((a), (b))
#define TSVD_FADD(a, b) __fadd_rn((a), (b))
#define TSVD_FSUB(a, b) __fsub_rn((a), (b))
#define TSVD_FDIV(a, b) __fdiv_rn((a), (b))
#define TSVD_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define TSVD_FSQRT(a) __fsqrt_rn(a)
#define TSVD_RINT(a) rintf(a)
#else
#define TSVD_FMUL(a, b) ((float)((a) * (b)))
#define TSVD_FADD(a, b) ((float)((a) + (b)))
#define TSVD_FSUB(a, b) ((float)((a) - (b)))
#define TSVD_FDIV(a, b) ((float)((a) / (b)))
#define TSVD_FMA(a, b, c) fmaf((a), (b), (c))
#define TSVD_FSQRT(a) sqrtf(a)
#define TSVD_RINT(a) rintf(a)
#endif

TSVD_HD uint32_t tsvd_f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
TSVD_HD float tsvd_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

typedef struct {
  uint32_t v[4];
} tsvd_philox4;

TSVD_HD void tsvd_mulhilo(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds; multipliers and Weyl key increments as published. */
TSVD_HD tsvd_philox4 tsvd_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                         uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    tsvd_mulhilo(M0, c0, &hi0, &lo0);
    tsvd_mulhilo(M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  tsvd_philox4 out;
  out.v[0] = c0;
  out.v[1] = c1;
  out.v[2] = c2;
  out.v[3] = c3;
  return out;
}

/* Natural log for x in (0, 1]: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
 * ln m = 2 atanh(t), t = (m-1)/(m+1), |t| < 0.1716, atanh by its series. */
TSVD_HD float tsvd_lnf(float x) {
  uint32_t bits = tsvd_f2u(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = tsvd_u2f((bits & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
  if (m > 1.41421356f) {
    m = TSVD_FMUL(m, 0.5f);
    e += 1;
  }
  float t = TSVD_FDIV(TSVD_FSUB(m, 1.0f), TSVD_FADD(m, 1.0f));
  float t2 = TSVD_FMUL(t, t);
  /* 1 + t2/3 + t2^2/5 + t2^3/7 + t2^4/9 + t2^5/11 (Horner) */
  float s = TSVD_FMA(t2, 0.0909090909f, 0.111111111f);
  s = TSVD_FMA(t2, s, 0.142857143f);
  s = TSVD_FMA(t2, s, 0.2f);
  s = TSVD_FMA(t2, s, 0.333333333f);
  s = TSVD_FMA(t2, s, 1.0f);
  float lnm = TSVD_FMUL(TSVD_FMUL(2.0f, t), s);
  const float LN2_HI = 0.693145752f;   /* ln 2 split: hi has 16 significant bits */
  const float LN2_LO = 1.42860677e-06f;
  float fe = (float)e;
  return TSVD_FADD(TSVD_FMUL(fe, LN2_HI), TSVD_FMA(fe, LN2_LO, lnm));
}

/* sin and cos of 2*pi*u for u in [0, 1): reduce to x = 2*pi*(u - q/4) with
 * |x| <= pi/4 (the subtraction is exact), Taylor polynomials, quadrant swap. */
TSVD_HD void tsvd_sincos_2pi(float u, float *sn, float *cs) {
  int q = (int)TSVD_RINT(TSVD_FMUL(u, 4.0f));
  float f = TSVD_FSUB(u, TSVD_FMUL((float)q, 0.25f));
  float x = TSVD_FMUL(f, 6.28318531f);
  float x2 = TSVD_FMUL(x, x);
  /* sin x = x (1 - x2/6 + x2^2/120 - x2^3/5040 + x2^4/362880) */
  float ps = TSVD_FMA(x2, 2.75573192e-06f, -1.98412698e-04f);
  ps = TSVD_FMA(x2, ps, 8.33333333e-03f);
  ps = TSVD_FMA(x2, ps, -1.66666667e-01f);
  ps = TSVD_FMA(x2, ps, 1.0f);
  float s = TSVD_FMUL(x, ps);
  /* cos x = 1 - x2/2 + x2^2/24 - x2^3/720 + x2^4/40320 - x2^5/3628800 */
  float pc = TSVD_FMA(x2, -2.75573192e-07f, 2.48015873e-05f);
  pc = TSVD_FMA(x2, pc, -1.38888889e-03f);
  pc = TSVD_FMA(x2, pc, 4.16666667e-02f);
  pc = TSVD_FMA(x2, pc, -0.5f);
  float c = TSVD_FMA(x2, pc, 1.0f);
  switch (q & 3) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

/* Round a float to the nearest half-precision value (ties to even), returned
 * as float. Inputs here are |x| < 6, far from the half overflow. */
TSVD_HD float tsvd_round_half(float x) {
  uint32_t bits = tsvd_f2u(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  if (e < -14) { /* half subnormal range: quantum 2^-24 */
    return TSVD_FMUL(TSVD_RINT(TSVD_FMUL(x, 16777216.0f)), 5.9604644775390625e-08f);
  }
  float ulp = tsvd_u2f((uint32_t)(e - 10 + 127) << 23);
  float inv = tsvd_u2f((uint32_t)(10 - e + 127) << 23);
  return TSVD_FMUL(TSVD_RINT(TSVD_FMUL(x, inv)), ulp);
}

/* Entry (row, col) of the Gaussian test matrix of `stream` under `seed`.
 * Columns 2j and 2j+1 share one Philox call (the Box-Muller pair). */
TSVD_HD float tsvd_gauss_entry(uint64_t seed, uint32_t stream, uint32_t row,
                               uint32_t col) {
  tsvd_philox4 r = tsvd_philox4x32_10(row, col >> 1, stream, 0x54535644u,
                                      (uint32_t)seed, (uint32_t)(seed >> 32));
  float u1 = TSVD_FMUL((float)((r.v[0] >> 8) + 1u), 5.9604644775390625e-08f); /* (0,1] */
  float u2 = TSVD_FMUL((float)(r.v[1] >> 8), 5.9604644775390625e-08f);        /* [0,1) */
  float rad = TSVD_FSQRT(TSVD_FMUL(-2.0f, tsvd_lnf(u1)));
  float sn, cs;
  tsvd_sincos_2pi(u2, &sn, &cs);
  float z = (col & 1u) ? TSVD_FMUL(rad, sn) : TSVD_FMUL(rad, cs);
  return tsvd_round_half(z);
}

/* Uniform 32-bit words for host-side generators (R-MAT, sampling). */
TSVD_HD uint32_t tsvd_rand_u32(uint64_t seed, uint32_t stream, uint64_t idx,
                               uint32_t lane) {
  tsvd_philox4 r = tsvd_philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32),
                                      stream, 0x524d4154u, (uint32_t)seed,
                                      (uint32_t)(seed >> 32));
  return r.v[lane & 3];
}

#endif /* TSVD_PHILOX_GAUSS_H */
