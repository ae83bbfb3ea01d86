// Batched FP32 GEMM for the wide merge: C = op(A) B with op(A) = A or A^T,
// row-major operands, problem z at offset z * stride of each operand.
//
// The merges wider than 256 columns (the reference's run.sh arity 8,
// Code/Tree_u_NC.cpp:723-850) run a subspace iteration whose products are
// plain fp32 GEMMs of at most |S| x 2048 by 2048 x 256; 64 x 64 output tiles
// give ~190 CTAs per problem at |S| = 3000, so no split of K is needed and
// every output element is a fixed-order fp32 sum (deterministic). Each of the
// 256 threads owns a 4 x 4 sub-tile; A and B tiles of 16 values of K are
// staged in shared memory, A transposed to [k][m] so both operands are read
// as float4 rows of the k-th slice.
#include <algorithm>

#include "internal.h"

namespace tsvd {

namespace {

constexpr int TM = 64, TN = 64, TK = 16;

template <bool TRANS_A>
__global__ void __launch_bounds__(256) sgemm_kernel(int M, int N, int K, const float *__restrict__ A,
                                                    int lda, int64_t sa, const float *__restrict__ B,
                                                    int ldb, int64_t sb, float *__restrict__ C,
                                                    int ldc, int64_t sc) {
  __shared__ __align__(16) float As[TK][TM + 4];
  __shared__ __align__(16) float Bs[TK][TN + 4];
  const int z = blockIdx.z;
  A += z * sa;
  B += z * sb;
  C += z * sc;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TK) {
    // A tile -> As[k][m]: 64 x 16 values, four per thread
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + q * 256;
      int mm, kk;
      if (TRANS_A) {  // A is K x M: a row of 64 m values per k
        kk = e >> 6;
        mm = e & 63;
      } else {        // A is M x K: a row of 16 k values per m
        mm = e >> 4;
        kk = e & 15;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TRANS_A ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      As[kk][mm] = v;
    }
    // B tile -> Bs[k][n]: 16 x 64 values
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + q * 256;
      const int kk = e >> 6, nn = e & 63;
      const int gk = k0 + kk, gn = n0 + nn;
      Bs[kk][nn] = (gk < K && gn < N) ? B[(int64_t)gk * ldb + gn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      const float4 a = *reinterpret_cast<const float4 *>(&As[kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4 *>(&Bs[kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn < N) C[(int64_t)gm * ldc + gn] = acc[i][j];
    }
  }
}

}  // namespace

tsvd_status sgemm_batched(bool trans_a, int M, int N, int K, const float *A, int lda, int64_t sa,
                          const float *B, int ldb, int64_t sb, float *C, int ldc, int64_t sc,
                          int nprob, cudaStream_t st) {
  if (M <= 0 || N <= 0 || nprob <= 0) return TSVD_OK;
  if (nprob > 65535) return fail(TSVD_ERR_INVALID, "sgemm: %d problems", nprob);
  const dim3 grid((unsigned)ceil_div(N, TN), (unsigned)ceil_div(M, TM), (unsigned)nprob);
  if (trans_a)
    sgemm_kernel<true><<<grid, 256, 0, st>>>(M, N, K, A, lda, sa, B, ldb, sb, C, ldc, sc);
  else
    sgemm_kernel<false><<<grid, 256, 0, st>>>(M, N, K, A, lda, sa, B, ldb, sb, C, ldc, sc);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

}  // namespace tsvd
