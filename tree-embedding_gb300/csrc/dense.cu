// Dense kernels of the blockwise randomized SVD and the tree merge.
//
//  gemm_fwd / gemm_bwd : the two products of every frPCA pass,
//      Y = A X   and   Z = A^T Y   (Code/frpca.c:259,280,282,294 via
//      csr_matrix_{,transpose_}matrix_mult, ..._ext.c:364-398),
//    with A stored once per block as A^T in half precision (vertex-major, the
//    layout the PPR state has) and the skinny operand split into hi + lo
//    halves so that it keeps ~22 significant bits. 5th-generation tensor
//    cores: tcgen05.mma kind::f16 into a tensor-memory accumulator (fp32),
//    operands brought into shared memory by TMA (cp.async.bulk.tensor) in a
//    5-stage pipeline of full / empty mbarriers.
//  gram_batched : X^T X with error-free products and compensated sums per
//    row chunk, chunks summed in fp64 (Code/frpca.c:101, cblas_dgemm TN).
//  chol_inverse_batched / apply_right_batched : CholeskyQR2 normalization,
//    replacing LUfraction (Code/frpca.c:4-41); the span of the basis, which
//    is all the power iteration keeps, is the same.
//  jacobi_eig_batched : two-sided cyclic Jacobi on the Gram, its rows spread
//    over the shared memory of a thread-block cluster, replacing
//    LAPACKE_dsyevd (frpca.c:102) and the Gram route to LAPACKE_dgesvd
//    (..._mkl.c:1278) for the merge.
#include <algorithm>
#include <map>
#include <mutex>
#include <cfloat>
#include <cstring>

#include <cooperative_groups.h>

#include "internal.h"
#include "jacobi_sched.h"

namespace tsvd {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
// ------------------------------------------------------------------ GEMM tiles
// The two frPCA products run on the 5th-generation tensor cores: one CTA
// computes three 128 x 144 fp32 tiles in tensor memory (TMEM) with tcgen05.mma
// kind::f16, issued by one thread. The operand tiles are brought into shared
// memory by the Tensor Memory Accelerator: one producer thread issues
// cp.async.bulk.tensor copies whose completion is counted (in bytes) on the
// stage's "full" mbarrier; the MMA thread waits on it, issues the stage's
// MMAs and commits them to the stage's "empty" mbarrier, which the producer
// waits on before refilling the stage. Four stages of 32 K values are in
// flight.
//
// Shared-memory layouts are the swizzled canonical ones of the tensor cores,
// written by the TMA with the matching swizzle, so that every copy moves
// whole 64- or 128-byte rows:
//  * skinny operand (hi and lo halves, [k][144] in global memory, MN-major):
//    three 64-column atoms of 32 K rows x 128 bytes, 128-byte swizzle
//    (columns 144-191 of the third atom are outside the tensor: zeros, never
//    read by an N = 144 MMA). Descriptor: LBO = 4 KB between atoms along N,
//    SBO = 1 KB between 8-row groups along K;
//  * A of the forward product (A^T [n_c][Sp]: M = Sp contiguous, MN-major):
//    six 64-row atoms of 32 K rows x 128 bytes, 128-byte swizzle; row tile h
//    is atoms 2h, 2h + 1 (LBO 4 KB, SBO 1 KB);
//  * A of the backward product (A^T rows are M, K = Sp contiguous, K-major):
//    one 128-row x 64-byte box per row tile, 64-byte swizzle (SBO = 512
//    bytes between 8-row groups); the second 16-deep K step starts 32 bytes
//    into the rows.
// Rows past a block's n_c and K past its end lie outside the tensors, and the
// TMA fills them with zeros. Every copy starts at an innermost coordinate
// that is a multiple of 8 values (16 bytes).
constexpr int BM = 128, MH = 3, BN = kLp, BK = 32, STAGES = 4, GEMM_THREADS = 128;
constexpr int kAtom = 64;                              // values per 128-byte swizzle row
constexpr int kAtomBytes = BK * 128;                   // one 32-row x 128-byte atom: 4 KB
constexpr int kBAtoms = (BN + kAtom - 1) / kAtom;      // 3
constexpr int SA_BYTES = BM * BK * 2;                  // 8 KB per row tile (two atoms)
constexpr int SB_BYTES = kBAtoms * kAtomBytes;         // 12 KB per skinny half
constexpr int STAGE_BYTES = MH * SA_BYTES + 2 * SB_BYTES;
constexpr size_t kGemmSmem = (size_t)STAGES * STAGE_BYTES + 2048;  // + alignment slack, barriers
constexpr int kLayoutSw128 = 2, kLayoutSw64 = 4;       // descriptor swizzle modes
constexpr int kTmemCols = 512;                         // MH accumulators, kAccStride apart
constexpr int kAccStride = 160;
static_assert(MH * kAccStride <= kTmemCols && kAccStride >= BN, "accumulators fit in TMEM");
static_assert(BN % 16 == 0 && BN <= 256, "tcgen05.mma with M = 128 needs N % 16 == 0, N <= 256");
static_assert(STAGE_BYTES % 1024 == 0 && SA_BYTES % 1024 == 0 && kAtomBytes % 1024 == 0,
              "swizzle atoms stay 1024-byte aligned");
static_assert(BM % kAtom == 0 && SA_BYTES == 2 * kAtomBytes, "a row tile is two atoms");

// Counts waits that ran out (a kernel that gives up skips its tile and
// frees its tensor memory; the host turns a non-zero count into an error).
__device__ int g_umma_timeouts = 0;

// tcgen05 shared-memory descriptor: start, leading / stride byte offsets (16-
// byte units), version 1, base offset 0, swizzle mode.
__device__ __forceinline__ uint64_t umma_smem_desc(uint32_t saddr, int lbo, int sbo, int layout) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)(layout & 7) << 61;
  return d;
}

// kind::f16 instruction descriptor: fp32 accumulator, fp16 A and B, A K-major
// (0) or MN-major (1), B MN-major, N = BN, M = BM.
__host__ __device__ constexpr uint32_t umma_idesc(int a_mn) {
  return (1u << 4) | ((uint32_t)a_mn << 15) | (1u << 16) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 24); ++it)
    if (mbar_try(bar, parity)) return true;
  return false;
}

// The same wait, also ending (false) once the CTA's failure flag is set.
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t bar, uint32_t parity,
                                                  volatile int *failed) {
  for (int it = 0; it < (1 << 24); ++it) {
    if (mbar_try(bar, parity)) return true;
    if (*failed) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

struct GemmArgs {
  const CUtensorMap *maps;  // 3 per problem: A, skinny hi, skinny lo
  const int32_t *ncols;
  int lda;  // Sp
  int has_lo;
  float *const *out;
  float scale;
  int splits;  // fwd split-K
};

// FWD: Y (Sp x BN) [+]= A (Sp x nc) * X (nc x BN), A given as A^T [nc][lda].
// BWD: Z (nc x BN) = A^T (nc x Sp) * Y (Sp x BN).
// The skinny operand is hi (+ lo), both accumulated into the same tile.
template <bool FWD>
__global__ void __launch_bounds__(GEMM_THREADS, 1) umma_gemm_kernel(GemmArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // swizzle atoms must sit on 1024-byte boundaries of the shared window
  unsigned char *stage_base =
      smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(stage_base + (size_t)STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(empty + STAGES);
  volatile int *failed = reinterpret_cast<volatile int *>(tslot + 1);
  const int prob = blockIdx.z;
  const int nc = a.ncols[prob];
  const int m0 = blockIdx.x * (BM * MH);
  const int mrows = FWD ? a.lda : nc;  // rows of the output
  if (m0 >= mrows) return;
  const int nk_total = FWD ? (nc + BK - 1) / BK : a.lda / BK;
  const int per = (nk_total + a.splits - 1) / a.splits;
  const int kt0 = blockIdx.y * per, kt1 = min(nk_total, kt0 + per);
  if (kt0 >= kt1) return;
  const int nk = kt1 - kt0;
  const CUtensorMap *map_a = a.maps + 3 * (int64_t)prob;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t tx_bytes = MH * SA_BYTES + (a.has_lo ? 2 : 1) * SB_BYTES;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(full + s), 1);
      mbar_init(smem_u32(empty + s), 1);
    }
    *failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(tslot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    // producer: fill stage i % STAGES with K tile kt0 + i once the MMAs that
    // read its previous contents (tile i - STAGES) have completed
    for (int j = 0; j < 3; ++j)
      asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(map_a + j))
                   : "memory");
    int filled = 0;
    for (int i = 0; i < nk; ++i) {
      const int st = i % STAGES;
      if (i >= STAGES &&
          !mbar_wait_or_fail(smem_u32(empty + st), (uint32_t)((i / STAGES - 1) & 1), failed)) {
        *failed = 1;
        break;
      }
      const uint32_t fb = smem_u32(full + st);
      const uint32_t sa = smem_u32(stage_base + (size_t)st * STAGE_BYTES);
      const int k0 = (kt0 + i) * BK;
      mbar_expect_tx(fb, tx_bytes);
      if (FWD) {  // six 64-row atoms of M at K rows k0 .. k0 + 31
#pragma unroll
        for (int t = 0; t < MH * BM / kAtom; ++t)
          tma_load_2d(sa + t * kAtomBytes, map_a, m0 + t * kAtom, k0, fb);
      } else {  // per row tile: 128 rows of M, K values k0 .. k0 + 31
#pragma unroll
        for (int h = 0; h < MH; ++h) tma_load_2d(sa + h * SA_BYTES, map_a, k0, m0 + h * BM, fb);
      }
#pragma unroll
      for (int t = 0; t < kBAtoms; ++t) {
        tma_load_2d(sa + MH * SA_BYTES + t * kAtomBytes, map_a + 1, t * kAtom, k0, fb);
        if (a.has_lo)
          tma_load_2d(sa + MH * SA_BYTES + SB_BYTES + t * kAtomBytes, map_a + 2, t * kAtom, k0, fb);
      }
      filled = i + 1;
    }
    // no copy may still be writing shared memory when the CTA exits: wait for
    // the last fill of every stage (those the MMA thread consumed are done)
    for (int i = max(0, filled - STAGES); i < filled; ++i)
      if (!mbar_wait(smem_u32(full + i % STAGES), (uint32_t)((i / STAGES) & 1))) *failed = 1;
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = umma_idesc(FWD ? 1 : 0);
    // per 16-deep K step: MN-major tiles advance two 8-row groups (2 KB),
    // the K-major A 32 bytes along its rows
    constexpr int a_lbo = FWD ? kAtomBytes : 16, a_sbo = FWD ? 1024 : 512;
    constexpr int a_layout = FWD ? kLayoutSw128 : kLayoutSw64, a_kstep = FWD ? 2048 : 32;
    int issued = 0;
    for (int i = 0; i < nk; ++i) {
      const int st = i % STAGES;
      if (!mbar_wait_or_fail(smem_u32(full + st), (uint32_t)((i / STAGES) & 1), failed)) {
        *failed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t sa = smem_u32(stage_base + (size_t)st * STAGE_BYTES);
      const uint32_t sbh = sa + MH * SA_BYTES, sbl = sbh + SB_BYTES;
#pragma unroll
      for (int ks = 0; ks < BK / 16; ++ks) {
        const uint64_t bdh = umma_smem_desc(sbh + ks * 2048, kAtomBytes, 1024, kLayoutSw128);
        const uint64_t bdl = umma_smem_desc(sbl + ks * 2048, kAtomBytes, 1024, kLayoutSw128);
        const uint32_t acc0 = (i > 0 || ks > 0) ? 1u : 0u;
#pragma unroll
        for (int h = 0; h < MH; ++h) {
          const uint64_t ad =
              umma_smem_desc(sa + h * SA_BYTES + ks * a_kstep, a_lbo, a_sbo, a_layout);
          const uint32_t td = tmem + (uint32_t)(h * kAccStride);
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(td),
              "l"(ad), "l"(bdh), "r"(idesc), "r"(acc0));
          if (a.has_lo)
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(td),
                "l"(ad), "l"(bdl), "r"(idesc), "r"(1u));
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smem_u32(empty + st))
          : "memory");
      issued = i + 1;
    }
    // the last commit covers every MMA issued before it; wait for it even
    // after a failure, so no MMA still writes the tensor memory freed below
    if (issued > 0) {
      const int li = issued - 1;
      if (!mbar_wait(smem_u32(empty + li % STAGES), (uint32_t)((li / STAGES) & 1))) *failed = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const bool ok = *failed == 0;
  if (!ok) {
    if (lane == 0) atomicAdd(&g_umma_timeouts, 1);
  } else {
    // epilogue: warp w reads TMEM lanes 32w..32w+31 of accumulator h = output
    // rows m0 + 128 h + 32 w + lane
    float *out = a.out[prob];
    const bool atomic = FWD && a.splits > 1;
#pragma unroll 1
    for (int h = 0; h < MH; ++h) {
      const int row = m0 + h * BM + warp * 32 + lane;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 16) {
        uint32_t v[16];
        const uint32_t ta =
            tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(h * kAccStride + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
            "%14,%15}, [%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
              "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (row < mrows) {
          float *o = out + (int64_t)row * BN + c0;
          if (atomic) {  // split-K partial tiles: float4 reductions (rows are 576-byte aligned)
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              atomicAdd(reinterpret_cast<float4 *>(o + j),
                        make_float4(__uint_as_float(v[j]) * a.scale,
                                    __uint_as_float(v[j + 1]) * a.scale,
                                    __uint_as_float(v[j + 2]) * a.scale,
                                    __uint_as_float(v[j + 3]) * a.scale));
          } else {
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              *reinterpret_cast<float4 *>(o + j) = make_float4(
                  __uint_as_float(v[j]) * a.scale, __uint_as_float(v[j + 1]) * a.scale,
                  __uint_as_float(v[j + 2]) * a.scale, __uint_as_float(v[j + 3]) * a.scale);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "n"(kTmemCols));
}

// ------------------------------------------------------------------ Gram
// Error-free product + TwoSum accumulation (Ogita, Rump, Oishi, "Accurate sum
// and dot product", SISC 2005): s + c carries the chunk sum to ~2^-44.
struct Comp {
  float s, c;
};
__device__ __forceinline__ void comp_add(Comp &acc, float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  float t = acc.s + p;
  float z = t - acc.s;
  float err = (acc.s - (t - z)) + (p - z);
  acc.s = t;
  acc.c += err + e;
}

constexpr int GRAM_MIN_ROWS = 128;    // rows per CTA at least (one fp64 partial per chunk)
constexpr int GRAM_MAX_CHUNKS = 2048;  // chunks over all problems (bounds the work buffer)
constexpr int GRAM_SUB = 32;      // rows staged in smem at a time
constexpr int GRAM_THREADS = 256;
constexpr int GRAM_TPT = 1;       // 4x4 output tiles per thread (79 registers: 3 CTAs per SM)
constexpr int GRAM_TILES_PER_CTA = GRAM_THREADS * GRAM_TPT;
constexpr int GRAM_LMAX = 256;

struct GramArgs {
  const float *const *x;
  const int32_t *rows;
  int ld;
  int l;
  int tiles;      // ceil(l/4)
  int nchunks;    // per problem
  int chunk_rows;
  double *work;   // [prob][chunk][l*l]
};

// grid: (row chunk, tile group, problem). Each thread owns <= 2 upper-triangle
// 4x4 tiles of the l x l output and accumulates them over the chunk's rows.
__global__ void __launch_bounds__(GRAM_THREADS) gram_partial_kernel(GramArgs a) {
  extern __shared__ __align__(16) float sx[];  // [GRAM_SUB][ld]
  const int prob = blockIdx.z, chunk = blockIdx.x;
  const int rows = a.rows[prob];
  const int r0 = chunk * a.chunk_rows;
  double *out = a.work + ((int64_t)prob * a.nchunks + chunk) * a.l * a.l;
  const int T = a.tiles;
  const int ntile_pairs = T * (T + 1) / 2;
  const float *x = a.x[prob];
  const int r1 = min(rows, r0 + a.chunk_rows);
  Comp acc[GRAM_TPT][16];
  int ti[GRAM_TPT], tj[GRAM_TPT];
  int my = 0;
#pragma unroll
  for (int k = 0; k < GRAM_TPT; ++k) {
    int t = blockIdx.y * GRAM_TILES_PER_CTA + k * GRAM_THREADS + threadIdx.x;
    ti[k] = tj[k] = 0;
    if (t < ntile_pairs) {
      int J = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
      while ((J + 1) * (J + 2) / 2 <= t) ++J;
      while (J * (J + 1) / 2 > t) --J;
      int I = t - J * (J + 1) / 2;
      ti[k] = I * 4;
      tj[k] = J * 4;
      my = k + 1;
    }
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[k][e] = Comp{0.f, 0.f};
  }
  const int sld = 4 * T;  // staged row stride covers every 4x4 tile column
  for (int rb = r0; rb < r1; rb += GRAM_SUB) {
    const int nr = min(GRAM_SUB, r1 - rb);
    __syncthreads();
    for (int i = threadIdx.x; i < GRAM_SUB * sld; i += blockDim.x) {
      int rr = i / sld, cc = i % sld;
      sx[i] = (rr < nr && cc < a.l) ? x[(int64_t)(rb + rr) * a.ld + cc] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GRAM_TPT; ++k) {
      if (k >= my) break;
      for (int rr = 0; rr < nr; ++rr) {
        const float *row = sx + rr * sld;
        float xi[4], xj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          xi[q] = row[ti[k] + q];
          xj[q] = row[tj[k] + q];
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) comp_add(acc[k][p * 4 + q], xi[p], xj[q]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < GRAM_TPT; ++k) {
    if (k >= my) break;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int i = ti[k] + p, j = tj[k] + q;
        if (i >= a.l || j >= a.l) continue;
        double v = (double)acc[k][p * 4 + q].s + (double)acc[k][p * 4 + q].c;
        out[i * a.l + j] = v;
        out[j * a.l + i] = v;
      }
  }
}

__global__ void gram_reduce_kernel(const double *__restrict__ work, int nchunks, int l,
                                   double *const *g, int nprob) {
  const int prob = blockIdx.y;
  const int64_t ll = (int64_t)l * l;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ll;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    const double *w = work + (int64_t)prob * nchunks * ll + i;
    for (int c = 0; c < nchunks; ++c) s += w[c * ll];
    g[prob][i] = s;
  }
}

// ------------------------------------------------------------------ Cholesky
constexpr int CHOL_THREADS = 512;
__global__ void __launch_bounds__(CHOL_THREADS) chol_inverse_kernel(double *const *gs,
                                                                    float *const *ts, int l) {
  extern __shared__ __align__(16) float sm[];
  const int LD = l + 1;
  float *L = sm;              // [l][LD]
  float *Li = sm + l * LD;    // [l][LD]
  __shared__ int drop[kLp];
  __shared__ float tol;
  const double *G = gs[blockIdx.x];
  float *T = ts[blockIdx.x];
  for (int i = threadIdx.x; i < l * l; i += blockDim.x) {
    int r = i / l, c = i % l;
    L[r * LD + c] = (float)G[i];
    Li[r * LD + c] = 0.f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float mx = 0.f;
    for (int i = 0; i < l; ++i) mx = fmaxf(mx, L[i * LD + i]);
    tol = mx * 1e-12f;
  }
  __syncthreads();
  for (int k = 0; k < l; ++k) {
    if (threadIdx.x == 0) {
      float d = L[k * LD + k];
      if (!(d > tol) || !(d > 0.f)) {
        drop[k] = 1;
        L[k * LD + k] = 1.f;
      } else {
        drop[k] = 0;
        L[k * LD + k] = sqrtf(d);
      }
    }
    __syncthreads();
    const float piv = L[k * LD + k];
    const int dk = drop[k];
    for (int i = k + 1 + threadIdx.x; i < l; i += blockDim.x)
      L[i * LD + k] = dk ? 0.f : L[i * LD + k] / piv;
    __syncthreads();
    const int n = l - k - 1;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      int i = k + 1 + t / n, j = k + 1 + t % n;
      if (j <= i) L[i * LD + j] -= L[i * LD + k] * L[j * LD + k];
    }
    __syncthreads();
  }
  // Li = L^{-1} by forward substitution, one column per thread.
  for (int j = threadIdx.x; j < l; j += blockDim.x) {
    Li[j * LD + j] = 1.f / L[j * LD + j];
    for (int i = j + 1; i < l; ++i) {
      float s = 0.f;
      for (int k = j; k < i; ++k) s += L[i * LD + k] * Li[k * LD + j];
      Li[i * LD + j] = -s / L[i * LD + i];
    }
  }
  __syncthreads();
  // T = R^{-1} = (L^{-1})^T, dropped directions zeroed.
  for (int i = threadIdx.x; i < l * kLp; i += blockDim.x) {
    int r = i / kLp, c = i % kLp;
    float v = 0.f;
    if (c < l && r < l && c >= r && !drop[c]) v = Li[c * LD + r];
    T[i] = v;
  }
}

// ------------------------------------------------------------------ X * W
// Y = X W diag(colscale) (rows x n_out, written up to ldy <= 144 columns,
// zero past n_out), optionally split into fp16 hi/lo. Register tiles: 256
// threads as 16 x 16, each thread 4 rows x 9 columns (c = tx + 16 j) of a
// 64-row tile; per k one float4 of X (the tile is staged transposed) and
// nine loads of W feed 36 FMAs. A CTA walks a contiguous range of
// (problem, row tile) items and restages W only when the problem changes.
// X may alias Y (in-place CholeskyQR): a tile is read whole before it is
// written.
constexpr int APPLY_RT = 64;          // rows per tile
constexpr int APPLY_THREADS = 256;
constexpr int APPLY_CJ = 9;           // columns per thread
constexpr int APPLY_WLD = 16 * APPLY_CJ;  // 144: staged W row
constexpr int APPLY_XLD = APPLY_RT + 4;   // transposed X tile row (16-byte aligned)
struct ApplyArgs {
  const float *const *x;
  const int32_t *rows;
  int ldx;
  const float *const *w;
  int ldw;
  int n_in, n_out;
  const float *const *colscale;
  float *const *y;
  int ldy;
  __half *const *yhi;
  __half *const *ylo;
  float split_scale;
  int tiles;  // row tiles per problem (of the largest)
  int nprob;
};

__global__ void __launch_bounds__(APPLY_THREADS) apply_right_kernel(ApplyArgs a) {
  extern __shared__ __align__(16) float sm[];
  float *sw = sm;                               // [n_in][APPLY_WLD]
  float *sxt = sm + a.n_in * APPLY_WLD;         // [n_in][APPLY_XLD] (X tile transposed)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t items = (int64_t)a.nprob * a.tiles;
  const int64_t per = (items + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = blockIdx.x * per, i1 = min(items, i0 + per);
  int cur = -1;
  for (int64_t it = i0; it < i1; ++it) {
    const int prob = (int)(it / a.tiles), r0 = (int)(it % a.tiles) * APPLY_RT;
    const int rows = a.rows[prob];
    if (r0 >= rows) continue;  // the same for every thread
    __syncthreads();           // the previous tile is written out
    if (prob != cur) {
      const float *W = a.w[prob];
      const float *cs = a.colscale ? a.colscale[prob] : nullptr;
      for (int i = threadIdx.x; i < a.n_in * APPLY_WLD; i += blockDim.x) {
        const int r = i / APPLY_WLD, c = i % APPLY_WLD;
        sw[i] = c < a.n_out ? W[(int64_t)r * a.ldw + c] * (cs ? cs[c] : 1.f) : 0.f;
      }
      cur = prob;
    }
    const float *X = a.x[prob];
    for (int i = threadIdx.x; i < APPLY_RT * a.n_in; i += blockDim.x) {
      const int rr = i / a.n_in, k = i % a.n_in;
      sxt[k * APPLY_XLD + rr] = r0 + rr < rows ? X[(int64_t)(r0 + rr) * a.ldx + k] : 0.f;
    }
    __syncthreads();
    float acc[4][APPLY_CJ];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int j = 0; j < APPLY_CJ; ++j) acc[r][j] = 0.f;
    for (int k = 0; k < a.n_in; ++k) {
      const float4 xv = *reinterpret_cast<const float4 *>(sxt + k * APPLY_XLD + ty * 4);
      const float *wr = sw + k * APPLY_WLD + tx;
#pragma unroll
      for (int j = 0; j < APPLY_CJ; ++j) {
        const float wv = wr[16 * j];
        acc[0][j] = fmaf(xv.x, wv, acc[0][j]);
        acc[1][j] = fmaf(xv.y, wv, acc[1][j]);
        acc[2][j] = fmaf(xv.z, wv, acc[2][j]);
        acc[3][j] = fmaf(xv.w, wv, acc[3][j]);
      }
    }
    float *Y = a.y[prob];
    __half *Yh = a.yhi ? a.yhi[prob] : nullptr;
    __half *Yl = a.ylo ? a.ylo[prob] : nullptr;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int row = r0 + ty * 4 + r;
      if (row >= rows) continue;
#pragma unroll
      for (int j = 0; j < APPLY_CJ; ++j) {
        const int c = tx + 16 * j;
        if (c >= a.ldy) continue;
        const float v = acc[r][j];  // zero past n_out (W staged as zero there)
        Y[(int64_t)row * a.ldy + c] = v;
        if (Yh) {
          const float sv = v * a.split_scale;
          const __half h = __float2half_rn(sv);
          Yh[(int64_t)row * a.ldy + c] = h;
          Yl[(int64_t)row * a.ldy + c] = __float2half_rn(sv - __half2float(h));
        }
      }
    }
  }
}

// ------------------------------------------------------------------ Jacobi
constexpr int JAC_THREADS = 1024;
constexpr int JAC_MAX_SWEEPS = 30;
constexpr int kJacMaxCluster = 8;  // CTAs per eigenproblem (portable cluster size)
constexpr int kJacRotBase = 512;   // first thread computing rotations (P <= 128 of them)
constexpr int kJacSendBase = 768;  // first thread broadcasting (2 L <= 256 rows)

struct JacobiArgs {
  double *const *g;
  int n;
  float *const *lambda;
  float2 *log;        // [prob][JAC_MAX_SWEEPS][np-1][np/2]
  int32_t *sweeps;    // [prob]
  int32_t *rank;      // [prob][n]
  int refine;         // 1: the diagonal is carried in fp64 (see jacobi_kernel)
  const float *const *vinit;  // replay starts from these rows (null: identity)
};

// Shared-memory layout of one CTA of jacobi_kernel (C CTAs per problem).
struct JacobiSmem {
  int n, np, P, L, nbuf;
  size_t off_dbase, off_lam, off_rows, off_pc, off_ps, off_pt, off_diag, off_coup, off_top,
      off_bot, off_flag, bytes;
  __host__ __device__ JacobiSmem(int n_, int C) {
    n = n_;
    np = n + (n & 1);
    P = np / 2;
    L = (P + C - 1) / C;
    nbuf = 2 * L + 4;  // the rows of the owned slots' players, mailboxes [2 parities][L, R]
    size_t o = 0;
    off_dbase = o; o += (size_t)np * sizeof(double);
    off_lam = o; o += (size_t)np * sizeof(double);
    off_rows = o; o += (size_t)nbuf * np * sizeof(float);
    off_pc = o; o += (size_t)P * sizeof(float);
    off_ps = o; o += (size_t)P * sizeof(float);
    off_pt = o; o += (size_t)P * sizeof(float);
    off_diag = o; o += (size_t)2 * np * sizeof(float);  // [parity][player]
    off_coup = o; o += (size_t)2 * P * sizeof(float);   // [parity][slot]
    off_top = o; o += (size_t)2 * L * sizeof(int);      // two map pairs (renamed each round)
    off_bot = o; o += (size_t)2 * L * sizeof(int);
    off_flag = o; o += (size_t)(JAC_MAX_SWEEPS + 1) * sizeof(int);
    bytes = (o + 15) & ~(size_t)15;
  }
};

// One symmetric eigenproblem per thread-block cluster of C CTAs: cyclic
// two-sided Jacobi in the round-robin order of circle_player (np/2 disjoint
// pairs per round, np - 1 rounds per sweep). CTA c owns the pair slots
// [c L, c L + L) and holds the full rows (indexed by player, so a warp's
// lanes touch consecutive words) of the two players of each owned slot.
// A round: every CTA applies all of the round's rotations to its rows, 2 x 2
// block by block (G <- J_k1^T G J_k2, each entry summed in an order that is
// the same for its transposed twin, so the two copies of an entry that
// different CTAs hold stay equal); then the schedule advances: each CTA
// passes one row to each neighbour (into the neighbour's mailbox, in
// distributed shared memory) and broadcasts, for every row it holds, the
// diagonal entry and the coupling to the row's next partner; after the one
// cluster barrier of the round, each CTA renames its rows (circle_arrivals,
// circle_next) and computes all rotations of the next round itself, from the
// same values in the same order, so every CTA has the same rotations without
// a second exchange. Mailboxes and broadcast values alternate between two
// buffers by round parity, so a fast CTA never overwrites what a slow one
// has yet to read.
//
// Rotate when the pair is coupled: relative to the pair (Demmel-Veselic) and
// above an absolute floor. The first pass only resolves the couplings above
// 1e-5 of max|a_ii| (a few sweeps: the Grams of merges and of frPCA's Z are
// nearly diagonal at that scale); it settles in fp32 the strong couplings
// whose small eigenvalues come from cancellation, which H = V^T G V then
// recomputes in fp64. Refinement mode (a.refine): g = H, the diagonal is kept
// as an fp64 base (dbase, fixed) plus an fp32 correction in the rows, so the
// small eigenvalues keep their relative accuracy: the rotation angle uses
// (dbase_q - dbase_p) rounded once, and the updates only move the
// corrections. The eigenvalues span 1e-7 of the largest, so below 1e-4 of it
// most pairs are still coupled; the refinement's floor (1e-11 of max|a_ii|)
// sits above the fp32 rounding its own rotations leave, so the tiny
// eigenvalues' pairs cannot cycle.
__global__ void __launch_bounds__(JAC_THREADS) jacobi_kernel(JacobiArgs a) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char jsm[];
  const int C = (int)cluster.num_blocks(), crank = (int)cluster.block_rank();
  const JacobiSmem lay(a.n, C);
  const int n = lay.n, np = lay.np, P = lay.P, L = lay.L;
  double *dbase = reinterpret_cast<double *>(jsm + lay.off_dbase);
  double *lam_all = reinterpret_cast<double *>(jsm + lay.off_lam);
  float *rows = reinterpret_cast<float *>(jsm + lay.off_rows);
  float *pc = reinterpret_cast<float *>(jsm + lay.off_pc);
  float *ps = reinterpret_cast<float *>(jsm + lay.off_ps);
  float *pt = reinterpret_cast<float *>(jsm + lay.off_pt);
  float *diag = reinterpret_cast<float *>(jsm + lay.off_diag);  // [2][np]
  float *coup = reinterpret_cast<float *>(jsm + lay.off_coup);  // [2][P]
  int *const top_m = reinterpret_cast<int *>(jsm + lay.off_top);  // [2][L]
  int *const bot_m = reinterpret_cast<int *>(jsm + lay.off_bot);
  int *flag = reinterpret_cast<int *>(jsm + lay.off_flag);  // [sweep]: some pair rotated
  int *top = top_m, *bot = bot_m;  // the current maps: slot s0+i -> row buffers
  const bool refine = a.refine != 0;
  const int prob = blockIdx.x / C;
  const int s0 = crank * L, nloc = min(P, s0 + L) - s0;  // >= 1 (host)
  const int cgroups = (int)blockDim.x / P;  // >= 8 (P <= 128)
  const double *Gin = a.g[prob];
  float2 *log = a.log + (int64_t)prob * JAC_MAX_SWEEPS * (np - 1) * P;
  // at every sweep start slot k holds players k (top) and np-1-k (bottom)
  auto player_of = [&](int i) { return (i & 1) ? np - 1 - (s0 + i / 2) : s0 + i / 2; };
  auto row_of = [&](int i) { return rows + (size_t)((i & 1) ? bot[i / 2] : top[i / 2]) * np; };
  for (int i = threadIdx.x; i < nloc; i += blockDim.x) {
    top[i] = 2 * i;
    bot[i] = 2 * i + 1;
  }
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    dbase[i] = (refine && i < n) ? Gin[(int64_t)i * n + i] : 0.0;
    diag[i] = (!refine && i < n) ? (float)Gin[(int64_t)i * n + i] : 0.f;
  }
  for (int k = threadIdx.x; k < P; k += blockDim.x) {  // round 0 pairs (k, np-1-k)
    const int q = np - 1 - k;
    coup[k] = q < n ? (float)Gin[(int64_t)k * n + q] : 0.f;
  }
  for (int i = threadIdx.x; i <= JAC_MAX_SWEEPS; i += blockDim.x) flag[i] = 0;
  for (int idx = threadIdx.x; idx < 2 * nloc * np; idx += blockDim.x) {
    const int b = idx / np, col = idx % np, x = player_of(b);
    float v = 0.f;
    if (x < n && col < n && !(refine && x == col)) v = (float)Gin[(int64_t)x * n + col];
    rows[(size_t)b * np + col] = v;
  }
  __syncthreads();
  // Rotations of round t (of sweep `sw`, global round g) for every slot, from
  // the broadcast values of parity `par`; threads < P.
  float dmax = 0.f;  // max|a_ii| at the start of the sweep (rotation warps)
  auto sweep_dmax = [&](int par) {
    float m = 0.f;
    for (int x = threadIdx.x & 31; x < n; x += 32)
      m = fmaxf(m, fabsf((float)(dbase[x] + (double)diag[par * np + x])));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
  };
  auto rotations = [&](int k, int t, int sw, int g, int par) {
    const int x = circle_player(k, t, np), y = circle_player(np - 1 - k, t, np);
    const int p = min(x, y), q = max(x, y);
    float c = 1.f, s = 0.f, tt = 0.f;
    if (q < n) {
      const float cp = diag[par * np + p], cq = diag[par * np + q], apq = coup[par * P + k];
      const float app = (float)(dbase[p] + (double)cp), aqq = (float)(dbase[q] + (double)cq);
      const float floor_abs = (refine ? 1e-11f : 1e-5f) * dmax;
      const float rel_tol = refine ? 1e-7f : 1e-6f;
      if (fabsf(apq) > floor_abs && fabsf(apq) > rel_tol * sqrtf(fabsf(app) * fabsf(aqq))) {
        const float diff = refine ? (float)(dbase[q] - dbase[p]) + (cq - cp) : aqq - app;
        float tau = diff / (2.f * apq);
        float sg = tau >= 0.f ? 1.f : -1.f;
        tt = sg / (fabsf(tau) + sqrtf(1.f + tau * tau));
        c = rsqrtf(1.f + tt * tt);
        s = tt * c;
        flag[sw] = 1;
      }
    }
    pc[k] = c;
    ps[k] = s;
    pt[k] = tt;
    if (k >= s0 && k < s0 + nloc) log[(int64_t)g * P + k] = make_float2(c, s);
  };
  // the rotations are computed by warps 16-19 and the broadcast sent by warps
  // 24-31, while warps 0-7 move rows, so the phases of a round overlap
  const int rt = (int)threadIdx.x - kJacRotBase, bt = (int)threadIdx.x - kJacSendBase;
  if (rt >= 0 && rt < ((P + 31) & ~31)) dmax = sweep_dmax(0);
  if (rt >= 0 && rt < P) rotations(rt, 0, 0, 0, 0);
  __syncthreads();
  int sweeps_done = JAC_MAX_SWEEPS;
  for (int g = 0;; ++g) {
    const int t = g % (np - 1);
    // every rotation applied to the owned rows, 2 x 2 block (owned slot k1,
    // slot k2) by block: a thread keeps one column slot k2 for the round and
    // walks the owned slots (groups of P threads; the column pair's players
    // and rotation are loaded once)
    if ((int)threadIdx.x < cgroups * P) {
      const int k2 = (int)threadIdx.x % P;
      const int x2 = circle_player(k2, t, np), y2 = circle_player(np - 1 - k2, t, np);
      const int p2 = min(x2, y2), q2 = max(x2, y2);
      const float c2 = pc[k2], s2v = ps[k2];
      for (int kl = (int)threadIdx.x / P; kl < nloc; kl += cgroups) {
        const int k1 = s0 + kl;
        const float s1v = ps[k1];
        if (s1v == 0.f && s2v == 0.f) continue;
        const int x1 = circle_player(k1, t, np), y1 = circle_player(np - 1 - k1, t, np);
        const int p1 = min(x1, y1), q1 = max(x1, y1);
        float *rp = rows + (x1 < y1 ? top[kl] : bot[kl]) * np;
        float *rq = rows + (x1 < y1 ? bot[kl] : top[kl]) * np;
        if (k2 == k1) {  // the rotation's own 2 x 2 block
          const float t1 = pt[k1];
          if (q1 < n && t1 != 0.f) {
            const float apq = rp[q1];
            rp[p1] -= t1 * apq;
            rq[q1] += t1 * apq;
            rp[q1] = 0.f;
            rq[p1] = 0.f;
          }
          continue;
        }
        const float c1 = pc[k1];
        const float cc = __fmul_rn(c1, c2), cs = __fmul_rn(c1, s2v), sc = __fmul_rn(s1v, c2),
                    ss = __fmul_rn(s1v, s2v);
        const float b00 = rp[p2], b01 = rp[q2], b10 = rq[p2], b11 = rq[q2];
        // J1^T B J2 with J = [[c, s], [-s, c]]; the twin block (k2, k1) sums
        // the same four products in the same pairs
        rp[p2] = __fsub_rn(__fadd_rn(__fmul_rn(cc, b00), __fmul_rn(ss, b11)),
                           __fadd_rn(__fmul_rn(cs, b01), __fmul_rn(sc, b10)));
        rp[q2] = __fsub_rn(__fadd_rn(__fmul_rn(cs, b00), __fmul_rn(cc, b01)),
                           __fadd_rn(__fmul_rn(ss, b10), __fmul_rn(sc, b11)));
        rq[p2] = __fsub_rn(__fadd_rn(__fmul_rn(sc, b00), __fmul_rn(cc, b10)),
                           __fadd_rn(__fmul_rn(ss, b01), __fmul_rn(cs, b11)));
        rq[q2] = __fadd_rn(__fadd_rn(__fmul_rn(ss, b00), __fmul_rn(cc, b11)),
                           __fadd_rn(__fmul_rn(sc, b01), __fmul_rn(cs, b10)));
      }
    }
    __syncthreads();
    // the next round: position j -> j - 1 (j >= 2), 1 -> np - 1, 0 stays
    const int g1 = g + 1, t1 = g1 % (np - 1), sw1 = g1 / (np - 1), par = g1 & 1;
    float *mbox = rows + (size_t)(2 * L + 2 * par) * np;  // [from left, from right]
    if (P >= 2) {  // hand-over: first owned top row left, last owned bottom row right
      if (crank > 0) {
        const float *src = rows + (size_t)top[0] * np;
        float *dst = cluster.map_shared_rank(mbox, crank - 1) + np;
        for (int i = threadIdx.x; i < np; i += blockDim.x) dst[i] = src[i];
      }
      if (crank < C - 1) {
        const float *src = rows + (size_t)bot[nloc - 1] * np;
        float *dst = cluster.map_shared_rank(mbox, crank + 1);
        for (int i = threadIdx.x; i < np; i += blockDim.x) dst[i] = src[i];
      }
    }
    // each held row's diagonal, and its coupling to its next partner (sent by
    // the lower-numbered of the two), to every CTA
    for (int i = bt; i >= 0 && i < 2 * nloc; i += JAC_THREADS - kJacSendBase) {
      const int k = s0 + i / 2, pos = (i & 1) ? np - 1 - k : k;
      const int x = circle_player(pos, t, np);
      const float *row = rows + (size_t)((i & 1) ? bot[i / 2] : top[i / 2]) * np;
      const int pos1 = pos == 0 ? 0 : (pos == 1 ? np - 1 : pos - 1);
      const int k1 = min(pos1, np - 1 - pos1), y = circle_player(np - 1 - pos1, t1, np);
      const float dv = row[x];
      const bool send_c = x < y;
      const float cv = (send_c && y < n) ? row[y] : 0.f;
      for (int r = 0; r < C; ++r) {
        cluster.map_shared_rank(diag, r)[par * np + x] = dv;
        if (send_c) cluster.map_shared_rank(coup, r)[par * P + k1] = cv;
      }
    }
    if (C > 1) cluster.sync(); else __syncthreads();  // a one-CTA barrier is 8x cheaper
    if (P >= 2) {  // rename into the other map pair; arrived rows take the freed buffers
      int dl, dr;
      circle_arrivals(top, bot, s0, nloc, P, &dl, &dr);
      int *ntop = top == top_m ? top_m + L : top_m, *nbot = bot == bot_m ? bot_m + L : bot_m;
      for (int i = threadIdx.x; i < nloc; i += blockDim.x)
        circle_next(top, bot, s0, nloc, P, i, dl, dr, &ntop[i], &nbot[i]);
      for (int i = threadIdx.x; i < np; i += blockDim.x) {
        if (dl >= 0) rows[(size_t)dl * np + i] = mbox[i];
        if (dr >= 0) rows[(size_t)dr * np + i] = mbox[np + i];
      }
      top = ntop;
      bot = nbot;
    }
    if (t1 == 0) {  // sweep boundary: stop after a sweep without rotations
      __syncthreads();
      if (!flag[sw1 - 1] || sw1 == JAC_MAX_SWEEPS) {  // the same in every CTA
        sweeps_done = sw1;
        break;
      }
      if (rt >= 0 && rt < ((P + 31) & ~31)) dmax = sweep_dmax(par);
    }
    if (rt >= 0 && rt < P) rotations(rt, t1, sw1, g1, par);
    __syncthreads();
  }
  if (crank == 0 && threadIdx.x == 0) a.sweeps[prob] = sweeps_done;
  // eigenvalues to every CTA of the cluster, then each ranks its own players
  for (int i = threadIdx.x; i < 2 * nloc; i += blockDim.x) {
    const int x = player_of(i);
    const double lx = dbase[x] + (double)row_of(i)[x];
    for (int r = 0; r < C; ++r) cluster.map_shared_rank(lam_all, r)[x] = lx;
  }
  if (C > 1) cluster.sync(); else __syncthreads();  // the last remote access is above
  float *lam = a.lambda[prob];
  for (int i = threadIdx.x; i < 2 * nloc; i += blockDim.x) {
    const int x = player_of(i);
    if (x >= n) continue;
    const double li = lam_all[x];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = lam_all[j];
      r += (lj > li) || (lj == li && j < x);
    }
    a.rank[prob * n + x] = r;
    lam[r] = (float)li;
  }
}

// V = product of the logged rotations, rows processed independently;
// column c of the product lands in column rank[c] of the output. The log is
// streamed into shared memory REPLAY_CHUNK rounds at a time with cp.async,
// double buffered, so a round waits on its barrier only, not on L2.
constexpr int REPLAY_ROWS = 16;
constexpr int REPLAY_CHUNK = 16;

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}

__global__ void __launch_bounds__(256) jacobi_replay_kernel(JacobiArgs a, float *const *vout) {
  extern __shared__ __align__(16) float sv[];  // [REPLAY_ROWS][n], then [2][REPLAY_CHUNK][P] float2
  const int n = a.n, np = n + (n & 1), P = np / 2;
  const int prob = blockIdx.y;
  const int r0 = blockIdx.x * REPLAY_ROWS;
  const int nr = min(REPLAY_ROWS, n - r0);
  if (nr <= 0) return;
  float2 *lb = reinterpret_cast<float2 *>(sv + ((REPLAY_ROWS * n + 1) & ~1));
  const float *vin = a.vinit ? a.vinit[prob] : nullptr;
  for (int i = threadIdx.x; i < REPLAY_ROWS * n; i += blockDim.x) {
    int rr = i / n, cc = i % n;
    sv[i] = rr >= nr ? 0.f : vin ? vin[(int64_t)(r0 + rr) * n + cc] : (r0 + rr == cc ? 1.f : 0.f);
  }
  const float2 *log = a.log + (int64_t)prob * JAC_MAX_SWEEPS * (np - 1) * P;
  const int rounds = a.sweeps[prob] * (np - 1);
  const int nchunks = (rounds + REPLAY_CHUNK - 1) / REPLAY_CHUNK;
  const int G = max(1, (int)blockDim.x / P);                // row groups (P <= 128)
  const int g = (int)threadIdx.x / P, k = (int)threadIdx.x % P;
  auto issue = [&](int c) {
    const int first = c * REPLAY_CHUNK, cnt = min(REPLAY_CHUNK, rounds - first);
    const float2 *src = log + (int64_t)first * P;
    float2 *dst = lb + (c & 1) * REPLAY_CHUNK * P;
    for (int i = threadIdx.x; i < cnt * P; i += blockDim.x) cp_async8(dst + i, src + i);
    cp_async_commit();
  };
  if (nchunks > 0) issue(0);
  for (int c = 0; c < nchunks; ++c) {
    if (c + 1 < nchunks) {
      issue(c + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // chunk c visible to every thread; sv initialized
    const float2 *buf = lb + (c & 1) * REPLAY_CHUNK * P;
    const int first = c * REPLAY_CHUNK, cnt = min(REPLAY_CHUNK, rounds - first);
    for (int q = 0; q < cnt; ++q) {
      const int t = (first + q) % (np - 1);
      // thread (group g, pair k): one rotation, applied to rows g, g+G, ...
      if (g < G) {
        const float2 cs = buf[q * P + k];
        const int x = circle_player(k, t, np), y = circle_player(np - 1 - k, t, np);
        const int p = min(x, y), qq = max(x, y);
        if (cs.y != 0.f && qq < n)
          for (int rr = g; rr < nr; rr += G) {
            const float vp = sv[rr * n + p], vq = sv[rr * n + qq];
            sv[rr * n + p] = cs.x * vp - cs.y * vq;
            sv[rr * n + qq] = cs.y * vp + cs.x * vq;
          }
      }
      __syncthreads();
    }
  }
  float *V = vout[prob];
  const int32_t *rank = a.rank + prob * n;
  for (int i = threadIdx.x; i < nr * n; i += blockDim.x) {
    int rr = i / n, cc = i % n;
    V[(int64_t)(r0 + rr) * n + rank[cc]] = sv[rr * n + cc];
  }
}

}  // namespace

// ------------------------------------------------------------------ host side
int sm_count() {
  // initialized once, thread-safely (a pipelined run calls this from two threads)
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

int grid_for(int64_t work_items, int threads_per_block, int blocks_per_sm) {
  int64_t need = ceil_div(std::max<int64_t>(work_items, 1), threads_per_block);
  int64_t cap = (int64_t)sm_count() * blocks_per_sm;
  return (int)std::max<int64_t>(1, std::min(need, cap));
}

// A kernel's dynamic shared-memory ceiling is a process-wide attribute, and
// sessions on other threads launch the same kernels with other sizes: it is
// only ever raised (under a lock), so no thread's launch can find it lowered
// below what that launch asks for.
static tsvd_status set_smem(const void *fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, size_t> ceiling;
  int dev = 0;
  TSVD_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(mu);
  size_t &cur = ceiling[std::make_pair(fn, dev)];
  if (bytes <= cur) return TSVD_OK;
  TSVD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return TSVD_OK;
}

// cuTensorMapEncodeTiled, resolved from the driver at run time (the library
// links only the runtime).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tensor_map_encoder() {
  static const EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e =
        cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// A row-major fp16 matrix [rows][pitch] (the first `cols` values of each row
// in use) as a 2-D tensor for the TMA: {cols, rows}, a {box_cols, box_rows}
// box, the given shared-memory swizzle.
static tsvd_status encode_2d(CUtensorMap *m, const __half *base, int64_t cols, int64_t rows,
                             int pitch, int box_cols, int box_rows, CUtensorMapSwizzle swz) {
  const EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return fail(TSVD_ERR_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  if (!base || (reinterpret_cast<uintptr_t>(base) & 15) != 0 || pitch % 8 != 0)
    return fail(TSVD_ERR_INVALID, "tensor map: operand %p / pitch %d not 16-byte aligned",
                (const void *)base, pitch);
  const cuuint64_t dims[2] = {(cuuint64_t)std::max<int64_t>(cols, 1),
                              (cuuint64_t)std::max<int64_t>(rows, 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * 2};
  const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  const cuuint32_t estride[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, (void *)base, dims, strides, box,
                        estride, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(TSVD_ERR_DEVICE,
                "cuTensorMapEncodeTiled: error %d (%lld x %lld, pitch %d, box %d x %d)", (int)r,
                (long long)rows, (long long)cols, pitch, box_rows, box_cols);
  return TSVD_OK;
}

tsvd_status gemm_encode_maps(int fwd, int nprob, const __half *const *at, const int32_t *nc,
                             int lda, const __half *const *hi, const __half *const *lo,
                             CUtensorMap *out) {
  for (int i = 0; i < nprob; ++i) {
    CUtensorMap *m = out + 3 * (int64_t)i;
    if (fwd)  // M = Sp along the rows of A^T, K = its n_c rows: 64 x 32 boxes
      TSVD_TRY(encode_2d(m, at[i], lda, nc[i], lda, kAtom, BK, CU_TENSOR_MAP_SWIZZLE_128B));
    else      // K = Sp along the rows, M = the n_c rows: 32 x 128 boxes
      TSVD_TRY(encode_2d(m, at[i], lda, nc[i], lda, BK, BM, CU_TENSOR_MAP_SWIZZLE_64B));
    const int64_t brows = fwd ? nc[i] : lda;
    TSVD_TRY(encode_2d(m + 1, hi[i], BN, brows, BN, kAtom, BK, CU_TENSOR_MAP_SWIZZLE_128B));
    if (lo && lo[i])
      TSVD_TRY(encode_2d(m + 2, lo[i], BN, brows, BN, kAtom, BK, CU_TENSOR_MAP_SWIZZLE_128B));
    else
      memset(m + 2, 0, sizeof(CUtensorMap));
  }
  return TSVD_OK;
}

tsvd_status gemm_fwd(const GemmBatch &gb, bool has_lo, float *const *y, float *y_base,
                     size_t y_bytes, int sp, int max_nc, float inv_xscale, cudaStream_t st) {
  if (gb.nprob == 0) return TSVD_OK;
  if (sp % BM != 0) return fail(TSVD_ERR_INVALID, "gemm_fwd: Sp = %d not a multiple of %d", sp, BM);
  if (!gb.maps) return fail(TSVD_ERR_INVALID, "gemm_fwd: no tensor maps");
  TSVD_TRY(set_smem((const void *)umma_gemm_kernel<true>, kGemmSmem));
  const int mtiles = (int)ceil_div(sp, BM * MH);
  int splits = 1;
  int64_t base_ctas = (int64_t)mtiles * gb.nprob;
  int64_t target = sm_count();  // one CTA per SM (shared memory)
  if (base_ctas < target)
    splits = (int)std::min<int64_t>(ceil_div(target, base_ctas),
                                    std::max<int64_t>(1, ceil_div(max_nc, 1024)));
  // split-K partial tiles are accumulated with atomics into zeroed outputs
  if (splits > 1) TSVD_CUDA(cudaMemsetAsync(y_base, 0, y_bytes, st));
  GemmArgs a{gb.maps, gb.ncols, gb.lda, has_lo ? 1 : 0, y, inv_xscale, splits};
  dim3 grid(mtiles, splits, gb.nprob);
  umma_gemm_kernel<true><<<grid, GEMM_THREADS, kGemmSmem, st>>>(a);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status gemm_bwd(const GemmBatch &gb, bool has_lo, float *const *z, int sp, int max_nc,
                     float inv_yscale, cudaStream_t st) {
  if (gb.nprob == 0 || max_nc == 0) return TSVD_OK;
  if (sp % BK != 0) return fail(TSVD_ERR_INVALID, "gemm_bwd: Sp = %d not a multiple of %d", sp, BK);
  if (!gb.maps) return fail(TSVD_ERR_INVALID, "gemm_bwd: no tensor maps");
  TSVD_TRY(set_smem((const void *)umma_gemm_kernel<false>, kGemmSmem));
  GemmArgs a{gb.maps, gb.ncols, sp, has_lo ? 1 : 0, z, inv_yscale, 1};
  dim3 grid((unsigned)ceil_div(max_nc, BM * MH), 1, gb.nprob);
  umma_gemm_kernel<false><<<grid, GEMM_THREADS, kGemmSmem, st>>>(a);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status gemm_check(cudaStream_t st) {
  int h = 0;
  TSVD_CUDA(cudaMemcpyFromSymbolAsync(&h, g_umma_timeouts, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  if (h != 0) {
    const int zero = 0;
    TSVD_CUDA(cudaMemcpyToSymbolAsync(g_umma_timeouts, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
    return fail(TSVD_ERR_TIMEOUT, "tensor-core GEMM: %d warps gave up waiting for their MMAs", h);
  }
  return TSVD_OK;
}

static void gram_chunks(int max_rows, int nprob, int *nchunks, int *chunk_rows) {
  int64_t want = ceil_div(std::max(max_rows, 1), GRAM_MIN_ROWS);
  int64_t cap = std::max<int64_t>(1, GRAM_MAX_CHUNKS / std::max(nprob, 1));
  int64_t nc = std::max<int64_t>(1, std::min(want, cap));
  int64_t cr = round_up(ceil_div(std::max(max_rows, 1), nc), 32);
  *chunk_rows = (int)cr;
  *nchunks = (int)ceil_div(std::max(max_rows, 1), cr);
}

size_t gram_work_bytes(int max_rows, int l, int nprob) {
  int nchunks, cr;
  gram_chunks(max_rows, nprob, &nchunks, &cr);
  return (size_t)nprob * nchunks * l * l * sizeof(double);
}

tsvd_status gram_batched(const float *const *x, const int32_t *rows, int max_rows, int l, int ld,
                         double *const *g, double *work, size_t work_bytes, int nprob,
                         cudaStream_t st) {
  if (nprob == 0) return TSVD_OK;
  if (l > GRAM_LMAX) return fail(TSVD_ERR_INVALID, "gram: l=%d > %d", l, GRAM_LMAX);
  int nchunks, chunk_rows;
  gram_chunks(max_rows, nprob, &nchunks, &chunk_rows);
  if (gram_work_bytes(max_rows, l, nprob) > work_bytes)
    return fail(TSVD_ERR_INVALID, "gram: work buffer too small");
  int tiles = (l + 3) / 4;
  int groups = (int)ceil_div(tiles * (tiles + 1) / 2, GRAM_TILES_PER_CTA);
  size_t smem = (size_t)GRAM_SUB * (4 * tiles) * sizeof(float);
  TSVD_TRY(set_smem((const void *)gram_partial_kernel, smem));
  // chunks past a problem's row count must contribute zeros
  TSVD_CUDA(cudaMemsetAsync(work, 0, gram_work_bytes(max_rows, l, nprob), st));
  GramArgs a{x, rows, ld, l, tiles, nchunks, chunk_rows, work};
  gram_partial_kernel<<<dim3(nchunks, groups, nprob), GRAM_THREADS, smem, st>>>(a);
  TSVD_LAUNCH_CHECK();
  gram_reduce_kernel<<<dim3((unsigned)ceil_div((int64_t)l * l, 256), nprob), 256, 0, st>>>(
      work, nchunks, l, g, nprob);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status chol_inverse_batched(double *const *g, float *const *t, int l, int nprob,
                                 cudaStream_t st) {
  if (nprob == 0) return TSVD_OK;
  if (l > kLp) return fail(TSVD_ERR_INVALID, "chol: l=%d > %d", l, kLp);
  size_t smem = (size_t)2 * l * (l + 1) * sizeof(float);
  TSVD_TRY(set_smem((const void *)chol_inverse_kernel, smem));
  chol_inverse_kernel<<<nprob, CHOL_THREADS, smem, st>>>(g, t, l);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

// One block per problem: the lower Cholesky factor of G in fp64 in global
// memory (it stays in L2), right-looking, a column per step. Directions whose
// pivot falls below 1e-13 of the largest diagonal entry are dropped: unit
// pivot, zero column, flag 1.0 after the factor (work: l*l + l doubles).
__global__ void __launch_bounds__(1024) chol_wide_kernel(double *const *gs, double *work, int l) {
  __shared__ double tol;
  const double *G = gs[blockIdx.x];
  double *A = work + (int64_t)blockIdx.x * (l * l + l);
  double *drop = A + (int64_t)l * l;
  for (int i = threadIdx.x; i < l * l; i += blockDim.x) A[i] = G[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int i = 0; i < l; ++i) mx = fmax(mx, A[(int64_t)i * l + i]);
    tol = mx * 1e-13;
  }
  __syncthreads();
  for (int k = 0; k < l; ++k) {
    if (threadIdx.x == 0) {
      const double d = A[(int64_t)k * l + k];
      const bool dk = !(d > tol) || !(d > 0.0);
      drop[k] = dk ? 1.0 : 0.0;
      A[(int64_t)k * l + k] = dk ? 1.0 : sqrt(d);
    }
    __syncthreads();
    const double piv = A[(int64_t)k * l + k];
    const bool dk = drop[k] != 0.0;
    for (int i = k + 1 + threadIdx.x; i < l; i += blockDim.x)
      A[(int64_t)i * l + k] = dk ? 0.0 : A[(int64_t)i * l + k] / piv;
    __syncthreads();
    const int n = l - k - 1;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int i = k + 1 + t / n, j = k + 1 + t % n;
      if (j <= i) A[(int64_t)i * l + j] -= A[(int64_t)i * l + k] * A[(int64_t)j * l + k];
    }
    __syncthreads();
  }
}

// y = x R^-1 with R = L^T, one thread per row: y_j = (x_j - sum_{k<j} y_k
// L[j][k]) / L[j][j] in fp64, dropped directions 0. x, y: rows x l (ld l) per
// problem at stride `stride`.
__global__ void trsm_rows_kernel(const float *__restrict__ x, float *__restrict__ y,
                                 const double *__restrict__ work, int rows, int l,
                                 int64_t stride) {
  const int prob = blockIdx.y;
  const double *L = work + (int64_t)prob * (l * l + l);
  const double *drop = L + (int64_t)l * l;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    const float *xr = x + prob * stride + (int64_t)r * l;
    float *yr = y + prob * stride + (int64_t)r * l;
    for (int j = 0; j < l; ++j) {
      double s = xr[j];
      const double *Lj = L + (int64_t)j * l;
      for (int k = 0; k < j; ++k) s -= (double)yr[k] * Lj[k];
      yr[j] = drop[j] != 0.0 ? 0.f : (float)(s / Lj[j]);
    }
  }
}

// Shifted Cholesky in fp32 for the basis of a subspace iteration: K + s I =
// L L^T with s = shift * trace(K) / l, so no direction is dropped and the
// result R^{-1} = L^{-T} makes a well-conditioned (not exactly orthonormal)
// basis. One block per problem, packed lower triangle in shared memory; L
// goes out packed (row i at i(i+1)/2). K: l x l fp32, problem b at b * l * l.
__global__ void __launch_bounds__(1024) chol_shift_kernel(const float *__restrict__ K,
                                                          float *__restrict__ Lout, int l,
                                                          float shift) {
  extern __shared__ float Lp[];  // l (l + 1) / 2
  __shared__ float tr;
  const float *Kb = K + (int64_t)blockIdx.x * l * l;
  float *Lb = Lout + (int64_t)blockIdx.x * l * (l + 1) / 2;
  for (int t = threadIdx.x; t < l * (l + 1) / 2; t += blockDim.x) {
    int i = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    const int j = t - i * (i + 1) / 2;
    Lp[t] = Kb[(int64_t)i * l + j];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float acc = 0.f;
    for (int i = 0; i < l; ++i) acc += Lp[i * (i + 1) / 2 + i];
    tr = fmaxf(acc, FLT_MIN) * shift / (float)l;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < l; i += blockDim.x) Lp[i * (i + 1) / 2 + i] += tr;
  __syncthreads();
  for (int k = 0; k < l; ++k) {
    const int kk = k * (k + 1) / 2 + k;
    if (threadIdx.x == 0) Lp[kk] = sqrtf(fmaxf(Lp[kk], tr));
    __syncthreads();
    const float piv = Lp[kk];
    for (int i = k + 1 + threadIdx.x; i < l; i += blockDim.x) Lp[i * (i + 1) / 2 + k] /= piv;
    __syncthreads();
    const int n = l - k - 1;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int i = k + 1 + t / n, j = k + 1 + t % n;
      if (j <= i) Lp[i * (i + 1) / 2 + j] -= Lp[i * (i + 1) / 2 + k] * Lp[j * (j + 1) / 2 + k];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < l * (l + 1) / 2; t += blockDim.x) Lb[t] = Lp[t];
}

// y = x L^{-T}, one warp per row: y_j = (x_j - sum_{k<j} y_k L[j][k]) / L[j][j]
// with the dot product split over the lanes; L packed in shared memory, the
// row's y in the warp's shared slice. x, y: rows x l, problem b at b * stride.
__global__ void __launch_bounds__(1024) trsm_warp_kernel(const float *__restrict__ x,
                                                         float *__restrict__ y,
                                                         const float *__restrict__ Lpk, int rows,
                                                         int l, int64_t stride) {
  extern __shared__ float sm[];
  float *Lp = sm;                                   // l (l + 1) / 2
  float *ys = sm + ((l * (l + 1) / 2 + 3) & ~3);    // [warps][l]
  const int prob = blockIdx.y;
  const float *Lb = Lpk + (int64_t)prob * l * (l + 1) / 2;
  for (int t = threadIdx.x; t < l * (l + 1) / 2; t += blockDim.x) Lp[t] = Lb[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  float *yw = ys + warp * l;
  for (int r = blockIdx.x * nwarps + warp; r < rows; r += gridDim.x * nwarps) {
    const float *xr = x + prob * stride + (int64_t)r * l;
    float *yr = y + prob * stride + (int64_t)r * l;
    for (int j = 0; j < l; ++j) {
      const float *Lj = Lp + j * (j + 1) / 2;
      float part = 0.f;
      for (int k = lane; k < j; k += 32) part = fmaf(yw[k], Lj[k], part);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(kFull, part, o);
      const float v = (xr[j] - part) / Lj[j];
      if (lane == 0) yw[j] = v;
      __syncwarp();
    }
    for (int j = lane; j < l; j += 32) yr[j] = yw[j];
    __syncwarp();
  }
}

tsvd_status chol_shift_solve_batched(const float *K, float *Lpk, const float *x, float *y,
                                     int rows, int l, int64_t stride, float shift, int nprob,
                                     cudaStream_t st) {
  if (nprob == 0) return TSVD_OK;
  if (l > 256 || l < 1) return fail(TSVD_ERR_INVALID, "chol shift: l=%d", l);
  const size_t csm = (size_t)l * (l + 1) / 2 * sizeof(float);
  const size_t tsm = (((size_t)l * (l + 1) / 2 + 3) & ~(size_t)3) * sizeof(float) +
                     (size_t)32 * l * sizeof(float);
  if (csm > 48 * 1024) TSVD_TRY(set_smem((const void *)chol_shift_kernel, csm));
  if (tsm > 48 * 1024) TSVD_TRY(set_smem((const void *)trsm_warp_kernel, tsm));
  chol_shift_kernel<<<nprob, 1024, csm, st>>>(K, Lpk, l, shift);
  TSVD_LAUNCH_CHECK();
  const int blocks = (int)std::min<int64_t>(ceil_div(rows, 32), 2 * sm_count() / std::max(nprob, 1) + 1);
  trsm_warp_kernel<<<dim3(blocks, nprob), 1024, tsm, st>>>(x, y, Lpk, rows, l, stride);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status chol_solve_wide_batched(double *const *g, double *work, const float *x, float *y,
                                    int rows, int l, int64_t stride, int nprob, cudaStream_t st) {
  if (nprob == 0) return TSVD_OK;
  if (l > 256 || l < 1) return fail(TSVD_ERR_INVALID, "chol wide: l=%d", l);
  chol_wide_kernel<<<nprob, 1024, 0, st>>>(g, work, l);
  TSVD_LAUNCH_CHECK();
  trsm_rows_kernel<<<dim3(ceil_div(rows, 128), nprob), 128, 0, st>>>(x, y, work, rows, l, stride);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status apply_right_batched(const float *const *x, const int32_t *rows, int max_rows, int ldx,
                                const float *const *w, int ldw, int n_in, int n_out,
                                const float *const *colscale, float *const *y, int ldy,
                                __half *const *yhi, __half *const *ylo, float split_scale,
                                int nprob, cudaStream_t st) {
  if (nprob == 0 || max_rows == 0) return TSVD_OK;
  if (n_out > APPLY_WLD || ldy > APPLY_WLD || n_in > 256 || n_in < 1)
    return fail(TSVD_ERR_INVALID, "apply_right: sizes %d %d %d", n_in, n_out, ldy);
  const size_t smem = (size_t)n_in * (APPLY_WLD + APPLY_XLD) * sizeof(float);
  TSVD_TRY(set_smem((const void *)apply_right_kernel, smem));
  const int tiles = (int)ceil_div(max_rows, APPLY_RT);
  const int per_sm = std::max(1, (int)((227 * 1024) / (smem + 1024)));
  const int64_t items = (int64_t)tiles * nprob;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(items, (int64_t)sm_count() * per_sm));
  ApplyArgs a{x, rows, ldx, w, ldw, n_in, n_out, colscale, y, ldy, yhi, ylo, split_scale, tiles,
              nprob};
  apply_right_kernel<<<grid, APPLY_THREADS, smem, st>>>(a);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

size_t jacobi_work_bytes(int n, int nprob) {
  int np = n + (n & 1);
  size_t logb = (size_t)nprob * JAC_MAX_SWEEPS * (np - 1) * (np / 2) * sizeof(float2);
  return round_up(logb, 256) + round_up((size_t)nprob * sizeof(int32_t), 256) +
         round_up((size_t)nprob * n * sizeof(int32_t), 256);
}

tsvd_status jacobi_eig_batched(double *const *g, int n, float *const *lambda, float *const *v,
                               int nprob, void *work, size_t work_bytes, cudaStream_t st,
                               int *sweeps_out, int refine, const float *const *vinit) {
  if (nprob == 0) return TSVD_OK;
  if (n > 256 || n < 2) return fail(TSVD_ERR_INVALID, "jacobi: n=%d", n);
  if (jacobi_work_bytes(n, nprob) > work_bytes) return fail(TSVD_ERR_INVALID, "jacobi: work");
  int np = n + (n & 1);
  char *w = (char *)work;
  JacobiArgs a;
  a.g = g;
  a.n = n;
  a.lambda = lambda;
  a.log = (float2 *)w;
  w += round_up((size_t)nprob * JAC_MAX_SWEEPS * (np - 1) * (np / 2) * sizeof(float2), 256);
  a.sweeps = (int32_t *)w;
  w += round_up((size_t)nprob * sizeof(int32_t), 256);
  a.rank = (int32_t *)w;
  a.refine = refine;
  a.vinit = vinit;
  const int P = np / 2;
  // CTAs per problem: as many as keep the whole batch within one wave of
  // clusters (up to 8), at least as many as the rows need for shared memory,
  // and no CTA without a slot
  const size_t smem_cap = 200 * 1024;
  int C = 1;
  while (C < kJacMaxCluster && (int64_t)nprob * 2 * C <= sm_count()) C *= 2;
  while (C < kJacMaxCluster && JacobiSmem(n, C).bytes > smem_cap) C *= 2;
  while (C > 1 && (C - 1) * JacobiSmem(n, C).L >= P) C /= 2;
  int cmin = 1;
  while (cmin < kJacMaxCluster && JacobiSmem(n, cmin).bytes > smem_cap) cmin *= 2;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(JAC_THREADS);
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  auto configure = [&](int c) -> tsvd_status {
    cfg.gridDim = dim3((unsigned)(nprob * c));
    cfg.dynamicSmemBytes = JacobiSmem(n, c).bytes;
    attr[0].val.clusterDim.x = (unsigned)c;
    return set_smem((const void *)jacobi_kernel, cfg.dynamicSmemBytes);
  };
  // a cluster must fit in one GPC: fewer CTAs per problem when the batch's
  // clusters would not all be resident at once (a second wave doubles the
  // time, as 16 clusters of 8 did)
  while (C > cmin) {
    TSVD_TRY(configure(C));
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, (const void *)jacobi_kernel, &cfg) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    if (active >= nprob) break;
    C /= 2;
  }
  TSVD_TRY(configure(C));
  if (cfg.dynamicSmemBytes > smem_cap)
    return fail(TSVD_ERR_INVALID, "jacobi: n=%d needs %zu B per CTA", n, cfg.dynamicSmemBytes);
  TSVD_CUDA(cudaLaunchKernelEx(&cfg, jacobi_kernel, a));
  const size_t rsmem = (size_t)((REPLAY_ROWS * n + 1) & ~1) * sizeof(float) +
                       (size_t)2 * REPLAY_CHUNK * P * sizeof(float2);
  if (rsmem > 48 * 1024) TSVD_TRY(set_smem((const void *)jacobi_replay_kernel, rsmem));
  jacobi_replay_kernel<<<dim3((unsigned)ceil_div(n, REPLAY_ROWS), nprob), 256, rsmem, st>>>(a, v);
  TSVD_LAUNCH_CHECK();
  if (sweeps_out) {
    std::vector<int32_t> h(nprob);
    TSVD_CUDA(cudaMemcpyAsync(h.data(), a.sweeps, nprob * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
    int mx = 0;
    for (int x : h) mx = std::max(mx, x);
    *sweeps_out = mx;
  }
  return TSVD_OK;
}

}  // namespace tsvd
