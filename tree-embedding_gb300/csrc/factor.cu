// Batched frPCA over dirty column blocks and batched tree merges.
//
// frPCA follows Code/frpca.c:239-326 (k = d, s = l - d oversampling, q
// passes over A): a Gaussian start (frpca.c:257), products with A and A^T,
// a normalization after every product, and a final eigSVD of A^T Q
// (frpca.c:294-312). Normalizations use CholeskyQR (one pass between
// products, CholeskyQR2 for the final basis) where the reference uses LU
// (LUfraction) or eigSVD; all return a basis of the same column space, which
// is the only thing the next product consumes. Normalizing
// A^T Q as well keeps every basis within one condition number of A, so the
// half-precision split operands stay accurate.
//
// The merge follows Code/Tree_u_NC.cpp:723-850: M = [B_1 ... B_h], the
// truncated SVD of M (dgesvd, ..._mkl.c:1259-1300) keeps U_d S_d; here the
// Gram M^T M is diagonalized by Jacobi and B_parent = M V_d (= U_d S_d); the
// root keeps U sqrt(S) = M V_d S^-1/2 (NC) or U = M V_d S^-1 (LP).
#include <algorithm>
#include <cmath>

#include "factor.h"
#include "philox_gauss.h"
#include "plain.h"

namespace tsvd {

namespace {

constexpr float kSplitScale = 4096.f;  // orthonormal bases: |x| <= 1 -> fp16 hi/lo

// Pointer arrays for one batch, staged in pinned memory and uploaded at once.
struct PtrPack {
  FrpcaWork &W;
  size_t used = 0;
  size_t iused = 0;
  explicit PtrPack(FrpcaWork &w) : W(w) {}
  template <typename T>
  T *const *add(const std::vector<T *> &v) {
    size_t at = used;
    for (size_t i = 0; i < v.size(); ++i) W.hptr[used++] = (void *)v[i];
    return reinterpret_cast<T *const *>(W.dptr + at);
  }
  const int32_t *add_int(const std::vector<int32_t> &v) {
    size_t at = iused;
    for (size_t i = 0; i < v.size(); ++i) W.hint[iused++] = v[i];
    return W.dint + at;
  }
  tsvd_status upload(cudaStream_t st) {
    if (used > W.ptr_slots || iused > W.ptr_slots)
      return fail(TSVD_ERR_INVALID, "pointer pack overflow");
    TSVD_CUDA(cudaMemcpyAsync(W.dptr, W.hptr, used * sizeof(void *), cudaMemcpyHostToDevice, st));
    TSVD_CUDA(cudaMemcpyAsync(W.dint, W.hint, iused * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    return TSVD_OK;
  }
};

__global__ void omega_kernel(__half *const *xhi, const int32_t *ncols, const int32_t *const *colmap,
                             const int32_t *col_base, const int32_t *block, int64_t rows_max, int l,
                             uint64_t seed) {
  const int prob = blockIdx.y;
  const int32_t nc = ncols[prob];
  __half *X = xhi[prob];
  const int32_t *cm = colmap[prob];
  const int32_t base = col_base[prob];
  const uint32_t stream = (uint32_t)block[prob];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)nc * kLp;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = (int32_t)(i / kLp);
    int j = (int)(i % kLp);
    float val = 0.f;
    if (j < l) {
      int32_t col = cm ? cm[c] - base : c;
      val = tsvd_gauss_entry(seed, stream, (uint32_t)col, (uint32_t)j);
    }
    X[i] = __float2half_rn(val);
  }
}

__global__ void randq_kernel(float *const *y, __half *const *qhi, __half *const *qlo,
                             const int32_t *block, int sp, int nsrc, int l, uint64_t seed,
                             float split) {
  const int prob = blockIdx.y;
  const uint32_t stream = 0x80000000u | (uint32_t)block[prob];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)sp * kLp;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t s = (int32_t)(i / kLp);
    int j = (int)(i % kLp);
    float val = (s < nsrc && j < l) ? tsvd_gauss_entry(seed, stream, (uint32_t)s, (uint32_t)j) : 0.f;
    y[prob][i] = val;
    float sv = val * split;
    __half h = __float2half_rn(sv);
    qhi[prob][i] = h;
    qlo[prob][i] = __float2half_rn(sv - __half2float(h));
  }
}

// sigma_j = sqrt(max(lambda_j, 0)), zeroed at or below 1e-4 (frpca.c:106-122).
__global__ void sigma_kernel(const float *const *lambda, int d, float *const *colscale,
                             float *const *colscale_inv, float *const *sigma_out,
                             double *sum_sigma2) {
  const int prob = blockIdx.x;
  __shared__ double red[32];
  double acc = 0.0;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    float lam = lambda[prob][j];
    float s = sqrtf(fmaxf(lam, 0.f));
    if (s <= 1e-4f) s = 0.f;
    colscale[prob][j] = s;
    if (colscale_inv) colscale_inv[prob][j] = s > 0.f ? 1.f / s : 0.f;
    if (sigma_out && sigma_out[prob]) sigma_out[prob][j] = s;
    acc += (double)s * (double)s;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    sum_sigma2[prob] = t;
  }
}

// Root/inner scaling of the merged factor: 1, s^-1/2 or s^-1.
__global__ void merge_scale_kernel(const float *const *lambda, int d, int mode,
                                   float *const *colscale, float *const *sigma_out) {
  const int prob = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    float s = sqrtf(fmaxf(lambda[prob][j], 0.f));
    float f = 1.f;
    if (mode == 1) f = s > 0.f ? rsqrtf(s) : 0.f;
    if (mode == 2) f = s > 0.f ? 1.f / s : 0.f;
    colscale[prob][j] = f;
    if (sigma_out[prob]) sigma_out[prob][j] = s;
  }
}

__global__ void concat_kernel(const float *const *children, int h, int d, int nsrc,
                              float *const *m) {
  const int prob = blockIdx.y;
  const int n = h * d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)nsrc * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = i / n;
    int c = (int)(i % n);
    m[prob][i] = children[prob * h + c / d][s * d + c % d];
  }
}

// CholeskyQR with `passes` passes (2 = CholeskyQR2); the last pass also writes
// the fp16 hi/lo split of the basis.
tsvd_status cholqr(FrpcaWork &W, float *const *x, const int32_t *rows, int max_rows,
                   double *const *g, float *const *t, __half *const *hi, __half *const *lo,
                   int nprob, cudaStream_t st, int passes) {
  for (int pass = 0; pass < passes; ++pass) {
    const bool last = pass == passes - 1;
    TSVD_TRY(gram_batched((const float *const *)x, rows, max_rows, W.l, kLp, g, W.gram_work,
                          W.gram_bytes, nprob, st));
    TSVD_TRY(chol_inverse_batched(g, t, W.l, nprob, st));
    TSVD_TRY(apply_right_batched((const float *const *)x, rows, max_rows, kLp,
                                 (const float *const *)t, kLp, W.l, W.l, nullptr, x, kLp,
                                 last ? hi : nullptr, last ? lo : nullptr, kSplitScale, nprob,
                                 st));
  }
  return TSVD_OK;
}

// U (nsrc x d fp32, ld d; orthonormal columns, |u| <= 1) -> hi + lo halves of
// U * scale in the [sp][kLp] layout of the skinny GEMM operand, zero padded.
__global__ void lp_split_kernel(const float *__restrict__ u, int nsrc, int d, int sp,
                                __half *__restrict__ hi, __half *__restrict__ lo, float scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)sp * kLp;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / kLp), c = (int)(i % kLp);
    const float x = (r < nsrc && c < d) ? u[(int64_t)r * d + c] * scale : 0.f;
    const __half h = __float2half_rn(x);
    hi[i] = h;
    lo[i] = __float2half_rn(x - __half2float(h));
  }
}

}  // namespace

tsvd_status frpca_work_alloc(FrpcaWork &W, int nmax, int64_t rows_max, int sp, int l, int d) {
  W.nmax = nmax;
  W.rows_max = std::max<int64_t>(rows_max, 1);
  W.sp = sp;
  W.l = l;
  W.d = d;
  size_t rk = (size_t)nmax * W.rows_max * kLp;
  size_t sk = (size_t)nmax * sp * kLp;
  TSVD_CUDA(cudaMalloc(&W.xhi, rk * sizeof(__half)));
  TSVD_CUDA(cudaMalloc(&W.xlo, rk * sizeof(__half)));
  TSVD_CUDA(cudaMalloc(&W.z, std::max(rk, (size_t)nmax * sp * 256) * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.y, sk * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.qhi, sk * sizeof(__half)));
  TSVD_CUDA(cudaMalloc(&W.qlo, sk * sizeof(__half)));
  TSVD_CUDA(cudaMalloc(&W.g, (size_t)nmax * 256 * 256 * sizeof(double)));
  TSVD_CUDA(cudaMalloc(&W.t, (size_t)nmax * kLp * kLp * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.lambda, (size_t)nmax * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.v, (size_t)nmax * 256 * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.colscale, (size_t)nmax * 2 * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.sums, (size_t)nmax * sizeof(double)));
  {
    // every batched Gram uses at most min(nprob * rows/128, 2048) row chunks
    const int64_t rows = std::max<int64_t>(W.rows_max, sp);
    const int64_t chunks = std::min<int64_t>((int64_t)nmax * ceil_div(rows, 128), 2048) + nmax;
    W.gram_bytes = (size_t)chunks * 256 * 256 * sizeof(double);
  }
  TSVD_CUDA(cudaMalloc(&W.gram_work, W.gram_bytes));
  W.jac_bytes = std::max(jacobi_work_bytes(256, nmax), jacobi_work_bytes(l, nmax));
  TSVD_CUDA(cudaMalloc(&W.jac_work, W.jac_bytes));
  W.ptr_slots = (size_t)nmax * 64 + 256;
  TSVD_CUDA(cudaMalloc(&W.dptr, W.ptr_slots * sizeof(void *)));
  TSVD_CUDA(cudaMallocHost(&W.hptr, W.ptr_slots * sizeof(void *)));
  TSVD_CUDA(cudaMalloc(&W.dint, W.ptr_slots * sizeof(int32_t)));
  TSVD_CUDA(cudaMallocHost(&W.hint, W.ptr_slots * sizeof(int32_t)));
  W.tmap_slots = (size_t)nmax * 6;
  TSVD_CUDA(cudaMalloc(&W.tmap_dev, W.tmap_slots * sizeof(CUtensorMap)));
  TSVD_CUDA(cudaMallocHost(&W.tmap_host, W.tmap_slots * sizeof(CUtensorMap)));
  for (double **p : {&W.dv, &W.dt, &W.dh})
    TSVD_CUDA(cudaMalloc(p, (size_t)nmax * 256 * 256 * sizeof(double)));
  {
    std::vector<double *> hp(nmax);
    for (int i = 0; i < nmax; ++i) hp[i] = W.dh + (int64_t)i * 256 * 256;
    TSVD_CUDA(cudaMalloc(&W.dh_ptrs, sizeof(double *) * nmax));
    TSVD_CUDA(cudaMemcpy(W.dh_ptrs, hp.data(), sizeof(double *) * nmax, cudaMemcpyHostToDevice));
  }
  return TSVD_OK;
}

void frpca_work_free(FrpcaWork &W) {
  cudaFree(W.xhi); cudaFree(W.xlo); cudaFree(W.z); cudaFree(W.y); cudaFree(W.qhi);
  cudaFree(W.qlo); cudaFree(W.g); cudaFree(W.t); cudaFree(W.lambda); cudaFree(W.v);
  cudaFree(W.colscale); cudaFree(W.sums); cudaFree(W.gram_work); cudaFree(W.jac_work); cudaFree(W.dptr);
  cudaFreeHost(W.hptr); cudaFree(W.dint); cudaFreeHost(W.hint);
  cudaFree(W.tmap_dev); cudaFreeHost(W.tmap_host);
  cudaFree(W.wm); cudaFree(W.wv); cudaFree(W.ww); cudaFree(W.wy); cudaFree(W.wy2);
  cudaFree(W.wchol); cudaFree(W.wnorm); cudaFree(W.wk);
  cudaFree(W.dv); cudaFree(W.dt); cudaFree(W.dh); cudaFree(W.dh_ptrs);
  cudaGetLastError();  // the launch checks read this slot: leave nothing from teardown in it
  W = FrpcaWork();
}

namespace {

__global__ void widen_kernel(const float *__restrict__ v, double *__restrict__ out, int64_t count,
                             int64_t stride_in, int64_t stride_out) {
  const int prob = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    out[prob * stride_out + i] = v[prob * stride_in + i];
}

// C = op(A) B for n x n row-major fp64 matrices, problem z at offset z * S;
// op(A) = A (trans_a 0) or A^T (1). 16 x 16 output tiles, k staged in shared
// memory.
__global__ void __launch_bounds__(256) dgemm_small_kernel(const double *__restrict__ A,
                                                          const double *__restrict__ B,
                                                          double *__restrict__ C, int n, int64_t S,
                                                          int trans_a) {
  __shared__ double sa[16][17], sb[16][17];
  const int z = blockIdx.z, ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  const int i = blockIdx.y * 16 + ty, j = blockIdx.x * 16 + tx;
  const double *Az = A + z * S, *Bz = B + z * S;
  double acc = 0.0;
  for (int k0 = 0; k0 < n; k0 += 16) {
    const int ka = k0 + tx, kb = k0 + ty;
    // sa[ty][tx] = op(A)[i][k0 + tx]
    sa[ty][tx] = (i < n && ka < n) ? (trans_a ? Az[(int64_t)ka * n + i] : Az[(int64_t)i * n + ka])
                                   : 0.0;
    sb[ty][tx] = (kb < n && j < n) ? Bz[(int64_t)kb * n + j] : 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) acc = fma(sa[ty][k], sb[k][tx], acc);
    __syncthreads();
  }
  if (i < n && j < n) C[z * S + (int64_t)i * n + j] = acc;
}

}  // namespace

// Eigenpairs of the Grams G[i] = W.g + i 256^2 (n x n fp64) to the accuracy
// the fp64 Gram carries. The fp32 Jacobi's absolute error, a few eps_32 times
// the largest eigenvalue, is a large relative error on the small ones (the
// Gram squares the spread of the singular values), so its eigenvectors V
// (W.v) are refined: H = V^T G V in fp64 (nearly diagonal), a Jacobi on H
// that carries the diagonal in fp64, its rotations replayed onto V. lam / v:
// pointer arrays to W.lambda / W.v of each problem.
tsvd_status eig_refined(FrpcaWork &W, double *const *d_g, int n, float *const *d_lam,
                        float *const *d_v, int nprob, cudaStream_t st) {
  TSVD_TRY(jacobi_eig_batched(d_g, n, d_lam, d_v, nprob, W.jac_work, W.jac_bytes, st,
                              &W.last_sweeps));
  const int64_t S = 256 * 256;
  widen_kernel<<<dim3(grid_for((int64_t)n * n, 256, 1), nprob), 256, 0, st>>>(W.v, W.dv,
                                                                            (int64_t)n * n, S, S);
  TSVD_LAUNCH_CHECK();
  // T = G V, H = V^T T (fp64)
  const dim3 grid(ceil_div(n, 16), ceil_div(n, 16), nprob);
  dgemm_small_kernel<<<grid, 256, 0, st>>>(W.g, W.dv, W.dt, n, S, 0);
  TSVD_LAUNCH_CHECK();
  dgemm_small_kernel<<<grid, 256, 0, st>>>(W.dv, W.dt, W.dh, n, S, 1);
  TSVD_LAUNCH_CHECK();
  // the rotations are replayed onto V in place (each replay block reads its
  // rows before writing them)
  return jacobi_eig_batched(W.dh_ptrs, n, d_lam, d_v, nprob, W.jac_work, W.jac_bytes, st,
                            &W.last_refine_sweeps, 1, (const float *const *)d_v);
}

tsvd_status frpca_batch(FrpcaWork &W, const FrpcaProblem *probs, int nprob, int q, uint64_t seed,
                        int nsrc, cudaStream_t st, double *sum_sigma2) {
  if (nprob == 0) return TSVD_OK;
  if (nprob > W.nmax) return fail(TSVD_ERR_INVALID, "frpca: %d problems > %d", nprob, W.nmax);
  if (q < 1) return fail(TSVD_ERR_INVALID, "frpca: q=%d", q);
  TSVD_CUDA(cudaStreamSynchronize(st));  // staging buffers are free again
  const int sp = W.sp, l = W.l, d = W.d;
  const int64_t RK = W.rows_max * kLp, SK = (int64_t)sp * kLp;
  std::vector<const __half *> at(nprob);
  std::vector<__half *> xhi(nprob), xlo(nprob), qhi(nprob), qlo(nprob);
  std::vector<float *> z(nprob), y(nprob), t(nprob), lam(nprob), v(nprob), cs(nprob), csi(nprob),
      bout(nprob), sout(nprob), uout(nprob), vout(nprob);
  std::vector<double *> g(nprob);
  std::vector<const int32_t *> cmap(nprob);
  std::vector<int32_t> ncols(nprob), sprows(nprob, sp), cbase(nprob), blk(nprob), srcrows(nprob, nsrc);
  int max_nc = 0;
  bool want_uv = false;
  for (int i = 0; i < nprob; ++i) {
    const FrpcaProblem &P = probs[i];
    at[i] = P.at;
    ncols[i] = P.ncols;
    max_nc = std::max(max_nc, P.ncols);
    if (P.ncols > W.rows_max) return fail(TSVD_ERR_INVALID, "frpca: block too wide");
    xhi[i] = W.xhi + i * RK;
    xlo[i] = W.xlo + i * RK;
    z[i] = W.z + i * RK;
    y[i] = W.y + i * SK;
    qhi[i] = W.qhi + i * SK;
    qlo[i] = W.qlo + i * SK;
    g[i] = W.g + (int64_t)i * 256 * 256;
    t[i] = W.t + (int64_t)i * kLp * kLp;
    lam[i] = W.lambda + i * 256;
    v[i] = W.v + (int64_t)i * 256 * 256;
    cs[i] = W.colscale + i * 512;
    csi[i] = W.colscale + i * 512 + 256;
    bout[i] = P.b_out;
    sout[i] = P.sigma_out;
    uout[i] = P.u_out;
    vout[i] = P.v_out;
    want_uv = want_uv || P.u_out || P.v_out;
    cmap[i] = P.colmap;
    cbase[i] = P.col_base;
    blk[i] = P.block;
  }
  const bool sparse = probs[0].sparse != nullptr;
  std::vector<const int64_t *> rptr(nprob), cptr(nprob);
  std::vector<const int32_t *> ridx(nprob), cidx(nprob);
  std::vector<const float *> rval(nprob), cval(nprob);
  for (int i = 0; i < nprob; ++i) {
    const SparseBlock *sb = probs[i].sparse;
    if ((sb != nullptr) != sparse)
      return fail(TSVD_ERR_INVALID, "frpca: a batch mixes sparse and dense blocks");
    if (!sb) continue;
    if (sb->cols != ncols[i] || sb->rows != sp)
      return fail(TSVD_ERR_INVALID, "frpca: sparse block %d x %d, expected %d x %d", sb->rows,
                  sb->cols, sp, ncols[i]);
    rptr[i] = sb->rowptr; ridx[i] = sb->colidx; rval[i] = sb->rval;
    cptr[i] = sb->colptr; cidx[i] = sb->rowidx; cval[i] = sb->cval;
  }
  PtrPack pk(W);
  auto d_at = pk.add(at);
  auto d_xhi = pk.add(xhi), d_xlo = pk.add(xlo), d_qhi = pk.add(qhi), d_qlo = pk.add(qlo);
  auto d_rptr = pk.add(rptr), d_cptr = pk.add(cptr);
  auto d_ridx = pk.add(ridx), d_cidx = pk.add(cidx);
  auto d_rval = pk.add(rval), d_cval = pk.add(cval);
  auto d_z = pk.add(z), d_y = pk.add(y), d_t = pk.add(t), d_lam = pk.add(lam), d_v = pk.add(v);
  auto d_cs = pk.add(cs), d_csi = pk.add(csi), d_bout = pk.add(bout), d_sout = pk.add(sout);
  auto d_uout = pk.add(uout), d_vout = pk.add(vout);
  auto d_g = pk.add(g);
  auto d_cmap = pk.add(cmap);
  const int32_t *d_nc = pk.add_int(ncols), *d_sprows = pk.add_int(sprows),
                *d_cbase = pk.add_int(cbase), *d_blk = pk.add_int(blk),
                *d_srcrows = pk.add_int(srcrows);
  TSVD_TRY(pk.upload(st));
  // tensor maps of the products: forward (A, X hi, X lo), backward (A, Q hi, Q lo)
  if (!sparse) {
    if ((size_t)nprob * 6 > W.tmap_slots)
      return fail(TSVD_ERR_INVALID, "frpca: %d problems exceed the tensor-map area", nprob);
    TSVD_TRY(gemm_encode_maps(1, nprob, at.data(), ncols.data(), sp, xhi.data(), xlo.data(),
                              W.tmap_host));
    TSVD_TRY(gemm_encode_maps(0, nprob, at.data(), ncols.data(), sp, qhi.data(), qlo.data(),
                              W.tmap_host + 3 * (size_t)nprob));
    TSVD_CUDA(cudaMemcpyAsync(W.tmap_dev, W.tmap_host, sizeof(CUtensorMap) * 6 * nprob,
                              cudaMemcpyHostToDevice, st));
  }
  const GemmBatch gb_fwd{d_nc, sp, nprob, W.tmap_dev};
  const GemmBatch gb_bwd{d_nc, sp, nprob, W.tmap_dev + 3 * (size_t)nprob};
  const size_t ybytes = (size_t)nprob * SK * sizeof(float);
  // Y = A X (sp x kLp) and Z = A^T Q (n_c x kLp): tensor-core GEMMs on the
  // half-precision A^T, or FP32 SpMM over the block's CSR / CSC
  auto prod_fwd = [&](const __half *const *hi, const __half *const *lo,
                      float scale) -> tsvd_status {
    if (sparse)
      return spmm_batched(d_rptr, d_ridx, d_rval, d_sprows, sp, hi, lo, d_y, scale, nprob, st);
    return gemm_fwd(gb_fwd, lo != nullptr, d_y, W.y, ybytes, sp, max_nc, scale, st);
  };
  auto prod_bwd = [&](const __half *const *hi, const __half *const *lo,
                      float scale) -> tsvd_status {
    if (sparse)
      return spmm_batched(d_cptr, d_cidx, d_cval, d_nc, max_nc, hi, lo, d_z, scale, nprob, st);
    return gemm_bwd(gb_bwd, lo != nullptr, d_z, sp, max_nc, scale, st);
  };
  const int niter = (q - 1) / 2;
  float in_scale = 1.f / kSplitScale;
  if (q % 2 == 0) {
    omega_kernel<<<dim3(grid_for((int64_t)max_nc * kLp, 256, 4), nprob), 256, 0, st>>>(
        d_xhi, d_nc, d_cmap, d_cbase, d_blk, W.rows_max, l, seed);
    TSVD_LAUNCH_CHECK();
    TSVD_TRY(prod_fwd((const __half *const *)d_xhi, nullptr, 1.f));
    TSVD_TRY(cholqr(W, d_y, d_sprows, sp, d_g, d_t, d_qhi, d_qlo, nprob, st, niter ? 1 : 2));
  } else {
    const float split = 2048.f;
    randq_kernel<<<dim3(grid_for(SK, 256, 4), nprob), 256, 0, st>>>(d_y, d_qhi, d_qlo, d_blk, sp,
                                                                      nsrc, l, seed, split);
    TSVD_LAUNCH_CHECK();
    in_scale = 1.f / split;
  }
  // Between products one CholeskyQR pass suffices: every product multiplies
  // the condition number of an (almost) orthonormal basis by at most
  // sigma_1 / sigma_l of A, and only the span goes on (the reference uses an
  // LU factor there, frpca.c:261-291). The last basis Q, which B = Q V S is
  // built from, gets both passes.
  for (int it = 1; it <= niter; ++it) {
    TSVD_TRY(prod_bwd((const __half *const *)d_qhi, (const __half *const *)d_qlo, in_scale));
    TSVD_TRY(cholqr(W, d_z, d_nc, max_nc, d_g, d_t, d_xhi, d_xlo, nprob, st, 1));
    TSVD_TRY(prod_fwd((const __half *const *)d_xhi, (const __half *const *)d_xlo,
                      1.f / kSplitScale));
    TSVD_TRY(cholqr(W, d_y, d_sprows, sp, d_g, d_t, d_qhi, d_qlo, nprob, st, it == niter ? 2 : 1));
    in_scale = 1.f / kSplitScale;
  }
  TSVD_TRY(prod_bwd((const __half *const *)d_qhi, (const __half *const *)d_qlo, in_scale));
  // eigSVD of Z = A^T Q (frpca.c:99-136): Gram, eigenpairs, top-d.
  TSVD_TRY(gram_batched((const float *const *)d_z, d_nc, max_nc, l, kLp, d_g, W.gram_work,
                        W.gram_bytes, nprob, st));
  TSVD_TRY(eig_refined(W, d_g, l, d_lam, d_v, nprob, st));
  double *d_sum2 = W.sums;
  sigma_kernel<<<nprob, 128, 0, st>>>((const float *const *)d_lam, d, d_cs, d_csi, d_sout, d_sum2);
  TSVD_LAUNCH_CHECK();
  // B = Q V_d diag(sigma) (Tree_u_NC.cpp:148-154)
  bool any_b = false;
  for (int i = 0; i < nprob; ++i) any_b = any_b || bout[i];
  if (any_b)
    TSVD_TRY(apply_right_batched((const float *const *)d_y, d_srcrows, nsrc, kLp,
                                 (const float *const *)d_v, l, l, d, (const float *const *)d_cs,
                                 d_bout, d, nullptr, nullptr, 1.f, nprob, st));
  if (want_uv) {
    TSVD_TRY(apply_right_batched((const float *const *)d_y, d_srcrows, nsrc, kLp,
                                 (const float *const *)d_v, l, l, d, nullptr, d_uout, d, nullptr,
                                 nullptr, 1.f, nprob, st));
    TSVD_TRY(apply_right_batched((const float *const *)d_z, d_nc, max_nc, kLp,
                                 (const float *const *)d_v, l, l, d, (const float *const *)d_csi,
                                 d_vout, d, nullptr, nullptr, 1.f, nprob, st));
  }
  std::vector<double> hs(nprob);
  TSVD_CUDA(cudaMemcpyAsync(hs.data(), d_sum2, sizeof(double) * nprob, cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  if (sum_sigma2)
    for (int i = 0; i < nprob; ++i) sum_sigma2[i] = hs[i];
  return gemm_check(st);
}

namespace {

// The Rayleigh-Ritz end of a merge: for each problem, the n-column matrix
// m[i] (|S| x n, ld n) -> Gram (compensated, fp64) -> Jacobi eigenpairs ->
// out = m V_d diag(f(s)), sigma_out = s (the d largest singular values).
tsvd_status merge_finish(FrpcaWork &W, const MergeProblem *probs, int nprob, int n, int nsrc,
                         int root_mode, const std::vector<float *> &m, cudaStream_t st) {
  const int d = W.d;
  std::vector<float *> lam(nprob), v(nprob), cs(nprob), out(nprob), sout(nprob);
  std::vector<double *> g(nprob);
  std::vector<int32_t> rows(nprob, nsrc);
  for (int i = 0; i < nprob; ++i) {
    g[i] = W.g + (int64_t)i * 256 * 256;
    lam[i] = W.lambda + i * 256;
    v[i] = W.v + (int64_t)i * 256 * 256;
    cs[i] = W.colscale + i * 512;
    out[i] = probs[i].out;
    sout[i] = probs[i].sigma_out;
  }
  TSVD_CUDA(cudaStreamSynchronize(st));  // the pointer staging area is reused
  PtrPack pk(W);
  auto d_m = pk.add(m);
  auto d_lam = pk.add(lam), d_v = pk.add(v), d_cs = pk.add(cs), d_out = pk.add(out),
       d_sout = pk.add(sout);
  auto d_g = pk.add(g);
  const int32_t *d_rows = pk.add_int(rows);
  TSVD_TRY(pk.upload(st));
  TSVD_TRY(gram_batched((const float *const *)d_m, d_rows, nsrc, n, n, d_g, W.gram_work,
                        W.gram_bytes, nprob, st));
  TSVD_TRY(eig_refined(W, d_g, n, d_lam, d_v, nprob, st));
  merge_scale_kernel<<<nprob, 128, 0, st>>>((const float *const *)d_lam, d, root_mode, d_cs,
                                            d_sout);
  TSVD_LAUNCH_CHECK();
  TSVD_TRY(apply_right_batched((const float *const *)d_m, d_rows, nsrc, n,
                               (const float *const *)d_v, n, n, d, (const float *const *)d_cs,
                               d_out, d, nullptr, nullptr, 1.f, nprob, st));
  return TSVD_OK;
}

__global__ void colnorm_kernel(const float *__restrict__ m, int64_t nsrc, int n,
                               float *__restrict__ norm) {
  const int prob = blockIdx.y;
  const float *M = m + (int64_t)prob * nsrc * n;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int64_t s = 0; s < nsrc; ++s) acc = fmaf(M[s * n + c], M[s * n + c], acc);
    norm[(int64_t)prob * n + c] = acc;
  }
}

// V[i] (n x p, row-major) = the columns sel[i][0..p) of the n x n identity.
__global__ void select_basis_kernel(const int32_t *__restrict__ sel, int n, int p,
                                    float *__restrict__ v) {
  const int prob = blockIdx.y;
  float *V = v + (int64_t)prob * n * p;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)n * p;
       i += (int64_t)gridDim.x * blockDim.x)
    V[i] = 0.f;
  __syncthreads();
  if (blockIdx.x == 0)
    for (int j = threadIdx.x; j < p; j += blockDim.x) V[(int64_t)sel[prob * p + j] * p + j] = 1.f;
}

__global__ void diag_sum_kernel(double *const *g, int l, double *out) {
  const int prob = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < l; i += blockDim.x) acc += g[prob][(int64_t)i * l + i];
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[prob] = red[0];
}


constexpr int64_t kWideK = 256 * 256 + 256 * 257 / 2;  // fp32 Gram + packed factor

// Buffers for up to `nprob` problems of n columns and W.sp rows.
tsvd_status wide_reserve(FrpcaWork &W, int nprob, int n) {
  const int nsrc = W.sp;
  const size_t need = (size_t)nprob * nsrc * n;
  if (need <= W.wide_cap && nprob <= W.wide_nprob && n <= W.wide_n && W.wm) return TSVD_OK;
  cudaFree(W.wm); cudaFree(W.wv); cudaFree(W.ww); cudaFree(W.wy); cudaFree(W.wy2);
  cudaFree(W.wchol); cudaFree(W.wnorm); cudaFree(W.wk);
  W.wm = W.wv = W.ww = W.wy = W.wy2 = W.wnorm = W.wk = nullptr;
  W.wchol = nullptr;
  W.wide_cap = 0;
  TSVD_CUDA(cudaMalloc(&W.wm, need * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.wv, (size_t)nprob * n * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.ww, (size_t)nprob * n * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.wy, (size_t)nprob * nsrc * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.wy2, (size_t)nprob * nsrc * 256 * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.wchol, (size_t)nprob * 2 * 256 * 256 * sizeof(double)));
  TSVD_CUDA(cudaMalloc(&W.wnorm, (size_t)nprob * n * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&W.wk, (size_t)nprob * kWideK * sizeof(float)));
  W.wide_cap = need;
  W.wide_nprob = nprob;
  W.wide_n = n;
  return TSVD_OK;
}

// x[i] (rows x p, ld p) -> x[i] R^-1 into y[i], R from the compensated Gram;
// energy (optional, host, nprob) receives trace(x^T x) = ||x||_F^2 per problem.
tsvd_status orthonormalize(FrpcaWork &W, float *x, int64_t xstride, float *y, int rows, int p,
                           int nprob, cudaStream_t st, double *energy) {
  std::vector<float *> xs(nprob);
  std::vector<double *> g(nprob);
  std::vector<int32_t> rr(nprob, rows);
  for (int i = 0; i < nprob; ++i) {
    xs[i] = x + i * xstride;
    g[i] = W.g + (int64_t)i * 256 * 256;
  }
  TSVD_CUDA(cudaStreamSynchronize(st));  // the pointer staging area is reused
  PtrPack pk(W);
  auto d_x = pk.add(xs);
  auto d_g = pk.add(g);
  const int32_t *d_rows = pk.add_int(rr);
  TSVD_TRY(pk.upload(st));
  TSVD_TRY(gram_batched((const float *const *)d_x, d_rows, rows, p, p, d_g, W.gram_work,
                        W.gram_bytes, nprob, st));
  if (energy) {
    diag_sum_kernel<<<nprob, 256, 0, st>>>(d_g, p, W.sums);
    TSVD_LAUNCH_CHECK();
    TSVD_CUDA(cudaMemcpyAsync(energy, W.sums, sizeof(double) * nprob, cudaMemcpyDeviceToHost, st));
  }
  TSVD_TRY(chol_solve_wide_batched(d_g, W.wchol, x, y, rows, p, xstride, nprob, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  return TSVD_OK;
}

// Merge of h * d > 256 columns. The top-d singular triplets of M = [B_1..B_h]
// (|S| x n) come from a p = min(256, n, |S|) dimensional basis V of M's
// dominant right singular subspace, found by subspace iteration
// (Y = M V, W = M^T Y, each product re-orthonormalized by CholeskyQR on a
// compensated Gram), started from the p columns of M with the largest norms
// and stopped when ||M V||_F^2 gains less than 1e-7 of itself. The result is
// then the merge of the p columns of M V (compensated Gram + Jacobi), the
// same arithmetic as a narrow merge. The products are plain fp32 GEMMs
// (sgemm_batched: fixed-order sums, 64 x 64 tiles).
tsvd_status merge_wide_core(FrpcaWork &W, const MergeProblem *probs, int nprob, int n, int nsrc,
                            int root_mode, cudaStream_t st);

tsvd_status merge_wide(FrpcaWork &W, const MergeProblem *probs, int nprob, int h, int nsrc,
                       int root_mode, cudaStream_t st) {
  const int d = W.d, n = h * d;
  if (nsrc > W.sp) return fail(TSVD_ERR_INVALID, "merge: |S| = %d > %d", nsrc, W.sp);
  TSVD_TRY(wide_reserve(W, std::max(nprob, W.nmax / h), n));
  const int64_t sm = (int64_t)nsrc * n;
  // M = [B_1 .. B_h], one |S| x n row-major matrix per problem
  {
    std::vector<const float *> ch((size_t)nprob * h);
    std::vector<float *> m(nprob);
    for (int i = 0; i < nprob; ++i) {
      for (int c = 0; c < h; ++c) ch[(size_t)i * h + c] = probs[i].children[c];
      m[i] = W.wm + i * sm;
    }
    TSVD_CUDA(cudaStreamSynchronize(st));
    PtrPack pk(W);
    auto d_ch = pk.add(ch);
    auto d_m = pk.add(m);
    TSVD_TRY(pk.upload(st));
    concat_kernel<<<dim3(grid_for((int64_t)nsrc * n, 256, 4), nprob), 256, 0, st>>>(d_ch, h, d,
                                                                                   nsrc, d_m);
    TSVD_LAUNCH_CHECK();
  }
  return merge_wide_core(W, probs, nprob, n, nsrc, root_mode, st);
}

// The wide merge of the n-column matrices already in W.wm (problem i at
// i |S| n, row-major |S| x n).
tsvd_status merge_wide_core(FrpcaWork &W, const MergeProblem *probs, int nprob, int n, int nsrc,
                            int root_mode, cudaStream_t st) {
  const int d = W.d;
  const int p = std::min(256, std::min(n, nsrc));
  if (p < d) return fail(TSVD_ERR_INVALID, "merge: %d rows or columns, below rank d = %d",
                         std::min(n, nsrc), d);
  const int64_t sm = (int64_t)nsrc * n, sv = (int64_t)n * p, sy = (int64_t)nsrc * p;
  // start: the p columns of M with the largest norms (the children's largest sigmas)
  colnorm_kernel<<<dim3(ceil_div(n, 256), nprob), 256, 0, st>>>(W.wm, nsrc, n, W.wnorm);
  TSVD_LAUNCH_CHECK();
  std::vector<float> norms((size_t)nprob * n);
  TSVD_CUDA(cudaMemcpyAsync(norms.data(), W.wnorm, sizeof(float) * norms.size(),
                            cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  std::vector<int32_t> sel((size_t)nprob * p);
  for (int i = 0; i < nprob; ++i) {
    std::vector<int32_t> idx(n);
    for (int c = 0; c < n; ++c) idx[c] = c;
    const float *nr = norms.data() + (size_t)i * n;
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return nr[a] > nr[b]; });
    std::copy(idx.begin(), idx.begin() + p, sel.begin() + (size_t)i * p);
  }
  {
    PtrPack pk(W);
    const int32_t *d_sel = pk.add_int(sel);
    TSVD_TRY(pk.upload(st));
    select_basis_kernel<<<dim3(1, nprob), 256, 0, st>>>(d_sel, n, p, W.wv);
    TSVD_LAUNCH_CHECK();
    TSVD_CUDA(cudaStreamSynchronize(st));
  }
  std::vector<double> energy(nprob), prev(nprob, 0.0);
  // x (rows x p, row-major, problem stride xs) -> y: fp32 Gram (problem i at
  // W.wk + i p p), shifted fp32 Cholesky (packed factors after all the
  // Grams), triangular solve.
  const int64_t kp = (int64_t)p * p;
  auto cheap_basis = [&](const float *x, int64_t xs, float *y, int rows) -> tsvd_status {
    // K = x^T x (p x p)
    TSVD_TRY(sgemm_batched(true, p, p, rows, x, p, xs, x, p, xs, W.wk, p, kp, nprob, st));
    TSVD_TRY(chol_shift_solve_batched(W.wk, W.wk + nprob * kp, x, y, rows, p, xs, 1e-6f, nprob,
                                      st));
    return TSVD_OK;
  };
  int it = 0;
  for (; it < 40; ++it) {
    // Y = M V (|S| x p)
    TSVD_TRY(sgemm_batched(false, nsrc, p, n, W.wm, n, sm, W.wv, p, sv, W.wy, p, sy, nprob, st));
    TSVD_TRY(cheap_basis(W.wy, sy, W.wy2, nsrc));
    // ||M V||_F^2 = trace(Y^T Y), from the diagonal of the Gram just formed
    std::vector<float> diag((size_t)nprob * p);
    for (int i = 0; i < nprob; ++i)
      TSVD_CUDA(cudaMemcpy2DAsync(diag.data() + (size_t)i * p, sizeof(float),
                                  W.wk + i * kp, (p + 1) * sizeof(float), sizeof(float), p,
                                  cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
    bool done = it > 0;
    for (int i = 0; i < nprob; ++i) {
      double e = 0.0;
      for (int j = 0; j < p; ++j) e += diag[(size_t)i * p + j];
      energy[i] = e;
      if (!(energy[i] - prev[i] <= 1e-6 * energy[i])) done = false;
    }
    prev = energy;
    if (done) break;
    // W = M^T Yq (n x p)
    TSVD_TRY(sgemm_batched(true, n, p, nsrc, W.wm, n, sm, W.wy2, p, sy, W.ww, p, sv, nprob, st));
    TSVD_TRY(cheap_basis(W.ww, sv, W.wv, n));
  }
  // one accurate CholeskyQR pass: an orthonormal V to working precision
  TSVD_CUDA(cudaMemcpyAsync(W.ww, W.wv, sizeof(float) * nprob * sv, cudaMemcpyDeviceToDevice, st));
  TSVD_TRY(orthonormalize(W, W.ww, sv, W.wv, n, p, nprob, st, nullptr));
  W.wide_iters = it + 1;
  // Rayleigh-Ritz: the narrow merge of the p columns of Z = M V
  const int64_t RK = std::max<int64_t>(W.rows_max * kLp, (int64_t)W.sp * 256);
  std::vector<float *> z(nprob);
  for (int i = 0; i < nprob; ++i) z[i] = W.z + i * RK;
  // Z = M V (|S| x p), problem i at W.z + i RK
  TSVD_TRY(sgemm_batched(false, nsrc, p, n, W.wm, n, sm, W.wv, p, sv, W.z, p, RK, nprob, st));
  return merge_finish(W, probs, nprob, p, nsrc, root_mode, z, st);
}

}  // namespace

tsvd_status merge_matrix(FrpcaWork &W, const float *m_host, int rows, int cols, float *out,
                         float *sigma_out, cudaStream_t st) {
  if (rows > W.sp) return fail(TSVD_ERR_INVALID, "merge: %d rows > %d", rows, W.sp);
  MergeProblem prob{};
  prob.out = out;
  prob.sigma_out = sigma_out;
  if (cols > 256) {
    TSVD_TRY(wide_reserve(W, 1, cols));
    TSVD_CUDA(cudaMemcpyAsync(W.wm, m_host, sizeof(float) * rows * cols, cudaMemcpyHostToDevice,
                              st));
    return merge_wide_core(W, &prob, 1, cols, rows, 0, st);
  }
  TSVD_CUDA(cudaMemcpyAsync(W.z, m_host, sizeof(float) * rows * cols, cudaMemcpyHostToDevice, st));
  return merge_finish(W, &prob, 1, cols, rows, 0, std::vector<float *>{W.z}, st);
}

tsvd_status merge_batch(FrpcaWork &W, const MergeProblem *probs, int nprob, int h, int nsrc,
                        int root_mode, cudaStream_t st) {
  W.wide_iters = 0;
  if (nprob == 0) return TSVD_OK;
  const int d = W.d, n = h * d;
  if (nprob > W.nmax) return fail(TSVD_ERR_INVALID, "merge: too many parents");
  if (n > 256) return merge_wide(W, probs, nprob, h, nsrc, root_mode, st);
  TSVD_CUDA(cudaStreamSynchronize(st));
  // per-parent concatenation buffers inside the z area (sized for both uses)
  const int64_t RK = std::max<int64_t>(W.rows_max * kLp, (int64_t)W.sp * 256);
  std::vector<const float *> ch((size_t)nprob * h);
  std::vector<float *> m(nprob);
  for (int i = 0; i < nprob; ++i) {
    for (int c = 0; c < h; ++c) ch[(size_t)i * h + c] = probs[i].children[c];
    m[i] = W.z + i * RK;
  }
  {
    PtrPack pk(W);
    auto d_ch = pk.add(ch);
    auto d_m = pk.add(m);
    TSVD_TRY(pk.upload(st));
    concat_kernel<<<dim3(grid_for((int64_t)nsrc * n, 256, 4), nprob), 256, 0, st>>>(d_ch, h, d,
                                                                                   nsrc, d_m);
    TSVD_LAUNCH_CHECK();
  }
  return merge_finish(W, probs, nprob, n, nsrc, root_mode, m, st);
}

tsvd_status lp_right_batch(FrpcaWork &W, const LpProblem *probs, int nprob, const float *u,
                           int nsrc, int d, cudaStream_t st) {
  if (nprob == 0) return TSVD_OK;
  if (nprob > W.nmax) return fail(TSVD_ERR_INVALID, "lp: too many blocks");
  if (d > kLp || nsrc > W.sp) return fail(TSVD_ERR_INVALID, "lp: d = %d, |S| = %d", d, nsrc);
  TSVD_CUDA(cudaStreamSynchronize(st));  // the pointer staging area is reused
  // one split of U, shared by every block
  lp_split_kernel<<<grid_for((int64_t)W.sp * kLp, 256, 4), 256, 0, st>>>(u, nsrc, d, W.sp, W.qhi,
                                                                         W.qlo, kSplitScale);
  TSVD_LAUNCH_CHECK();
  std::vector<const __half *> at(nprob), yhi(nprob, W.qhi), ylo(nprob, W.qlo);
  std::vector<float *> z(nprob);
  std::vector<int32_t> nc(nprob);
  int max_nc = 0;
  for (int i = 0; i < nprob; ++i) {
    at[i] = probs[i].at;
    z[i] = probs[i].v_out;
    nc[i] = probs[i].ncols;
    max_nc = std::max(max_nc, (int)probs[i].ncols);
  }
  if (max_nc == 0) return TSVD_OK;
  if ((size_t)nprob * 3 > W.tmap_slots)
    return fail(TSVD_ERR_INVALID, "lp: %d blocks exceed the tensor-map area", nprob);
  PtrPack pk(W);
  auto d_z = pk.add(z);
  const int32_t *d_nc = pk.add_int(nc);
  TSVD_TRY(pk.upload(st));
  TSVD_TRY(gemm_encode_maps(0, nprob, at.data(), nc.data(), W.sp, yhi.data(), ylo.data(),
                            W.tmap_host));
  TSVD_CUDA(cudaMemcpyAsync(W.tmap_dev, W.tmap_host, sizeof(CUtensorMap) * 3 * nprob,
                            cudaMemcpyHostToDevice, st));
  const GemmBatch gb{d_nc, W.sp, nprob, W.tmap_dev};
  TSVD_TRY(gemm_bwd(gb, true, d_z, W.sp, max_nc, 1.f / kSplitScale, st));
  return gemm_check(st);
}

}  // namespace tsvd
