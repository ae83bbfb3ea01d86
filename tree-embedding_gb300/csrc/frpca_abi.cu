// frPCA over a caller's CSR matrix: the drop-in for Code/frpca.c:239-326
// (frPCA(mat_csr*, mat**, mat**, mat**, k, q)) and a status-returning form.
//
// tsvd_frpca densifies the CSR on the device into the half-precision A^T
// layout of the mixed form (non-empty columns only, values scaled by a power
// of two into half range) and factorizes it on the tensor cores;
// tsvd_frpca_fp32 (and the legacy frPCA symbol) keep the values in FP32 as a
// CSR / CSC pair and run both products as SpMM (the plain form's products).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "factor.h"
#include "internal.h"
#include "plain.h"

using namespace tsvd;

namespace {

uint64_t g_frpca_seed = 20231;

__global__ void scatter_csr_kernel(const int32_t *rows, const int32_t *cidx, const float *vals,
                                   int64_t nnz, int sp, __half *at) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x)
    at[(int64_t)cidx[i] * sp + rows[i]] = __float2half_rn(vals[i]);
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() { cudaFree(p); }
  tsvd_status alloc(size_t n) {
    TSVD_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)));
    return TSVD_OK;
  }
};

}  // namespace

extern "C" void tsvd_set_frpca_seed(uint64_t seed) { g_frpca_seed = seed; }

namespace {

// A caller's CSR with its empty columns compacted away: triplets in row
// order (explicit zeros dropped), the compacted -> original column map and
// the largest magnitude.
struct HostBlock {
  std::vector<int32_t> trow, tcol, cmap;
  std::vector<double> tval;
  double vmax = 0.0;
};

tsvd_status host_block(int32_t nrows, int32_t ncols, int64_t nnz, const int64_t *row_ptr,
                       const int32_t *col_idx, const double *values, int32_t index_base,
                       HostBlock &H) {
  if (nrows < 1 || ncols < 1 || nnz < 0 || !row_ptr || (nnz > 0 && (!col_idx || !values)))
    return fail(TSVD_ERR_INVALID, "frpca: bad matrix arguments");
  if (index_base != 0 && index_base != 1) return fail(TSVD_ERR_INVALID, "frpca: index_base");
  std::vector<int32_t> cmap_inv(ncols, -1);
  H.trow.reserve(nnz);
  H.tcol.reserve(nnz);
  H.tval.reserve(nnz);
  for (int32_t i = 0; i < nrows; ++i) {
    int64_t b = row_ptr[i] - index_base, e = row_ptr[i + 1] - index_base;
    if (b < 0 || e < b || e > nnz) return fail(TSVD_ERR_INVALID, "frpca: bad row pointers");
    for (int64_t t = b; t < e; ++t) {
      int32_t c = col_idx[t] - index_base;
      if (c < 0 || c >= ncols) return fail(TSVD_ERR_INVALID, "frpca: column out of range");
      if (values[t] == 0.0) continue;
      if (!std::isfinite(values[t])) return fail(TSVD_ERR_NUMERIC, "frpca: non-finite value");
      if (std::fabs(values[t]) > (double)FLT_MAX)
        return fail(TSVD_ERR_INVALID, "frpca: |value| above the float range");
      cmap_inv[c] = 1;
      H.trow.push_back(i);
      H.tcol.push_back(c);
      H.tval.push_back(values[t]);
      H.vmax = std::max(H.vmax, std::fabs(values[t]));
    }
  }
  for (int32_t c = 0; c < ncols; ++c)
    if (cmap_inv[c] > 0) {
      cmap_inv[c] = (int32_t)H.cmap.size();
      H.cmap.push_back(c);
    }
  for (auto &c : H.tcol) c = cmap_inv[c];
  return TSVD_OK;
}

// frPCA of a compacted host block; fp32 = 0: half-precision A^T on the tensor
// cores; fp32 = 1: FP32 CSR / CSC with SpMM products.
tsvd_status frpca_host(int32_t nrows, int32_t ncols, const HostBlock &H, int32_t k, int32_t q,
                       uint64_t seed, int fp32, double *U, double *S, double *V) {
  if (k < 1 || k + 5 > kLp || q < 1) return fail(TSVD_ERR_INVALID, "frpca: k=%d q=%d", k, q);
  const int32_t nc = (int32_t)H.cmap.size();
  const int64_t nnz = (int64_t)H.tval.size();
  // power-of-two scale so that max |a| lands at 2^14 (exact, undone on sigma)
  int e2 = 0;
  if (H.vmax > 0) std::frexp(H.vmax, &e2);
  const double scale = std::ldexp(1.0, 14 - e2);
  const int sp = (int)round_up(nrows, kRowPad);
  const int l = k + 5;
  std::vector<float> hu((size_t)sp * k, 0.f), hv((size_t)std::max(nc, 1) * k, 0.f), hs(k, 0.f);
  if (nc > 0) {
    std::vector<float> tval(nnz);
    for (int64_t t = 0; t < nnz; ++t) tval[t] = (float)((float)H.tval[t] * scale);
    DevBuf<__half> at;
    DevBuf<int32_t> drow, dcol, dcmap, didx_r, didx_c;
    DevBuf<float> dval, du, dv, ds, dval_r, dval_c;
    DevBuf<int64_t> dptr_r, dptr_c;
    SparseBlock sb;
    TSVD_TRY(dcmap.alloc(nc));
    TSVD_TRY(du.alloc((size_t)sp * k));
    TSVD_TRY(dv.alloc((size_t)nc * k));
    TSVD_TRY(ds.alloc(k));
    cudaStream_t st;
    TSVD_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    tsvd_status s1 = TSVD_OK;
    if (fp32) {
      // CSR over the padded rows and CSC over the compacted columns, both with
      // ascending minor indices (counting sorts of the row-ordered triplets)
      std::vector<int64_t> rp(sp + 1, 0), cp(nc + 1, 0);
      for (int64_t t = 0; t < nnz; ++t) {
        rp[H.trow[t] + 1]++;
        cp[H.tcol[t] + 1]++;
      }
      for (int i = 0; i < sp; ++i) rp[i + 1] += rp[i];
      for (int c = 0; c < nc; ++c) cp[c + 1] += cp[c];
      std::vector<int32_t> ci(nnz), ri(nnz);
      std::vector<float> rv(nnz), cv(nnz);
      std::vector<int64_t> rpos(rp.begin(), rp.end() - 1), cpos(cp.begin(), cp.end() - 1);
      std::vector<int64_t> order(nnz);
      for (int64_t t = 0; t < nnz; ++t) order[t] = t;
      std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return H.trow[a] != H.trow[b] ? H.trow[a] < H.trow[b] : H.tcol[a] < H.tcol[b];
      });
      for (int64_t t : order) {
        const int64_t a = rpos[H.trow[t]]++;
        ci[a] = H.tcol[t];
        rv[a] = tval[t];
        const int64_t b = cpos[H.tcol[t]]++;
        ri[b] = H.trow[t];
        cv[b] = tval[t];
      }
      TSVD_TRY(dptr_r.alloc(sp + 1));
      TSVD_TRY(dptr_c.alloc(nc + 1));
      TSVD_TRY(didx_r.alloc(nnz));
      TSVD_TRY(didx_c.alloc(nnz));
      TSVD_TRY(dval_r.alloc(nnz));
      TSVD_TRY(dval_c.alloc(nnz));
      TSVD_CUDA(cudaMemcpyAsync(dptr_r.p, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(dptr_c.p, cp.data(), sizeof(int64_t) * cp.size(), cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(didx_r.p, ci.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(didx_c.p, ri.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(dval_r.p, rv.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(dval_c.p, cv.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice, st));
      sb.rows = sp;
      sb.cols = nc;
      sb.nnz = nnz;
      sb.rowptr = dptr_r.p;
      sb.colidx = didx_r.p;
      sb.rval = dval_r.p;
      sb.colptr = dptr_c.p;
      sb.rowidx = didx_c.p;
      sb.cval = dval_c.p;
      TSVD_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
    } else {
      TSVD_TRY(at.alloc((size_t)nc * sp));
      TSVD_TRY(drow.alloc(nnz));
      TSVD_TRY(dcol.alloc(nnz));
      TSVD_TRY(dval.alloc(nnz));
      TSVD_CUDA(cudaMemsetAsync(at.p, 0, sizeof(__half) * nc * sp, st));
      TSVD_CUDA(cudaMemcpyAsync(drow.p, H.trow.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(dcol.p, H.tcol.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
      TSVD_CUDA(cudaMemcpyAsync(dval.p, tval.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice, st));
      scatter_csr_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(drow.p, dcol.p, dval.p, nnz, sp, at.p);
      TSVD_LAUNCH_CHECK();
      TSVD_CUDA(cudaStreamSynchronize(st));  // tval goes out of scope
    }
    TSVD_CUDA(cudaMemcpyAsync(dcmap.p, H.cmap.data(), sizeof(int32_t) * nc, cudaMemcpyHostToDevice, st));
    FrpcaWork W;
    s1 = frpca_work_alloc(W, 1, nc, sp, l, k);
    if (s1 == TSVD_OK) {
      FrpcaProblem P;
      P.block = 0;
      P.at = at.p;
      P.ncols = nc;
      P.colmap = dcmap.p;
      P.col_base = 0;
      P.b_out = nullptr;
      P.sigma_out = ds.p;
      P.u_out = du.p;
      P.v_out = dv.p;
      P.sparse = fp32 ? &sb : nullptr;
      double ssum = 0;
      s1 = frpca_batch(W, &P, 1, q, seed, nrows, st, &ssum);
    }
    if (s1 == TSVD_OK) {
      cudaMemcpyAsync(hu.data(), du.p, sizeof(float) * hu.size(), cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(hv.data(), dv.p, sizeof(float) * (size_t)nc * k, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(hs.data(), ds.p, sizeof(float) * k, cudaMemcpyDeviceToHost, st);
      cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) s1 = fail(TSVD_ERR_DEVICE, "frpca: %s", cudaGetErrorString(e));
    }
    frpca_work_free(W);
    cudaStreamDestroy(st);
    if (s1 != TSVD_OK) return s1;
  }
  // outputs: descending sigma; U nrows x k, V ncols x k, column-major
  for (int j = 0; j < k; ++j) {
    if (S) S[j] = hs[j] / scale;
    if (U)
      for (int32_t i = 0; i < nrows; ++i) U[(size_t)j * nrows + i] = hu[(size_t)i * k + j];
    if (V) {
      for (int32_t c = 0; c < ncols; ++c) V[(size_t)j * ncols + c] = 0.0;
      for (int32_t c = 0; c < nc; ++c) V[(size_t)j * ncols + H.cmap[c]] = hv[(size_t)c * k + j];
    }
  }
  return TSVD_OK;
}

}  // namespace

extern "C" tsvd_status tsvd_frpca(int32_t nrows, int32_t ncols, int64_t nnz, const int64_t *row_ptr,
                                  const int32_t *col_idx, const double *values, int32_t index_base,
                                  int32_t k, int32_t q, uint64_t seed, double *U, double *S,
                                  double *V) {
  HostBlock H;
  TSVD_TRY(host_block(nrows, ncols, nnz, row_ptr, col_idx, values, index_base, H));
  return frpca_host(nrows, ncols, H, k, q, seed, 0, U, S, V);
}

extern "C" tsvd_status tsvd_frpca_fp32(int32_t nrows, int32_t ncols, int64_t nnz,
                                       const int64_t *row_ptr, const int32_t *col_idx,
                                       const double *values, int32_t index_base, int32_t k,
                                       int32_t q, uint64_t seed, double *U, double *S,
                                       double *V) {
  HostBlock H;
  TSVD_TRY(host_block(nrows, ncols, nnz, row_ptr, col_idx, values, index_base, H));
  return frpca_host(nrows, ncols, H, k, q, seed, 1, U, S, V);
}

extern "C" void frPCA(mat_csr *A, mat **U, mat **S, mat **V, int k, int q) {
  if (!A || !U || !S || !V || !*U || !*S || !*V) {
    fail(TSVD_ERR_INVALID, "frPCA: null argument");
    return;
  }
  const int m = A->nrows, n = A->ncols;
  std::vector<int64_t> rp(m + 1, 0);
  std::vector<int32_t> ci;
  std::vector<double> va;
  ci.reserve(A->nnz > 0 ? A->nnz : 0);
  va.reserve(A->nnz > 0 ? A->nnz : 0);
  for (int i = 0; i < m; ++i) {
    for (int t = A->pointerB[i] - 1; t < A->pointerE[i] - 1; ++t) {
      ci.push_back(A->cols[t] - 1);
      va.push_back(A->values[t]);
    }
    rp[i + 1] = (int64_t)ci.size();
  }
  std::vector<double> u((size_t)m * k), s(k), v((size_t)n * k);
  // the caller's doubles enter as FP32 (SpMM products), the precision the
  // reference's path keeps most closely on this hardware
  tsvd_status st = tsvd_frpca_fp32(m, n, (int64_t)ci.size(), rp.data(), ci.data(), va.data(), 0,
                                   k, q, g_frpca_seed, u.data(), s.data(), v.data());
  mat *Um = *U, *Sm = *S, *Vm = *V;
  if (st != TSVD_OK) {
    std::memset(Um->d, 0, sizeof(double) * (size_t)Um->nrows * Um->ncols);
    std::memset(Sm->d, 0, sizeof(double) * (size_t)Sm->nrows * Sm->ncols);
    std::memset(Vm->d, 0, sizeof(double) * (size_t)Vm->nrows * Vm->ncols);
    return;
  }
  // ascending order, as dsyevd hands them to the reference (frpca.c:298-310)
  for (int j = 0; j < k; ++j) {
    int src = k - 1 - j;
    Sm->d[j] = s[src];
    std::memcpy(Um->d + (size_t)j * Um->nrows, u.data() + (size_t)src * m, sizeof(double) * m);
    std::memcpy(Vm->d + (size_t)j * Vm->nrows, v.data() + (size_t)src * n, sizeof(double) * n);
  }
}

// dense_sub_svd_function (Code/Tree_u_NC.cpp:238-262) over
// truncated_singular_value_decomposition (matrix_vector_functions_intel_mkl.c
// :1259-1300): US = U_d diag(s_d) of the dense rows x cols matrix M
// (column-major, as the reference's mat), sigma = s_d descending. The tree
// merge's own path: compensated Gram, Jacobi refined in fp64, and for more
// than 256 columns the subspace iteration of the wide merge.
extern "C" tsvd_status tsvd_merge_svd(int32_t rows, int32_t cols, const double *M, int32_t d,
                                      double *US, double *sigma) {
  if (rows < 1 || cols < 1 || !M || !US || !sigma) return fail(TSVD_ERR_INVALID, "merge_svd: bad arguments");
  if (d < 1 || d > std::min(rows, cols) || d > kLp || cols > 2048 || (cols > 256 && std::min(rows, 256) < d))
    return fail(TSVD_ERR_INVALID, "merge_svd: d = %d for %d x %d (d <= %d, cols <= 2048)", d, rows,
                cols, kLp);
  std::vector<float> m((size_t)rows * cols);  // row-major fp32, as the merge keeps factors
  for (int32_t j = 0; j < cols; ++j)
    for (int32_t i = 0; i < rows; ++i) m[(size_t)i * cols + j] = (float)M[(size_t)j * rows + i];
  const int sp = (int)round_up(rows, kRowPad);
  DevBuf<float> dout, dsig;
  TSVD_TRY(dout.alloc((size_t)rows * d));
  TSVD_TRY(dsig.alloc(d));
  cudaStream_t st;
  TSVD_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  FrpcaWork W;
  tsvd_status s1 = frpca_work_alloc(W, 1, rows, sp, std::min(kLp, d + 5), d);
  std::vector<float> hu((size_t)rows * d), hs(d);
  if (s1 == TSVD_OK) s1 = merge_matrix(W, m.data(), rows, cols, dout.p, dsig.p, st);
  if (s1 == TSVD_OK) {
    cudaMemcpyAsync(hu.data(), dout.p, sizeof(float) * hu.size(), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hs.data(), dsig.p, sizeof(float) * d, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s1 = fail(TSVD_ERR_DEVICE, "merge_svd: %s", cudaGetErrorString(e));
  }
  frpca_work_free(W);
  cudaStreamDestroy(st);
  if (s1 != TSVD_OK) return s1;
  for (int32_t j = 0; j < d; ++j) {
    sigma[j] = hs[j];
    for (int32_t i = 0; i < rows; ++i) US[(size_t)j * rows + i] = hu[(size_t)i * d + j];
  }
  return TSVD_OK;
}
