// Column blocks of the |S| x N proximity matrix: column compaction, the log
// transform, Frobenius norms for the lazy-update test, half-precision A^T.
//
// Reference: the column partition of Code/Tree_u_NC.cpp:396-432 and the
// per-block transform + norm test of Code/ppr_computation_store_dynamic.h
// (Log_sparse_matrix_entries :2527-2561, _LP :2598-2638,
// _with_norm_computation :2649-2732, _with_norm_computation_LP :2742-2826).
// The reference densifies, sparsifies, copies to COO and then to CSR for
// every dirty block (Tree_u_NC.cpp:91-135); here one pass over the reserve
// vectors writes the transformed block as A^T in half precision (the operand
// of the tensor-core products) and accumulates ||A||_F^2 and ||A - A_old||_F^2.
// Columns (vertices) whose reserve has never been non-zero are left out of
// A^T; the set only grows, so a column keeps its slot across snapshots.
#include "blocks.h"
#include "ppr.h"

namespace tsvd {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Append the block's newly non-zero vertices (vmark == 1) in vertex order;
// colpos (optional) receives each appended vertex's compacted column.
__global__ void __launch_bounds__(1024) colmap_update_kernel(uint8_t *__restrict__ vmark,
                                                             int32_t *__restrict__ colmap,
                                                             int32_t *__restrict__ colpos,
                                                             int32_t *__restrict__ ncols,
                                                             int32_t n, int32_t col_dim,
                                                             int32_t nparts) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t base;
  const int b = blockIdx.x;
  const int32_t v0 = b * col_dim;
  const int32_t v1 = b == nparts - 1 ? n : v0 + col_dim;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) base = ncols[b];
  __syncthreads();
  for (int32_t c0 = v0; c0 < v1; c0 += blockDim.x) {
    int32_t v = c0 + threadIdx.x;
    int f = v < v1 && vmark[v] == 1;
    unsigned m = __ballot_sync(kFull, f);
    if (lane == 0) warp_sums[warp] = __popc(m);
    __syncthreads();
    int32_t before = 0, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < warp) before += warp_sums[w];
      total += warp_sums[w];
    }
    if (f) {
      const int32_t c = base + before + __popc(m & ((1u << lane) - 1u));
      colmap[v0 + c] = v;
      if (colpos) colpos[v] = c;
      vmark[v] = 2;
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) ncols[b] = base;
}

__device__ __forceinline__ float transform(float x, const MaterializeArgs &a) {
  switch (a.transform) {
    case TSVD_TRANSFORM_LOG10_NC:
      return x > a.rmin_f ? log10f(x * a.inv_rmin_f) : 0.f;
    case TSVD_TRANSFORM_LOG10_LP:
      return x != 0.f ? log10f(1.f + x * a.inv_rmin_f) : 0.f;
    default:
      return x > 0.f ? fmaxf(0.f, logf(x * a.n_f)) : 0.f;
  }
}

struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// grid: (column groups, block). One warp per column; each lane owns 4
// consecutive sources per step (8-byte half stores, 16-byte float loads).
__global__ void __launch_bounds__(256) materialize_kernel(MaterializeArgs a) {
  const int b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int32_t nc = a.ncols[b];
  const int32_t nc_old = a.ncols_old[b];
  const int32_t cbase = b * a.col_dim;
  const __half *old = a.at_old[b];
  __half *out = a.at_new[b];
  KahanF k2, kd;
  unsigned long long nnz = 0, stored = 0;
  for (int32_t c = blockIdx.x * 8 + warp; c < nc; c += gridDim.x * 8) {
    const int32_t v = a.colmap[cbase + c];
    const __half *orow = old + (int64_t)c * a.sp;
    __half *nrow = out + (int64_t)c * a.sp;
    const bool has_old = c < nc_old;
    for (int32_t s0 = lane * 4; s0 < a.sp; s0 += 128) {
      const int64_t cell = ppr_cell(v, s0, a.n);
      float4 x = __ldcs(reinterpret_cast<const float4 *>(a.p1 + cell));
      if (a.p2) {
        float4 y = __ldcs(reinterpret_cast<const float4 *>(a.p2 + cell));
        x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
      }
      float xs[4] = {x.x, x.y, x.z, x.w};
      __half2 o01 = make_half2(__float2half(0.f), __float2half(0.f)), o23 = o01;
      if (has_old) {
        uint2 raw = *reinterpret_cast<const uint2 *>(orow + s0);
        o01 = *reinterpret_cast<__half2 *>(&raw.x);
        o23 = *reinterpret_cast<__half2 *>(&raw.y);
      }
      float ov[4] = {__low2float(o01), __high2float(o01), __low2float(o23), __high2float(o23)};
      __half hv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool in = s0 + q < a.nsrc;
        float val = in ? transform(xs[q], a) : 0.f;
        hv[q] = __float2half_rn(val);
        k2.add(val * val);
        float d = val - ov[q];
        kd.add(d * d);
        nnz += val != 0.f;
        stored += in && xs[q] != 0.f;
      }
      __half2 h01 = __halves2half2(hv[0], hv[1]), h23 = __halves2half2(hv[2], hv[3]);
      uint2 raw;
      raw.x = *reinterpret_cast<uint32_t *>(&h01);
      raw.y = *reinterpret_cast<uint32_t *>(&h23);
      *reinterpret_cast<uint2 *>(nrow + s0) = raw;
    }
  }
  // Columns that were in the old block but not in the new one cannot exist:
  // the column set only grows.
  double s2 = (double)k2.s - (double)k2.c, sd = (double)kd.s - (double)kd.c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_down_sync(kFull, s2, o);
    sd += __shfl_down_sync(kFull, sd, o);
    nnz += __shfl_down_sync(kFull, nnz, o);
    stored += __shfl_down_sync(kFull, stored, o);
  }
  __shared__ double r2[8], rd[8];
  __shared__ unsigned long long rn[8], rs[8];
  if (lane == 0) { r2[warp] = s2; rd[warp] = sd; rn[warp] = nnz; rs[warp] = stored; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t2 = 0, td = 0;
    unsigned long long tn = 0, ts = 0;
    for (int w = 0; w < 8; ++w) { t2 += r2[w]; td += rd[w]; tn += rn[w]; ts += rs[w]; }
    atomicAdd(&a.norm2[b], t2);
    atomicAdd(&a.diff2[b], td);
    atomicAdd(&a.nnz[b], tn);
    atomicAdd(&a.stored[b], ts);
  }
}

}  // namespace

tsvd_status colmap_update(uint8_t *vmark, int32_t *colmap, int32_t *colpos, int32_t *ncols,
                          int32_t n, int32_t col_dim, int32_t nparts, cudaStream_t st) {
  colmap_update_kernel<<<nparts, 1024, 0, st>>>(vmark, colmap, colpos, ncols, n, col_dim, nparts);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status materialize_blocks(const MaterializeArgs &a, int nparts, int32_t max_nc,
                               cudaStream_t st) {
  TSVD_CUDA(cudaMemsetAsync(a.norm2, 0, sizeof(double) * nparts, st));
  TSVD_CUDA(cudaMemsetAsync(a.diff2, 0, sizeof(double) * nparts, st));
  TSVD_CUDA(cudaMemsetAsync(a.nnz, 0, sizeof(unsigned long long) * nparts, st));
  TSVD_CUDA(cudaMemsetAsync(a.stored, 0, sizeof(unsigned long long) * nparts, st));
  if (max_nc == 0) return TSVD_OK;
  int gx = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(max_nc, 8),
                                                       ceil_div(8ll * sm_count(), nparts)));
  materialize_kernel<<<dim3(gx, nparts), 256, 0, st>>>(a);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

}  // namespace tsvd
