// Device graph store: per-vertex adjacency rows with slack, appended in
// insertion order and regrown (compacted into a fresh array with 50% slack
// per row) only when some row overflows.
//
// Replaces UGraph::inputDynamicGraph (Code/Graph_dynamic.h:530-605) and
// Graph::inputDirectedDynamicGraph (:119-238): the reference grows every
// touched row by new[] + memcpy each snapshot; here a batch costs one stable
// sort of its entries by vertex plus one scatter, and rows move only on
// regrowth. Row contents and order match the reference row for row.
#include <algorithm>

#include "internal.h"

namespace tsvd {

namespace {

__global__ void count_kernel(const uint32_t *__restrict__ keys, int64_t count,
                             int32_t *__restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[keys[i]], 1);
}

__global__ void overflow_kernel(const int64_t *__restrict__ off,
                                const int32_t *__restrict__ deg,
                                const int32_t *__restrict__ cnt, int32_t n,
                                int32_t *__restrict__ flag) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    if (cnt[v] > 0 && (int64_t)deg[v] + cnt[v] > off[v + 1] - off[v]) {
      *flag = 1;
    }
  }
}

__global__ void new_capacity_kernel(const int32_t *__restrict__ deg,
                                    const int32_t *__restrict__ cnt, int32_t n,
                                    int32_t *__restrict__ cap) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int32_t d = deg[v] + cnt[v];
    cap[v] = d == 0 ? 0 : d + (d >> 1) + 2;
  }
}

// One warp per row: copy the stored entries into the regrown array.
__global__ void copy_rows_kernel(const int64_t *__restrict__ off_old,
                                 const int32_t *__restrict__ nbr_old,
                                 const int64_t *__restrict__ off_new,
                                 int32_t *__restrict__ nbr_new,
                                 const int32_t *__restrict__ deg, int32_t n) {
  const int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int32_t d = deg[v];
    const int32_t *src = nbr_old + off_old[v];
    int32_t *dst = nbr_new + off_new[v];
    for (int32_t j = lane; j < d; j += 32) dst[j] = src[j];
  }
}

__global__ void append_kernel(const uint32_t *__restrict__ skeys,
                              const uint32_t *__restrict__ svals, int64_t count,
                              const int64_t *__restrict__ seg,
                              const int64_t *__restrict__ off,
                              const int32_t *__restrict__ deg,
                              int32_t *__restrict__ nbr) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count;
       q += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = skeys[q];
    int64_t rank = q - seg[v];
    nbr[off[v] + deg[v] + rank] = (int32_t)svals[q];
  }
}

__global__ void add_counts_kernel(int32_t *__restrict__ deg,
                                  const int32_t *__restrict__ cnt, int32_t n) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    deg[v] += cnt[v];
}

int key_bits_for(int32_t n) {
  int b = 1;
  while (b < 32 && (1ll << b) < n) ++b;
  return ((b + 7) / 8) * 8;
}

}  // namespace

void adjacency_free(Adjacency &A) {
  cudaFree(A.off);
  cudaFree(A.deg);
  cudaFree(A.former);
  cudaFree(A.nbr);
  A = Adjacency();
}

tsvd_status adjacency_append(Adjacency &A, const uint32_t *keys, const uint32_t *vals,
                             int64_t count, InsertScratch &scr, cudaStream_t st) {
  const int32_t n = A.n;
  // former degrees are taken for every vertex before the batch is applied
  TSVD_CUDA(cudaMemcpyAsync(A.former, A.deg, sizeof(int32_t) * n,
                            cudaMemcpyDeviceToDevice, st));
  if (count == 0) return TSVD_OK;
  // scratch layout
  size_t need = 0;
  auto take = [&](size_t bytes) {
    size_t at = need;
    need += round_up((int64_t)bytes, 256);
    return at;
  };
  size_t o_k = take(sizeof(uint32_t) * count), o_v = take(sizeof(uint32_t) * count);
  size_t o_ka = take(sizeof(uint32_t) * count), o_va = take(sizeof(uint32_t) * count);
  size_t o_cnt = take(sizeof(int32_t) * n), o_seg = take(sizeof(int64_t) * (n + 1));
  size_t o_flag = take(sizeof(int32_t) * 4);
  size_t o_tmp = take(std::max(sort_tmp_bytes(count), scan_tmp_bytes(n + 1)));
  if (scr.bytes < need) {
    cudaFree(scr.buf);
    scr.buf = nullptr;
    scr.bytes = 0;
    TSVD_CUDA(cudaMalloc(&scr.buf, need));
    scr.bytes = need;
  }
  char *base = (char *)scr.buf;
  uint32_t *k = (uint32_t *)(base + o_k), *v = (uint32_t *)(base + o_v);
  uint32_t *ka = (uint32_t *)(base + o_ka), *va = (uint32_t *)(base + o_va);
  int32_t *cnt = (int32_t *)(base + o_cnt);
  int64_t *seg = (int64_t *)(base + o_seg);
  int32_t *flag = (int32_t *)(base + o_flag);
  void *tmp = base + o_tmp;

  TSVD_CUDA(cudaMemcpyAsync(k, keys, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, st));
  TSVD_CUDA(cudaMemcpyAsync(v, vals, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, st));
  bool in_alt = false;
  TSVD_TRY(stable_sort_pairs(k, v, ka, va, count, key_bits_for(n), tmp, st, &in_alt));
  uint32_t *sk = in_alt ? ka : k, *sv = in_alt ? va : v;

  TSVD_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n, st));
  TSVD_CUDA(cudaMemsetAsync(flag, 0, sizeof(int32_t), st));
  int g = grid_for(count, 256);
  count_kernel<<<g, 256, 0, st>>>(sk, count, cnt);
  TSVD_LAUNCH_CHECK();
  int gn = grid_for(n, 256);
  overflow_kernel<<<gn, 256, 0, st>>>(A.off, A.deg, cnt, n, flag);
  TSVD_LAUNCH_CHECK();
  int32_t h_flag = 0;
  TSVD_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  if (h_flag) {
    // Regrow: new capacities, new row starts, copy the stored rows.
    int32_t *cap = (int32_t *)seg;  // reuse as int32 scratch before the scan below
    new_capacity_kernel<<<gn, 256, 0, st>>>(A.deg, cnt, n, cap);
    TSVD_LAUNCH_CHECK();
    int64_t *off_new = nullptr;
    TSVD_CUDA(cudaMalloc(&off_new, sizeof(int64_t) * (n + 1)));
    tsvd_status s1 = scan_i32_to_i64(cap, off_new, n, tmp, st);
    if (s1 != TSVD_OK) { cudaFree(off_new); return s1; }
    int64_t total = 0;
    TSVD_CUDA(cudaMemcpyAsync(&total, off_new + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
    int32_t *nbr_new = nullptr;
    cudaError_t e = cudaMalloc(&nbr_new, sizeof(int32_t) * std::max<int64_t>(total, 1));
    if (e != cudaSuccess) {
      cudaFree(off_new);
      return fail(TSVD_ERR_OOM, "adjacency regrow: %lld entries", (long long)total);
    }
    if (A.nbr) {
      copy_rows_kernel<<<grid_for((int64_t)n * 32, 256), 256, 0, st>>>(A.off, A.nbr, off_new,
                                                                         nbr_new, A.deg, n);
      TSVD_LAUNCH_CHECK();
    }
    TSVD_CUDA(cudaStreamSynchronize(st));
    cudaFree(A.nbr);
    cudaFree(A.off);
    A.nbr = nbr_new;
    A.off = off_new;
    A.cap_total = total;
  }
  TSVD_TRY(scan_i32_to_i64(cnt, seg, n, tmp, st));
  append_kernel<<<g, 256, 0, st>>>(sk, sv, count, seg, A.off, A.deg, A.nbr);
  TSVD_LAUNCH_CHECK();
  add_counts_kernel<<<gn, 256, 0, st>>>(A.deg, cnt, n);
  TSVD_LAUNCH_CHECK();
  A.m += count;
  return TSVD_OK;
}

}  // namespace tsvd
