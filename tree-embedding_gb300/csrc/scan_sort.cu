// Device prefix sums and a stable LSD radix sort of (key, value) pairs.
//
// The sort gives the graph-store insert its order guarantee: entries of one
// vertex keep the order in which the edge file listed them (the reference
// appends in file order, Code/Graph_dynamic.h:590-596).
#include <cstdio>

#include "internal.h"

namespace tsvd {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ int64_t block_exclusive_scan(int64_t v, int64_t *warp_sums, int64_t *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int64_t before = warp > 0 ? warp_sums[warp - 1] : 0;
  if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
  return before + x - v;  // exclusive
}

template <typename T>
__global__ void tile_reduce_kernel(const T *__restrict__ in, int64_t n,
                                   int64_t *__restrict__ sums) {
  __shared__ int64_t ws[32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += (int64_t)in[base + i];
  int64_t tot;
  block_exclusive_scan<T>(s, ws, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void tile_scan_kernel(const T *__restrict__ in, int64_t n,
                                 const int64_t *__restrict__ tile_off,
                                 int64_t *__restrict__ out) {
  __shared__ int64_t ws[32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? (int64_t)in[base + i] : 0;
    s += v[i];
  }
  int64_t tot;
  int64_t ex = block_exclusive_scan<T>(s, ws, &tot) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  // out[n] = grand total, written by the tile holding element n-1.
  if (base < n && base + kScanItems >= n) out[n] = ex;
}

__global__ void set_zero_total(int64_t *out) { out[0] = 0; }

template <typename T>
tsvd_status scan_impl(const T *in, int64_t *out, int64_t n, char *tmp, cudaStream_t st) {
  if (n == 0) {
    set_zero_total<<<1, 1, 0, st>>>(out);
    TSVD_LAUNCH_CHECK();
    return TSVD_OK;
  }
  int64_t tiles = ceil_div(n, kScanTile);
  if (tiles == 1) {
    tile_scan_kernel<T><<<1, kScanThreads, 0, st>>>(in, n, nullptr, out);
    TSVD_LAUNCH_CHECK();
    return TSVD_OK;
  }
  int64_t *sums = (int64_t *)tmp;
  int64_t *sums_scan = sums + round_up(tiles, 32);
  char *rest = (char *)(sums_scan + round_up(tiles + 1, 32));
  tile_reduce_kernel<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums);
  TSVD_LAUNCH_CHECK();
  TSVD_TRY(scan_impl<int64_t>(sums, sums_scan, tiles, rest, st));
  tile_scan_kernel<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums_scan, out);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

// ------------------------------------------------------------ radix sort
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 16;
constexpr int kSortTile = kSortThreads * kSortRounds;
constexpr int kSortWarps = kSortThreads / 32;

__global__ void radix_hist_kernel(const uint32_t *__restrict__ keys, int64_t n,
                                  int shift, int64_t ntiles,
                                  int32_t *__restrict__ hist) {
  __shared__ int32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
    int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xff], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void radix_scatter_kernel(const uint32_t *__restrict__ keys,
                                     const uint32_t *__restrict__ vals, int64_t n,
                                     int shift, int64_t ntiles,
                                     const int64_t *__restrict__ offs,
                                     uint32_t *__restrict__ keys_out,
                                     uint32_t *__restrict__ vals_out) {
  __shared__ int64_t base[256];
  __shared__ int32_t running[256];
  __shared__ int32_t wcnt[kSortWarps][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base[tid] = offs[(int64_t)tid * ntiles + blockIdx.x];
  running[tid] = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) wcnt[w][tid] = 0;
  __syncthreads();
  const unsigned lt_mask = (1u << lane) - 1u;
  int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
    int64_t i = tile0 + (int64_t)r * kSortThreads + tid;
    bool valid = i < n;
    uint32_t key = valid ? keys[i] : 0u;
    uint32_t val = valid ? vals[i] : 0u;
    int digit = valid ? (int)((key >> shift) & 0xff) : 256;
    unsigned peers = __match_any_sync(0xffffffffu, digit);
    int rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    {  // counts -> exclusive offsets across warps, then advance the running count
      int32_t s = running[tid];
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        int32_t c = wcnt[w][tid];
        wcnt[w][tid] = s;
        s += c;
      }
      running[tid] = s;
    }
    __syncthreads();
    if (valid) {
      int64_t dst = base[digit] + wcnt[warp][digit] + rank;
      keys_out[dst] = key;
      vals_out[dst] = val;
    }
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) wcnt[w][tid] = 0;
    __syncthreads();
  }
}

}  // namespace

size_t scan_tmp_bytes(int64_t n) {
  size_t total = 0;
  int64_t m = n;
  while (m > kScanTile) {
    int64_t tiles = ceil_div(m, kScanTile);
    total += (size_t)(round_up(tiles, 32) + round_up(tiles + 1, 32)) * sizeof(int64_t);
    m = tiles;
  }
  return total + 256;
}

tsvd_status scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, void *tmp,
                            cudaStream_t st) {
  return scan_impl<int32_t>(in, out, n, (char *)tmp, st);
}

size_t sort_tmp_bytes(int64_t n) {
  int64_t ntiles = ceil_div(std::max<int64_t>(n, 1), kSortTile);
  size_t hist = (size_t)256 * ntiles;
  return round_up(hist * sizeof(int32_t), 256) + round_up((hist + 1) * sizeof(int64_t), 256) +
         scan_tmp_bytes((int64_t)hist);
}

tsvd_status stable_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                              uint32_t *vals_alt, int64_t n, int key_bits, void *tmp,
                              cudaStream_t st, bool *result_in_alt) {
  *result_in_alt = false;
  if (n <= 1) return TSVD_OK;
  int64_t ntiles = ceil_div(n, kSortTile);
  size_t hist_n = (size_t)256 * ntiles;
  char *p = (char *)tmp;
  int32_t *hist = (int32_t *)p;
  p += round_up(hist_n * sizeof(int32_t), 256);
  int64_t *offs = (int64_t *)p;
  p += round_up((hist_n + 1) * sizeof(int64_t), 256);
  uint32_t *ka = keys, *va = vals, *kb = keys_alt, *vb = vals_alt;
  for (int shift = 0; shift < key_bits; shift += 8) {
    radix_hist_kernel<<<(unsigned)ntiles, 256, 0, st>>>(ka, n, shift, ntiles, hist);
    TSVD_LAUNCH_CHECK();
    TSVD_TRY(scan_i32_to_i64(hist, offs, (int64_t)hist_n, p, st));
    radix_scatter_kernel<<<(unsigned)ntiles, kSortThreads, 0, st>>>(ka, va, n, shift, ntiles,
                                                                  offs, kb, vb);
    TSVD_LAUNCH_CHECK();
    std::swap(ka, kb);
    std::swap(va, vb);
    *result_in_alt = !*result_in_alt;
  }
  return TSVD_OK;
}

}  // namespace tsvd
