// The plain GPU form: cell-by-cell forward push in fp64 arithmetic, FP32
// CSR/CSC blocks and FP32 SpMM frPCA products (see plain.h).
//
// Reference: the per-source push and refresh of
// Code/ppr_computation_store_dynamic.h (nodegree_DenseDynamicForwardPush
// :1394-1498, nodegree_DenseDirectedDynamicForwardPush :2945-3030,
// ...Transpose :3356-3437; refresh :2035-2121, :3811-3898, :4133-4228) and
// the CSR products of frPCA (csr_matrix_{,transpose_}matrix_mult,
// Code/matrix_vector_functions_intel_mkl_ext.c:364-398, over the CSR the
// drivers build per block, Code/Tree_u_NC.cpp:91-135).
#include <algorithm>
#include <cmath>

#include "plain.h"

namespace tsvd {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void mark_cell(uint32_t *bits, int64_t cell) {
  atomicOr(bits + (cell >> 5), 1u << (cell & 31));
}

struct PlainArgs {
  const int2 *front;
  const unsigned long long *front_count;  // may exceed cap: entries beyond it were not stored
  float *r, *p;
  const int64_t *off;
  const int32_t *deg, *nbr, *former;
  int32_t n, nsrc;
  uint32_t *cbits;
  double alpha, one_minus_alpha;
  float rmax_f;
  int undirected, intdiv;
  uint8_t *vmark;
  unsigned long long *stats;
  int2 *next;
  unsigned long long *next_count;
  int64_t cap;
  int64_t nwords;
  const int32_t *upd;
  const int32_t *nupd;
};

// One warp per frontier cell (v, s): lane 0 takes the residue, adds
// alpha r to the reserve and computes (1 - alpha) r / deg(v) in fp64; the
// lanes then add it to r(u, s) of every neighbour u with one scalar atomic
// each and mark the touched cells.
__global__ void __launch_bounds__(256) plain_push_kernel(PlainArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nitems = (int64_t)min(*a.front_count, (unsigned long long)a.cap);
  unsigned long long pushes = 0, upd = 0;
  for (int64_t i = gw; i < nitems; i += nw) {
    const int2 it = a.front[i];
    const int32_t v = it.x, s = it.y;
    const int64_t cell = ppr_cell(v, s, a.n);
    const int32_t d = a.deg[v];
    float w = 0.f;
    int go = 0;
    if (lane == 0) {
      const float x0 = a.r[cell];
      if (x0 > a.rmax_f) {
        if (d == 0) {
          // isolated source of an undirected graph: pi = alpha r, r kept
          // (ppr:1433-1441); directed dangling vertices are skipped
          if (a.undirected) {
            a.p[cell] = (float)(a.alpha * (double)x0);
            if (a.vmark[v] == 0) a.vmark[v] = 1;
          }
        } else {
          const float x = atomicExch(a.r + cell, 0.0f);
          a.p[cell] = (float)((double)a.p[cell] + a.alpha * (double)x);
          w = (float)(a.one_minus_alpha * (double)x / (double)d);
          if (a.vmark[v] == 0) a.vmark[v] = 1;
          go = 1;
          pushes += 1;
          upd += (unsigned long long)d;
        }
      }
    }
    go = __shfl_sync(kFull, go, 0);
    if (!go) continue;
    w = __shfl_sync(kFull, w, 0);
    const int32_t *nb = a.nbr + a.off[v];
    for (int32_t j = lane; j < d; j += 32) {
      const int64_t c = ppr_cell(__ldg(nb + j), s, a.n);
      atomicAdd(a.r + c, w);
      mark_cell(a.cbits, c);
    }
  }
  if (lane == 0 && (pushes || upd)) {
    atomicAdd(a.stats + 0, pushes);
    atomicAdd(a.stats + 1, upd);
  }
}

// One thread per bitset word (32 sources of one vertex): each touched cell
// with a residue above rmax and a non-zero degree goes to the next frontier;
// cells that do not fit (the list is bounded) stay marked for a later round.
__global__ void __launch_bounds__(256) plain_collect_kernel(PlainArgs a) {
  for (int64_t wi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; wi < a.nwords;
       wi += (int64_t)gridDim.x * blockDim.x) {
    uint32_t bits = a.cbits[wi];
    if (!bits) continue;
    uint32_t keep = 0;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int64_t cell = wi * 32 + b;
      const int64_t run = cell >> 6;
      const int32_t c = (int32_t)(run / a.n);
      const int32_t v = (int32_t)(run - (int64_t)c * a.n);
      const int32_t s = c * 64 + (int32_t)(cell & 63);
      if (s >= a.nsrc || a.deg[v] == 0 || !(a.r[cell] > a.rmax_f)) continue;
      const unsigned long long slot = atomicAdd(a.next_count, 1ull);
      if (slot < (unsigned long long)a.cap)
        a.next[slot] = make_int2(v, s);
      else
        keep |= 1u << b;
    }
    a.cbits[wi] = keep;
  }
}

// Dynamic refresh, one thread per (updated vertex u, source s): for every
// new slot j >= 1 of u (the reference skips j == 0, ppr:2086-2093), in fp64,
//   p_u *= (j+1)/j ; r_u -= p_u/(j+1)/alpha ; r_w += (1-alpha) p_u/(j+1)/alpha.
__global__ void __launch_bounds__(256) plain_refresh_kernel(PlainArgs a) {
  const int64_t total = (int64_t)(*a.nupd) * a.nsrc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = a.upd[i / a.nsrc];
    const int32_t s = (int32_t)(i % a.nsrc);
    const int32_t j0 = a.former[u], j1 = a.deg[u];
    const int64_t cu = ppr_cell(u, s, a.n);
    const int32_t *nb = a.nbr + a.off[u];
    double pu = (double)a.p[cu], rdelta = 0.0;
    bool any = false;
    for (int32_t j = max(j0, 1); j < j1; ++j) {
      any = true;
      const double f = a.intdiv ? (double)((j + 1) / j) : (double)(j + 1) / (double)j;
      pu *= f;
      const double q = pu / (double)(j + 1) / a.alpha;
      rdelta -= q;
      const int64_t cw = ppr_cell(__ldg(nb + j), s, a.n);
      atomicAdd(a.r + cw, (float)(a.one_minus_alpha * q));
      mark_cell(a.cbits, cw);
    }
    if (any) {
      a.p[cu] = (float)pu;
      atomicAdd(a.r + cu, (float)rdelta);
    }
    if (any || (!a.intdiv && j0 == 0 && j1 > 0)) mark_cell(a.cbits, cu);
  }
}

// r = e_s for every source; the first frontier is the sources themselves
// (an isolated source of an undirected graph is pushed once too: its
// reserve becomes alpha, as in the reference).
__global__ void plain_seed_kernel(const int32_t *__restrict__ sources, int32_t nsrc,
                                  float *__restrict__ r, int32_t n, int2 *__restrict__ front,
                                  unsigned long long *__restrict__ count) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nsrc; k += gridDim.x * blockDim.x) {
    r[ppr_cell(sources[k], k, n)] = 1.0f;
    front[k] = make_int2(sources[k], k);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = (unsigned long long)nsrc;
}

__global__ void plain_zero_kernel(float4 *__restrict__ x, int64_t n4) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void plain_list_updated_kernel(const int32_t *__restrict__ deg,
                                          const int32_t *__restrict__ former, int32_t n,
                                          int32_t *__restrict__ out, int32_t *__restrict__ count) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    if (deg[v] > former[v]) out[atomicAdd(count, 1)] = v;
}

float largest_float_not_above(double x) {
  float f = (float)x;
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}

// ------------------------------------------------------------ block build
__device__ __forceinline__ float block_transform(float x, const BlockSource &a) {
  switch (a.transform) {
    case TSVD_TRANSFORM_LOG10_NC:
      return x > a.rmin_f ? log10f(x * a.inv_rmin_f) : 0.f;
    case TSVD_TRANSFORM_LOG10_LP:
      return x != 0.f ? log10f(1.f + x * a.inv_rmin_f) : 0.f;
    default:
      return x > 0.f ? fmaxf(0.f, logf(x * a.n_f)) : 0.f;
  }
}

// The four values of sources s0..s0+3 of compacted column c (vertex v): the
// stored half-precision A^T, or the transform of the reserve (the same fp32
// expression the block materialization rounds to half precision).
__device__ __forceinline__ void cell4(const BlockSource &a, int64_t c, int32_t v, int32_t s0,
                                      float *out) {
  if (a.at) {
    const uint2 raw = *reinterpret_cast<const uint2 *>(a.at + c * a.sp + s0);
    const __half2 h01 = *reinterpret_cast<const __half2 *>(&raw.x);
    const __half2 h23 = *reinterpret_cast<const __half2 *>(&raw.y);
    out[0] = __low2float(h01);
    out[1] = __high2float(h01);
    out[2] = __low2float(h23);
    out[3] = __high2float(h23);
    return;
  }
  const int64_t cell = ppr_cell(v, s0, a.n);
  float4 x = __ldcs(reinterpret_cast<const float4 *>(a.p1 + cell));
  if (a.p2) {
    const float4 y = __ldcs(reinterpret_cast<const float4 *>(a.p2 + cell));
    x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
  }
  const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) out[q] = s0 + q < a.nsrc ? block_transform(xs[q], a) : 0.f;
}

// pass 0: count the non-zeros of every column; pass 1: write them (CSC, rows
// ascending), with each entry's column and row for the CSR transpose.
template <int PASS>
__global__ void __launch_bounds__(256) csc_kernel(BlockSource a, int32_t *cnt,
                                                  const int64_t *colptr, int32_t *rowidx,
                                                  float *cval, int32_t *ecol, uint32_t *keys,
                                                  uint32_t *vals) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = gw; c < a.ncols; c += nw) {
    const int32_t v = a.at ? 0 : a.colmap[c];
    int64_t pos = PASS ? colptr[c] : 0;
    int32_t total = 0;
    for (int32_t s0 = lane * 4; s0 < a.sp; s0 += 128) {
      float x[4];
      cell4(a, c, v, s0, x);
      const int mine = (x[0] != 0.f) + (x[1] != 0.f) + (x[2] != 0.f) + (x[3] != 0.f);
      int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
      }
      const int step_total = __shfl_sync(kFull, incl, 31);
      if (PASS) {
        int64_t at = pos + incl - mine;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (x[q] != 0.f) {
            rowidx[at] = s0 + q;
            cval[at] = x[q];
            ecol[at] = (int32_t)c;
            keys[at] = (uint32_t)(s0 + q);
            vals[at] = (uint32_t)at;
            ++at;
          }
        pos += step_total;
      }
      total += step_total;
    }
    if (!PASS && lane == 0) cnt[c] = total;
  }
}

__global__ void row_count_kernel(const uint32_t *__restrict__ keys, int64_t nnz,
                                 int32_t *__restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + keys[i], 1);
}

__global__ void csr_gather_kernel(const uint32_t *__restrict__ order, int64_t nnz,
                                  const int32_t *__restrict__ ecol, const float *__restrict__ cval,
                                  int32_t *__restrict__ colidx, float *__restrict__ rval) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t e = order[i];
    colidx[i] = ecol[e];
    rval[i] = cval[e];
  }
}

// --------------------------------------------------------------- SpMM
struct SpmmArgs {
  const int64_t *const *ptr;
  const int32_t *const *idx;
  const float *const *val;
  const int32_t *rows_out;
  const __half *const *hi, *const *lo;
  float *const *y;
  float scale;
};

// One warp per output row: lane l accumulates half2 columns l, l + 32 and
// (lanes 0-7) l + 64 of the kLp = 144 wide row; the row's entries are read
// 32 at a time by the lanes and broadcast.
__global__ void __launch_bounds__(256) spmm_kernel(SpmmArgs a) {
  const int prob = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int32_t rows = a.rows_out[prob];
  const int64_t *ptr = a.ptr[prob];
  const int32_t *idx = a.idx[prob];
  const float *val = a.val[prob];
  const __half2 *hi = reinterpret_cast<const __half2 *>(a.hi[prob]);
  const __half2 *lo = a.lo ? reinterpret_cast<const __half2 *>(a.lo[prob]) : nullptr;
  float2 *y = reinterpret_cast<float2 *>(a.y[prob]);
  constexpr int H = kLp / 2;  // 72 half2 per row
  const bool third = lane + 64 < H;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < rows; r += nw) {
    float2 acc0 = make_float2(0.f, 0.f), acc1 = acc0, acc2 = acc0;
    const int64_t t0 = ptr[r], t1 = ptr[r + 1];
    for (int64_t tb = t0; tb < t1; tb += 32) {
      const int cnt = (int)(t1 - tb < 32 ? t1 - tb : 32);
      const int32_t my_c = lane < cnt ? idx[tb + lane] : 0;
      const float my_v = lane < cnt ? val[tb + lane] : 0.f;
      for (int k = 0; k < cnt; ++k) {
        const int64_t row = (int64_t)__shfl_sync(kFull, my_c, k) * H;
        const float v = __shfl_sync(kFull, my_v, k);
        float2 x0 = __half22float2(hi[row + lane]);
        float2 x1 = __half22float2(hi[row + lane + 32]);
        float2 x2 = third ? __half22float2(hi[row + lane + 64]) : make_float2(0.f, 0.f);
        if (lo) {
          const float2 l0 = __half22float2(lo[row + lane]);
          const float2 l1 = __half22float2(lo[row + lane + 32]);
          x0.x += l0.x; x0.y += l0.y; x1.x += l1.x; x1.y += l1.y;
          if (third) {
            const float2 l2 = __half22float2(lo[row + lane + 64]);
            x2.x += l2.x; x2.y += l2.y;
          }
        }
        acc0.x = fmaf(v, x0.x, acc0.x); acc0.y = fmaf(v, x0.y, acc0.y);
        acc1.x = fmaf(v, x1.x, acc1.x); acc1.y = fmaf(v, x1.y, acc1.y);
        acc2.x = fmaf(v, x2.x, acc2.x); acc2.y = fmaf(v, x2.y, acc2.y);
      }
    }
    float2 *out = y + r * H;
    out[lane] = make_float2(acc0.x * a.scale, acc0.y * a.scale);
    out[lane + 32] = make_float2(acc1.x * a.scale, acc1.y * a.scale);
    if (third) out[lane + 64] = make_float2(acc2.x * a.scale, acc2.y * a.scale);
  }
}

}  // namespace

// ------------------------------------------------------------------ push
tsvd_status plain_alloc(PlainPpr &Q, int32_t n, int32_t sp, int64_t cap) {
  Q.nwords = ceil_div((int64_t)n * sp, 32);
  TSVD_CUDA(cudaMalloc(&Q.cbits, Q.nwords * sizeof(uint32_t)));
  TSVD_CUDA(cudaMemset(Q.cbits, 0, Q.nwords * sizeof(uint32_t)));
  // bounded frontier: cells that do not fit wait in the bitset for a later round
  Q.cap = std::min<int64_t>((int64_t)n * sp, cap > 0 ? cap : (int64_t)1 << 26);
  for (int i = 0; i < 2; ++i) TSVD_CUDA(cudaMalloc(&Q.front[i], Q.cap * sizeof(int2)));
  TSVD_CUDA(cudaMalloc(&Q.counters, 8 * sizeof(unsigned long long)));
  TSVD_CUDA(cudaMemset(Q.counters, 0, 8 * sizeof(unsigned long long)));
  TSVD_CUDA(cudaMallocHost(&Q.host_counters, 8 * sizeof(unsigned long long)));
  TSVD_CUDA(cudaMalloc(&Q.stats, 2 * sizeof(unsigned long long)));
  for (auto &e : Q.kev) TSVD_CUDA(cudaEventCreate(&e));
  return TSVD_OK;
}

void plain_free(PlainPpr &Q) {
  cudaFree(Q.cbits);
  cudaFree(Q.front[0]);
  cudaFree(Q.front[1]);
  cudaFree(Q.counters);
  cudaFreeHost(Q.host_counters);
  cudaFree(Q.stats);
  for (auto &e : Q.kev)
    if (e) cudaEventDestroy(e);
  Q = PlainPpr();
}

static PlainArgs plain_args(PlainPpr &Q, PprState &P, const Adjacency &A, const PprParams &prm) {
  PlainArgs a{};
  a.r = P.r;
  a.p = P.p;
  a.off = A.off;
  a.deg = A.deg;
  a.nbr = A.nbr;
  a.former = A.former;
  a.n = P.n;
  a.nsrc = P.nsrc;
  a.cbits = Q.cbits;
  a.alpha = prm.alpha;
  a.one_minus_alpha = 1.0 - prm.alpha;
  a.rmax_f = largest_float_not_above(prm.rmax);
  a.undirected = prm.undirected;
  a.intdiv = prm.intdiv;
  a.cap = Q.cap;
  a.nwords = Q.nwords;
  return a;
}

tsvd_status plain_refresh(PlainPpr &Q, PprState &P, const Adjacency &A,
                          const int32_t *sources_dev, bool from_scratch, const PprParams &prm,
                          cudaStream_t st) {
  if (from_scratch) {
    const int64_t cells = (int64_t)P.n * P.sp;
    plain_zero_kernel<<<grid_for(cells / 4, 256, 8), 256, 0, st>>>(reinterpret_cast<float4 *>(P.r),
                                                                   cells / 4);
    TSVD_LAUNCH_CHECK();
    plain_zero_kernel<<<grid_for(cells / 4, 256, 8), 256, 0, st>>>(reinterpret_cast<float4 *>(P.p),
                                                                   cells / 4);
    TSVD_LAUNCH_CHECK();
    TSVD_CUDA(cudaMemsetAsync(Q.cbits, 0, Q.nwords * sizeof(uint32_t), st));
    if ((int64_t)P.nsrc > Q.cap)
      return fail(TSVD_ERR_INVALID, "plain push: a frontier of %lld entries holds fewer than the "
                  "%d sources", (long long)Q.cap, P.nsrc);
    plain_seed_kernel<<<grid_for(P.nsrc, 256), 256, 0, st>>>(sources_dev, P.nsrc, P.r, P.n,
                                                             Q.front[0], Q.counters + 0);
    TSVD_LAUNCH_CHECK();
    Q.primed = true;
  } else {
    TSVD_CUDA(cudaMemsetAsync(P.counters + 5, 0, sizeof(int32_t), st));
    plain_list_updated_kernel<<<grid_for(A.n, 256), 256, 0, st>>>(A.deg, A.former, A.n, P.upd,
                                                                   P.counters + 5);
    TSVD_LAUNCH_CHECK();
    PlainArgs a = plain_args(Q, P, A, prm);
    a.upd = P.upd;
    a.nupd = P.counters + 5;
    plain_refresh_kernel<<<grid_for((int64_t)A.n * 8, 256, 16), 256, 0, st>>>(a);
    TSVD_LAUNCH_CHECK();
  }
  Q.seeded = true;
  return TSVD_OK;
}

tsvd_status plain_push(PlainPpr &Q, PprState &P, const Adjacency &A, const PprParams &prm,
                       uint8_t *vmark, cudaStream_t st, PushStats *out) {
  if (!Q.seeded) return fail(TSVD_ERR_STATE, "plain push before refresh");
  PlainArgs a = plain_args(Q, P, A, prm);
  a.vmark = vmark;
  a.stats = Q.stats;
  TSVD_CUDA(cudaMemsetAsync(Q.stats, 0, 2 * sizeof(unsigned long long), st));
  const int gcol = grid_for(Q.nwords, 256, 8);
  const int gpush = grid_for((int64_t)1 << 30, 256, 8);
  Q.cur = 0;
  if (!Q.primed) {
    // first frontier: every cell the refresh marked
    TSVD_CUDA(cudaMemsetAsync(Q.counters, 0, 8 * sizeof(unsigned long long), st));
    a.next = Q.front[0];
    a.next_count = Q.counters + 0;
    plain_collect_kernel<<<gcol, 256, 0, st>>>(a);
    TSVD_LAUNCH_CHECK();
  }
  Q.primed = false;
  int64_t rounds = 0;
  double kernel_ms = 0;
  const int per_check = 4;
  for (;;) {
    for (int k = 0; k < per_check; ++k) {
      const int cur = Q.cur, nxt = 1 - Q.cur;
      a.front = Q.front[cur];
      a.front_count = Q.counters + cur;
      a.next = Q.front[nxt];
      a.next_count = Q.counters + nxt;
      TSVD_CUDA(cudaMemsetAsync(Q.counters + nxt, 0, sizeof(unsigned long long), st));
      TSVD_CUDA(cudaEventRecord(Q.kev[2 * k], st));
      plain_push_kernel<<<gpush, 256, 0, st>>>(a);
      TSVD_LAUNCH_CHECK();
      TSVD_CUDA(cudaEventRecord(Q.kev[2 * k + 1], st));
      plain_collect_kernel<<<gcol, 256, 0, st>>>(a);
      TSVD_LAUNCH_CHECK();
      Q.cur = nxt;
      ++rounds;
    }
    TSVD_CUDA(cudaMemcpyAsync(Q.host_counters, Q.counters, 8 * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, st));
    TSVD_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < per_check; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, Q.kev[2 * k], Q.kev[2 * k + 1]) == cudaSuccess) kernel_ms += ms;
    }
    if (Q.host_counters[Q.cur] == 0) break;
    if (rounds >= prm.max_rounds)
      return fail(TSVD_ERR_TIMEOUT, "plain push: %lld rounds without convergence",
                  (long long)rounds);
  }
  unsigned long long hs[2];
  TSVD_CUDA(cudaMemcpyAsync(hs, Q.stats, sizeof hs, cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  if (out) {
    out->rounds = rounds;
    out->pushes = (int64_t)hs[0];
    out->edge_updates = (int64_t)hs[1];
    out->items = (int64_t)hs[0];
    out->item_edges = (int64_t)hs[1];
    out->kernel_ms = kernel_ms;
  }
  Q.seeded = false;
  return TSVD_OK;
}

// ----------------------------------------------------------- block build
void plain_block_free(PlainBlockWork &W) {
  cudaFree(W.blk.rowptr); cudaFree(W.blk.colidx); cudaFree(W.blk.rval);
  cudaFree(W.blk.colptr); cudaFree(W.blk.rowidx); cudaFree(W.blk.cval);
  cudaFree(W.cnt); cudaFree(W.keys); cudaFree(W.vals); cudaFree(W.keys_alt);
  cudaFree(W.vals_alt); cudaFree(W.ecol); cudaFree(W.tmp);
  W = PlainBlockWork();
}

static tsvd_status block_reserve(PlainBlockWork &W, int64_t nnz, int32_t cols, int32_t rows) {
  if (nnz > W.nnz_cap) {
    const int64_t cap = std::max<int64_t>(nnz + nnz / 8, 1 << 16);
    cudaFree(W.blk.colidx); cudaFree(W.blk.rval); cudaFree(W.blk.rowidx); cudaFree(W.blk.cval);
    cudaFree(W.keys); cudaFree(W.vals); cudaFree(W.keys_alt); cudaFree(W.vals_alt);
    cudaFree(W.ecol);
    W.blk.colidx = W.blk.rowidx = W.ecol = nullptr;
    W.blk.rval = W.blk.cval = nullptr;
    W.keys = W.vals = W.keys_alt = W.vals_alt = nullptr;
    W.nnz_cap = 0;
    TSVD_CUDA(cudaMalloc(&W.blk.colidx, cap * sizeof(int32_t)));
    TSVD_CUDA(cudaMalloc(&W.blk.rval, cap * sizeof(float)));
    TSVD_CUDA(cudaMalloc(&W.blk.rowidx, cap * sizeof(int32_t)));
    TSVD_CUDA(cudaMalloc(&W.blk.cval, cap * sizeof(float)));
    TSVD_CUDA(cudaMalloc(&W.keys, cap * sizeof(uint32_t)));
    TSVD_CUDA(cudaMalloc(&W.vals, cap * sizeof(uint32_t)));
    TSVD_CUDA(cudaMalloc(&W.keys_alt, cap * sizeof(uint32_t)));
    TSVD_CUDA(cudaMalloc(&W.vals_alt, cap * sizeof(uint32_t)));
    TSVD_CUDA(cudaMalloc(&W.ecol, cap * sizeof(int32_t)));
    W.nnz_cap = cap;
  }
  const int64_t maxdim = std::max<int64_t>(cols, rows);
  if (cols > W.cols_cap || rows > W.rows_cap) {
    cudaFree(W.blk.colptr); cudaFree(W.blk.rowptr); cudaFree(W.cnt);
    W.blk.colptr = W.blk.rowptr = nullptr;
    W.cnt = nullptr;
    W.cols_cap = std::max<int64_t>(cols, W.cols_cap);
    W.rows_cap = std::max<int64_t>(rows, W.rows_cap);
    TSVD_CUDA(cudaMalloc(&W.blk.colptr, (W.cols_cap + 1) * sizeof(int64_t)));
    TSVD_CUDA(cudaMalloc(&W.blk.rowptr, (W.rows_cap + 1) * sizeof(int64_t)));
    TSVD_CUDA(cudaMalloc(&W.cnt, (std::max(W.cols_cap, W.rows_cap) + 1) * sizeof(int32_t)));
  }
  const size_t need = std::max(std::max(scan_tmp_bytes(maxdim + 1), sort_tmp_bytes(W.nnz_cap)),
                               (size_t)256);
  if (need > W.tmp_bytes) {
    cudaFree(W.tmp);
    W.tmp = nullptr;
    W.tmp_bytes = 0;
    TSVD_CUDA(cudaMalloc(&W.tmp, need));
    W.tmp_bytes = need;
  }
  return TSVD_OK;
}

tsvd_status plain_block_build(PlainBlockWork &W, const BlockSource &src, int64_t nnz_hint,
                              cudaStream_t st) {
  const int32_t cols = src.ncols, rows = src.sp;
  TSVD_TRY(block_reserve(W, std::max<int64_t>(nnz_hint, 1), std::max(cols, 1), rows));
  SparseBlock &B = W.blk;
  B.rows = rows;
  B.cols = cols;
  const int g = grid_for((int64_t)std::max(cols, 1) * 32, 256, 8);
  if (cols > 0) {
    csc_kernel<0><<<g, 256, 0, st>>>(src, W.cnt, nullptr, nullptr, nullptr, nullptr, nullptr,
                                     nullptr);
    TSVD_LAUNCH_CHECK();
  }
  TSVD_TRY(scan_i32_to_i64(W.cnt, B.colptr, cols, W.tmp, st));
  int64_t nnz = 0;
  TSVD_CUDA(cudaMemcpyAsync(&nnz, B.colptr + cols, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  if (nnz > W.nnz_cap) {  // the materialization's count was a lower bound: grow and recount
    TSVD_TRY(block_reserve(W, nnz, cols, rows));
  }
  B.nnz = nnz;
  if (cols > 0 && nnz > 0) {
    csc_kernel<1><<<g, 256, 0, st>>>(src, nullptr, B.colptr, B.rowidx, B.cval, W.ecol, W.keys,
                                     W.vals);
    TSVD_LAUNCH_CHECK();
  }
  // CSR: a stable sort of the entries by row keeps every row's columns ascending
  TSVD_CUDA(cudaMemsetAsync(W.cnt, 0, (rows + 1) * sizeof(int32_t), st));
  if (nnz > 0) {
    row_count_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(W.keys, nnz, W.cnt);
    TSVD_LAUNCH_CHECK();
  }
  TSVD_TRY(scan_i32_to_i64(W.cnt, B.rowptr, rows, W.tmp, st));
  if (nnz > 0) {
    int bits = 1;
    while ((1ll << bits) < rows) ++bits;
    bool in_alt = false;
    TSVD_TRY(stable_sort_pairs(W.keys, W.vals, W.keys_alt, W.vals_alt, nnz, bits, W.tmp, st,
                               &in_alt));
    const uint32_t *order = in_alt ? W.vals_alt : W.vals;
    csr_gather_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(order, nnz, W.ecol, B.cval, B.colidx,
                                                          B.rval);
    TSVD_LAUNCH_CHECK();
  }
  return TSVD_OK;
}

tsvd_status spmm_batched(const int64_t *const *ptr, const int32_t *const *idx,
                         const float *const *val, const int32_t *rows_out, int max_rows,
                         const __half *const *hi, const __half *const *lo, float *const *y,
                         float scale, int nprob, cudaStream_t st) {
  if (nprob == 0 || max_rows == 0) return TSVD_OK;
  SpmmArgs a{ptr, idx, val, rows_out, hi, lo, y, scale};
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(max_rows, 8),
                                                             ceil_div(8ll * sm_count(), nprob)));
  spmm_kernel<<<dim3(gx, nprob), 256, 0, st>>>(a);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

}  // namespace tsvd
