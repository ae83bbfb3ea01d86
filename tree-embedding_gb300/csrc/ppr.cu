// Dynamic forward-push PPR for all sources at once.
//
// State: r and p (float, |S| padded to Sp, a multiple of kChunk = 64),
// chunk-major: cell (v, s) is ((s / 64) * n + v) * 64 + s % 64. One warp
// holds the 64 sources of one chunk of one vertex, lane l the float2 of
// sources 2l and 2l + 1, so a push of vertex v for a chunk is one 256-byte
// vector atomic add (two adjacent lines) per neighbour, and the lines of one
// chunk are contiguous. Scattered read-modify-writes of 256-byte runs reach
// about 1.5x the line rate of 128-byte ones on HBM3e, and the push is bound
// by exactly these updates.
//
// Reference: the per-source FIFO push of Code/ppr_computation_store_dynamic.h
// (nodegree_DenseDynamicForwardPush :1394-1498, nodegree_DenseDirected...
// :2945-3030, ...Transpose :3356-3437) and its dynamic refresh (:2035-2121,
// :3811-3898, :4133-4228). The FIFO becomes frontier-synchronous rounds:
// every (v, chunk) in the frontier exchanges r[v][s] > rmax to zero, adds
// alpha*r to p[v][s] and scatters (1-alpha)*r/deg(v) to every neighbour. The
// next frontier is every touched (u, chunk) with some residue above rmax and
// a non-zero degree (collect_kernel over the touched bitset).
// The loop ends when a frontier is empty: every eligible residue <= rmax,
// the same invariant the FIFO leaves behind.
#include <algorithm>
#include <cmath>

#include "internal.h"
#include "ppr.h"

namespace tsvd {

namespace {

constexpr int kHeavy = 1024;  // neighbours per warp work unit for hub vertices
constexpr unsigned kFull = 0xffffffffu;

// Sets the bit of (u, chunk c) in a chunk-major bitset (bit c * n + u). The
// result is unused, so this is a fire-and-forget reduction (RED.OR). The
// touched set of a whole round (n * chunks bits) stays in L2, and chunk-major
// order makes the next frontier come out grouped by chunk, so the residual
// lines a stretch of a push round hits lie in one chunk's n * 128 bytes.
__device__ __forceinline__ void mark_pair(uint32_t *bits, int32_t u, int32_t c, int32_t n) {
  const int64_t idx = (int64_t)c * n + u;
  atomicOr(bits + (idx >> 5), 1u << (idx & 31));
}


struct StatAcc {
  unsigned long long pushes = 0, upd = 0, items = 0, iedges = 0;
};

// Only lane 0 of a warp counts; it adds its counts to one of kStatSlots
// slots (no block barrier, so a warp that runs out of items leaves at once).
__device__ __forceinline__ void flush_stats(const StatAcc &acc, unsigned long long *gstats) {
  if ((threadIdx.x & 31) != 0) return;
  unsigned long long *slot = gstats + (blockIdx.x % kStatSlots) * 4;
  if (acc.pushes) atomicAdd(slot + 0, acc.pushes);
  if (acc.upd) atomicAdd(slot + 1, acc.upd);
  if (acc.items) atomicAdd(slot + 2, acc.items);
  if (acc.iedges) atomicAdd(slot + 3, acc.iedges);
}

// Scatter w (sources 2 lane, 2 lane + 1; zero for sources not pushed) of
// vertex v's chunk c to neighbours [j0, j1): fire-and-forget vector atomic
// adds, and every neighbour's (u, chunk) is marked in the touched bitset for
// collect_kernel. Each half-warp takes one neighbour per instruction, lane q
// adding sources 4q..4q+3 as one float4 (RED.v4): two 256-byte runs per warp
// instruction, half the L1 requests of one float2 per lane and neighbour.
__device__ __forceinline__ void scatter_range(const PushArgs &a, const int32_t *nb, int32_t c,
                                              float2 w, int32_t j0, int32_t j1, int32_t mine) {
  const int lane = threadIdx.x & 31;
  const int q = lane & 15, half = lane >> 4;
  const float4 w4 = make_float4(__shfl_sync(kFull, w.x, 2 * q), __shfl_sync(kFull, w.y, 2 * q),
                                __shfl_sync(kFull, w.x, 2 * q + 1),
                                __shfl_sync(kFull, w.y, 2 * q + 1));
  const bool act = w4.x != 0.0f || w4.y != 0.0f || w4.z != 0.0f || w4.w != 0.0f;
  // r cells of (u, c * 64 + 4 q + {0..3}) = rc + 16 u
  float4 *rc = reinterpret_cast<float4 *>(a.r + (int64_t)c * a.n * kChunk) + q;
  // `mine` holds the ids of neighbours [j0, j0 + 32); each batch loads the
  // next batch's ids before issuing its own atomics
  for (int32_t jb = j0; jb < j1; jb += 32) {
    const int32_t jn = min(32, j1 - jb);
    const int32_t next = lane < j1 - jb - 32 ? __ldg(nb + jb + 32 + lane) : 0;
    for (int32_t t = 0; t < jn; t += 2) {
      const int32_t u = __shfl_sync(kFull, mine, (t + half) & 31);
      if (act && t + half < jn) atomicAdd(rc + (int64_t)u * (kChunk / 4), w4);
    }
    // each lane marks the neighbour it loaded: 32 independent reductions
    if (lane < jn) mark_pair(a.tflag, mine, c, a.n);
    mine = next;
  }
}

__global__ void __launch_bounds__(256) push_kernel(PushArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t nitems = *a.front_count;
  StatAcc acc;
  int2 it = gw < nitems ? __ldg(a.front + gw) : make_int2(0, 0);
  for (int64_t i = gw; i < nitems; i += nw) {
    const int32_t v = it.x, c = it.y;
    // the warp's next item is loaded while this one is pushed
    it = i + nw < nitems ? __ldg(a.front + i + nw) : make_int2(0, 0);
    // Everything the item needs that does not depend on its residues is
    // requested at once: degree, row start, reserve line, first neighbour ids
    // (only this warp writes the reserve of (v, chunk c) in a round).
    const int32_t d = a.deg[v];
    const int64_t o = a.off[v];
    const int32_t s0 = c * kChunk + 2 * lane;  // this lane's sources: s0, s0 + 1
    float *rp = a.r + ppr_cell(v, s0, a.n);
    float *pp = a.p + ppr_cell(v, s0, a.n);
    float2 x = __ldcg(reinterpret_cast<const float2 *>(rp));
    const float2 pv = __ldcg(reinterpret_cast<const float2 *>(pp));
    const int32_t *nb = a.nbr + o;
    const int32_t mine0 = lane < d ? __ldg(nb + lane) : 0;
    const bool in0 = s0 < a.nsrc, in1 = s0 + 1 < a.nsrc;
    // push above the current level of the threshold schedule (for hubs only
    // when hub_deg is set); sources between rmax and that level are parked
    // in the pending set for a later level
    const float th = (a.hub_deg > 0 && d < a.hub_deg) ? a.rmax_f : a.theta_f;
    bool act0 = in0 && x.x > th, act1 = in1 && x.y > th;
    const bool any = __any_sync(kFull, act0 || act1);
    // Co-push: once the lines are pushed for some source, the other sources
    // of the chunk with a residue above co_f ride along. The 256-byte atomic
    // per neighbour is paid either way; pushing a residue below rmax is a
    // valid push step (the push identity holds) that the FIFO would do later
    // or not at all, so it only tightens the error bound.
    if (any && a.co_f < th) {
      act0 = in0 && x.x > a.co_f;
      act1 = in1 && x.y > a.co_f;
    }
    if (th > a.rmax_f && d > 0 &&
        __any_sync(kFull, (in0 && !act0 && x.x > a.rmax_f) || (in1 && !act1 && x.y > a.rmax_f)) &&
        lane == 0)
      mark_pair(a.pend, v, c, a.n);
    if (!any) continue;
    const bool act = act0 || act1;
    if (d == 0) {
      // Isolated source of an undirected graph: the reference assigns
      // pi = alpha * r and keeps r (ppr:1433-1441); directed dangling
      // vertices are skipped (ppr:2971-2976).
      if (a.undirected && act0) pp[0] = a.alpha_f * x.x;
      if (a.undirected && act1) pp[1] = a.alpha_f * x.y;
      if (a.undirected && lane == 0 && a.vmark[v] == 0) a.vmark[v] = 1;
      continue;
    }
    if (act0) x.x = atomicExch(rp, 0.0f);
    if (act1) x.y = atomicExch(rp + 1, 0.0f);
    const float sc = a.one_minus_alpha_f / (float)d;
    const float2 w = make_float2(act0 ? x.x * sc : 0.0f, act1 ? x.y * sc : 0.0f);
    if (act)  // only this warp writes the reserve of (v, chunk c) in a round
      *reinterpret_cast<float2 *>(pp) = make_float2(act0 ? fmaf(a.alpha_f, x.x, pv.x) : pv.x,
                                                    act1 ? fmaf(a.alpha_f, x.y, pv.y) : pv.y);
    const int npush = __popc(__ballot_sync(kFull, act0)) + __popc(__ballot_sync(kFull, act1));
    if (lane == 0) {
      if (a.vmark[v] == 0) a.vmark[v] = 1;
      acc.pushes += npush;
      acc.upd += (unsigned long long)npush * (unsigned long long)d;
      acc.items += 1;
      acc.iedges += (unsigned long long)d;
    }
    if (d > kHeavy) {
      // Hub vertex: park the lane weights and split the neighbour list into
      // kHeavy-sized units processed by push_heavy_kernel.
      const int32_t units = (d + kHeavy - 1) / kHeavy;
      int32_t slot = 0, u0 = 0, ok = 0;
      if (lane == 0) {
        slot = atomicAdd(a.heavy_count, 1);
        u0 = atomicAdd(a.unit_count, units);
        ok = slot < a.heavy_cap && (int64_t)u0 + units <= a.unit_cap;
      }
      ok = __shfl_sync(kFull, ok, 0);
      slot = __shfl_sync(kFull, slot, 0);
      u0 = __shfl_sync(kFull, u0, 0);
      const bool units_reserved = (int64_t)u0 + units <= a.unit_cap;
      if (ok) {
        reinterpret_cast<float2 *>(a.heavy_w)[(int64_t)slot * 32 + lane] = w;
        if (lane == 0) a.heavy_item[slot] = make_int2(v, c);
      }
      if (units_reserved)
        for (int32_t k = lane; k < units; k += 32)
          a.units[u0 + k] = make_int2(ok ? slot : -1, k * kHeavy);
      if (ok) continue;
      // buffers full: process this hub inline
    }
    scatter_range(a, nb, c, w, 0, d, mine0);
  }
  flush_stats(acc, a.stats);
}

__global__ void __launch_bounds__(256) push_heavy_kernel(PushArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t nunits = min(*a.unit_count, a.unit_cap);
  for (int64_t i = gw; i < nunits; i += nw) {
    int2 u = a.units[i];
    if (u.x < 0) continue;
    int2 it = a.heavy_item[u.x];
    const float2 w = reinterpret_cast<const float2 *>(a.heavy_w)[(int64_t)u.x * 32 + lane];
    const int32_t d = a.deg[it.x];
    const int32_t *nb = a.nbr + a.off[it.x];
    const int32_t j1 = min(d, u.y + kHeavy);
    const int32_t mine0 = lane < j1 - u.y ? __ldg(nb + u.y + lane) : 0;
    scatter_range(a, nb, it.y, w, u.y, j1, mine0);
  }
}

// Scan the touched bitset; for each touched (u, chunk) with some residue
// above theta and deg(u) > 0, append it to the next frontier. Clears the bits.
// A warp takes the set bits of a word eight at a time: lane group g (4 lanes)
// reads pair g's 256-byte residue run as sixteen float4 (four per lane), so
// eight runs are in flight per warp. Padding sources (s >= |S|) hold zero
// residue.
__global__ void __launch_bounds__(256) collect_kernel(CollectArgs a) {
  __shared__ int2 buf[2048];
  __shared__ int32_t nbuf, gbase;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, gl = lane & 3;
  const int64_t words_per_iter = 64;  // 8 warps x 8 words
  for (int64_t w0 = (int64_t)blockIdx.x * words_per_iter; w0 < a.nwords;
       w0 += (int64_t)gridDim.x * words_per_iter) {
    if (threadIdx.x == 0) nbuf = 0;
    // the warp's eight words in one load (lanes 0-7): in the late rounds of a
    // push almost every word is zero, and eight dependent loads per warp made
    // the scan of the bitset cost 0.14 ms a round
    const int64_t wbase = w0 + warp * 8;
    const uint32_t wv = (lane < 8 && wbase + lane < a.nwords) ? __ldcg(a.tflag + wbase + lane) : 0u;
    __syncthreads();
    for (int k = 0; k < 8; ++k) {
      const int64_t wi = wbase + k;
      if (wi >= a.nwords) break;
      uint32_t bits = __shfl_sync(kFull, wv, k);
      if (!bits) continue;
      if (lane == 0) a.tflag[wi] = 0;
      while (bits) {
        // the next (up to) eight set bits, one per lane group
        uint32_t rest = bits;
        int mybit = -1;
        for (int g = 0; g < 8 && rest; ++g) {
          const int bpos = __ffs(rest) - 1;
          rest &= rest - 1;
          if (g == grp) mybit = bpos;
        }
        bits = rest;
        int32_t u = 0, c = 0, du = 0;
        bool live = mybit >= 0;
        if (live) {
          const int64_t idx = wi * 32 + mybit;
          u = (int32_t)(idx % a.n);
          c = (int32_t)(idx / a.n);
          du = a.deg[u];
          live = du != 0;
        }
        const float th = (a.hub_deg > 0 && du < a.hub_deg) ? a.rmax_f : a.theta_f;
        float m = 0.f;
        if (live) {
          const float4 *line =
              reinterpret_cast<const float4 *>(a.r + ppr_cell(u, c * kChunk, a.n));
          const float4 x0 = __ldcg(line + gl), x1 = __ldcg(line + gl + 4);
          const float4 x2 = __ldcg(line + gl + 8), x3 = __ldcg(line + gl + 12);
          const float m0 = fmaxf(fmaxf(fmaxf(x0.x, x0.y), fmaxf(x0.z, x0.w)),
                                 fmaxf(fmaxf(x1.x, x1.y), fmaxf(x1.z, x1.w)));
          const float m1 = fmaxf(fmaxf(fmaxf(x2.x, x2.y), fmaxf(x2.z, x2.w)),
                                 fmaxf(fmaxf(x3.x, x3.y), fmaxf(x3.z, x3.w)));
          m = fmaxf(m0, m1);
        }
        const unsigned above = __ballot_sync(kFull, live && m > th);
        const unsigned parked =
            __ballot_sync(kFull, live && th > a.rmax_f && m > a.rmax_f) & ~above;
        const unsigned gmask = 0xFu << (grp * 4);
        if (gl == 0 && live) {
          if (above & gmask) buf[atomicAdd(&nbuf, 1)] = make_int2(u, c);
          else if (parked & gmask) mark_pair(a.pend, u, c, a.n);  // for a lower level
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) gbase = nbuf ? atomicAdd(a.next_count, nbuf) : 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nbuf; i += blockDim.x) {
      const int64_t dst = (int64_t)gbase + i;
      if (dst < a.cap) a.next[dst] = buf[i];
      else atomicExch(a.overflow, 1);
    }
    __syncthreads();
  }
}

// Dynamic refresh of the new adjacency slots of vertex u, for one chunk of
// sources: for slot j >= 1 (the reference skips j == 0, ppr:2086-2093),
//   p_u *= (j+1)/j ; r_u -= p_u/(j+1)/alpha ; r_w += (1-alpha) p_u/(j+1)/alpha.
// The work is walked chunk by chunk and, within a chunk, in vertex order: a
// warp takes 32 consecutive vertices of one chunk and refreshes those that
// gained slots, so consecutive warps read and write consecutive stretches of
// the chunk's reserve runs. (With the reserve in host memory these accesses
// cross NVLink-C2C, where scattered 256-byte requests run several times
// slower than ordered ones.)
__global__ void __launch_bounds__(256) refresh_kernel(RefreshArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t groups = ((int64_t)a.n + 31) / 32;
  const int64_t nitems = groups * a.chunks;
  for (int64_t i = gw; i < nitems; i += nw) {
    const int32_t c = (int32_t)(i / groups);
    const int32_t ubase = (int32_t)((i % groups) * 32);
    const int32_t mine = ubase + lane;
    int32_t j0m = 0, j1m = 0;
    if (mine < a.n) {
      j0m = __ldg(a.former + mine);
      j1m = __ldg(a.deg + mine);
    }
    unsigned todo = __ballot_sync(kFull, j1m > j0m);
    while (todo) {
      const int k = __ffs(todo) - 1;
      todo &= todo - 1;
      const int32_t u = ubase + k;
      const int32_t j0 = __shfl_sync(kFull, j0m, k), j1 = __shfl_sync(kFull, j1m, k);
      const int32_t s0 = c * kChunk + 2 * lane;  // this lane's sources: s0, s0 + 1
      const bool valid = s0 < a.nsrc;            // padding sources hold zeros and stay zero
      const int32_t *nb = a.nbr + a.off[u];
      float2 *pu = reinterpret_cast<float2 *>(a.p + ppr_cell(u, s0, a.n));
      float2 pf = valid ? *pu : make_float2(0.0f, 0.0f);
      float2 rdelta = make_float2(0.0f, 0.0f);
      bool any = false;
      for (int32_t j = max(j0, 1); j < j1; ++j) {
        any = true;
        const int32_t w = __ldg(nb + j);
        const float jp1 = (float)(j + 1);
        if (a.intdiv) {
          const float f = (float)((j + 1) / j);
          pf.x = pf.x * f;
          pf.y = pf.y * f;
        } else {
          const float f = jp1 / (float)j;
          pf.x = pf.x * f;
          pf.y = pf.y * f;
        }
        const float2 q = make_float2(pf.x / jp1, pf.y / jp1);  // p_u / (j+1)
        rdelta.x -= q.x * a.inv_alpha_f;
        rdelta.y -= q.y * a.inv_alpha_f;
        if (valid)
          atomicAdd(reinterpret_cast<float2 *>(a.r + ppr_cell(w, s0, a.n)),
                    make_float2(q.x * a.oma_over_alpha_f, q.y * a.oma_over_alpha_f));
        if (lane == 0) mark_pair(a.tflag, w, c, a.n);
      }
      if (any) {
        if (valid) {
          *pu = pf;
          atomicAdd(reinterpret_cast<float2 *>(a.r + ppr_cell(u, s0, a.n)), rdelta);
        }
      }
      // A formerly dangling vertex (j0 == 0) may hold residue it could not
      // push; in exact mode it is re-examined like any touched vertex. The
      // reference's dense path skips slot 0 entirely (ppr:2086-2093).
      if ((any || (!a.intdiv && j0 == 0 && j1 > 0)) && lane == 0)
        mark_pair(a.tflag, u, c, a.n);
    }
  }
}

// Lowering the threshold: parked (vertex, chunk) pairs become touched again.
__global__ void unpark_kernel(uint32_t *__restrict__ tflag, uint32_t *__restrict__ pend,
                              int64_t nwords) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nwords;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = pend[i];
    if (b) {
      tflag[i] |= b;
      pend[i] = 0;
    }
  }
}


__global__ void init_sources_kernel(const int32_t *__restrict__ sources, int32_t nsrc,
                                    float *__restrict__ r, int32_t n,
                                    int2 *__restrict__ front, int32_t *__restrict__ count) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nsrc;
       k += gridDim.x * blockDim.x) {
    int32_t v = sources[k];
    r[ppr_cell(v, k, n)] = 1.0f;
    front[k] = make_int2(v, k / kChunk);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = nsrc;
}

// Zero fill with 16-byte stores (also for p in mapped host memory).
__global__ void zero_kernel(float4 *__restrict__ x, int64_t n4) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

tsvd_status zero_floats(float *x, size_t count, cudaStream_t st) {
  // count is a multiple of 4: n * Sp with Sp a multiple of kChunk
  zero_kernel<<<grid_for((int64_t)(count / 4), 256, 8), 256, 0, st>>>(
      reinterpret_cast<float4 *>(x), (int64_t)(count / 4));
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

float largest_float_not_above(double x) {
  float f = (float)x;
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}

}  // namespace

tsvd_status ppr_alloc(PprState &P, int32_t n, int32_t nsrc, int32_t sp, bool host_reserve) {
  P.n = n;
  P.nsrc = nsrc;
  P.sp = sp;
  if (sp % kChunk) return fail(TSVD_ERR_INVALID, "ppr: padded |S| %d not a multiple of %d", sp, kChunk);
  P.chunks = sp / kChunk;
  size_t cells = (size_t)n * sp;
  TSVD_CUDA(cudaMalloc(&P.r, cells * sizeof(float)));
  TSVD_CUDA(cudaMemset(P.r, 0, cells * sizeof(float)));
  if (host_reserve) {
    void *h = nullptr;
    if (cudaHostAlloc(&h, cells * sizeof(float), cudaHostAllocMapped | cudaHostAllocPortable) !=
        cudaSuccess) {
      cudaGetLastError();
      return fail(TSVD_ERR_OOM, "ppr: %.1f GB of pinned host memory for the reserve",
                  cells * 4.0 / 1e9);
    }
    P.p_host = static_cast<float *>(h);
    void *d = nullptr;
    TSVD_CUDA(cudaHostGetDevicePointer(&d, h, 0));
    P.p = static_cast<float *>(d);
  } else {
    TSVD_CUDA(cudaMalloc(&P.p, cells * sizeof(float)));
  }
  TSVD_TRY(zero_floats(P.p, cells, nullptr));
  TSVD_CUDA(cudaDeviceSynchronize());
  P.nwords = ceil_div((int64_t)n * P.chunks, 32);
  TSVD_CUDA(cudaMalloc(&P.tflag, P.nwords * sizeof(uint32_t)));
  TSVD_CUDA(cudaMemset(P.tflag, 0, P.nwords * sizeof(uint32_t)));
  TSVD_CUDA(cudaMalloc(&P.pend, P.nwords * sizeof(uint32_t)));
  TSVD_CUDA(cudaMemset(P.pend, 0, P.nwords * sizeof(uint32_t)));
  P.cap = (int64_t)n * P.chunks;
  for (int i = 0; i < 2; ++i) TSVD_CUDA(cudaMalloc(&P.front[i], P.cap * sizeof(int2)));
  P.heavy_cap = 1 << 20;
  P.unit_cap = 1 << 22;
  TSVD_CUDA(cudaMalloc(&P.heavy_w, (size_t)P.heavy_cap * kChunk * sizeof(float)));
  TSVD_CUDA(cudaMalloc(&P.heavy_item, (size_t)P.heavy_cap * sizeof(int2)));
  TSVD_CUDA(cudaMalloc(&P.units, (size_t)P.unit_cap * sizeof(int2)));
  TSVD_CUDA(cudaMalloc(&P.upd, (size_t)n * sizeof(int32_t)));
  TSVD_CUDA(cudaMalloc(&P.counters, 16 * sizeof(int32_t)));
  TSVD_CUDA(cudaMemset(P.counters, 0, 16 * sizeof(int32_t)));
  TSVD_CUDA(cudaMalloc(&P.stats, kStatSlots * 4 * sizeof(unsigned long long)));
  TSVD_CUDA(cudaMallocHost(&P.host_counters, 16 * sizeof(int32_t)));
  for (auto &e : P.kev) TSVD_CUDA(cudaEventCreate(&e));
  return TSVD_OK;
}

void ppr_free(PprState &P) {
  cudaFree(P.r);
  if (P.p_host)
    cudaFreeHost(P.p_host);
  else
    cudaFree(P.p);
  cudaFree(P.tflag); cudaFree(P.pend);
  cudaFree(P.front[0]); cudaFree(P.front[1]);
  cudaFree(P.heavy_w); cudaFree(P.heavy_item); cudaFree(P.units);
  cudaFree(P.upd); cudaFree(P.counters); cudaFree(P.stats);
  cudaFreeHost(P.host_counters);
  for (auto &e : P.kev)
    if (e) cudaEventDestroy(e);
  P = PprState();
}

// counters: [0],[1] frontier counts, [2] heavy count, [3] unit count,
// [4] overflow flag, [5] number of updated vertices.
tsvd_status ppr_refresh(PprState &P, const Adjacency &A, const int32_t *sources_dev,
                        bool from_scratch, const PprParams &prm, uint8_t *vmark,
                        cudaStream_t st) {
  (void)vmark;
  if (from_scratch) {
    TSVD_CUDA(cudaMemsetAsync(P.r, 0, (size_t)P.n * P.sp * sizeof(float), st));
    TSVD_TRY(zero_floats(P.p, (size_t)P.n * P.sp, st));
    TSVD_CUDA(cudaMemsetAsync(P.tflag, 0, P.nwords * sizeof(uint32_t), st));
    TSVD_CUDA(cudaMemsetAsync(P.pend, 0, P.nwords * sizeof(uint32_t), st));
    P.cur = 0;
    init_sources_kernel<<<grid_for(P.nsrc, 256), 256, 0, st>>>(sources_dev, P.nsrc, P.r, P.n,
                                                                  P.front[0], P.counters + 0);
    TSVD_LAUNCH_CHECK();
    P.seeded = true;
    return TSVD_OK;
  }
  // vertices with new slots
  TSVD_CUDA(cudaMemsetAsync(P.counters + 5, 0, sizeof(int32_t), st));
  RefreshArgs ra;
  ra.n = P.n; ra.chunks = P.chunks; ra.nsrc = P.nsrc;
  ra.sp = P.sp; ra.off = A.off; ra.deg = A.deg; ra.former = A.former; ra.nbr = A.nbr;
  ra.r = P.r; ra.p = P.p; ra.tflag = P.tflag; ra.intdiv = prm.intdiv;
  ra.inv_alpha_f = (float)(1.0 / prm.alpha);
  ra.oma_over_alpha_f = (float)((1.0 - prm.alpha) / prm.alpha);
  refresh_kernel<<<grid_for((A.n + 31) / 32 * (int64_t)P.chunks * 32, 256, 16), 256, 0, st>>>(ra);
  TSVD_LAUNCH_CHECK();
  // seed the frontier from the touched (vertex, chunk) pairs
  P.cur = 0;
  TSVD_CUDA(cudaMemsetAsync(P.counters + 0, 0, sizeof(int32_t), st));
  CollectArgs ca;
  ca.tflag = P.tflag; ca.nwords = P.nwords; ca.n = P.n; ca.chunks = P.chunks; ca.nsrc = P.nsrc;
  ca.sp = P.sp; ca.r = P.r; ca.deg = A.deg; ca.rmax_f = largest_float_not_above(prm.rmax);
  ca.theta_f = ca.rmax_f; ca.hub_deg = 0; ca.pend = P.pend;
  ca.next = P.front[0]; ca.next_count = P.counters + 0; ca.cap = P.cap;
  ca.overflow = P.counters + 4;
  collect_kernel<<<grid_for(ceil_div(P.nwords, 64) * 256, 256, 8), 256, 0, st>>>(ca);
  TSVD_LAUNCH_CHECK();
  P.seeded = true;
  return TSVD_OK;
}

namespace {

// One push (one PPR state), advanced check_every rounds at a time.
struct PushJob {
  PprState *P = nullptr;
  cudaStream_t st = nullptr;
  PushArgs pa{};
  CollectArgs ca{};
  int gpush = 0, gcol = 0;
  int level = 0;
  bool done = false;
  int64_t rounds = 0;
  double kernel_ms = 0;
};

tsvd_status job_begin(PushJob &J, PprState &P, const Adjacency &A, const PprParams &prm,
                      uint8_t *vmark, cudaStream_t st) {
  if (!P.seeded) return fail(TSVD_ERR_STATE, "push before refresh");
  J.P = &P;
  J.st = st;
  TSVD_CUDA(cudaMemsetAsync(P.stats, 0, kStatSlots * 4 * sizeof(unsigned long long), st));
  TSVD_CUDA(cudaMemsetAsync(P.counters + 4, 0, sizeof(int32_t), st));
  const float rmax_f = largest_float_not_above(prm.rmax);
  PushArgs &pa = J.pa;
  pa.r = P.r; pa.p = P.p; pa.off = A.off; pa.deg = A.deg; pa.nbr = A.nbr;
  pa.n = P.n; pa.sp = P.sp; pa.nsrc = P.nsrc; pa.chunks = P.chunks; pa.tflag = P.tflag; pa.pend = P.pend;
  pa.alpha_f = (float)prm.alpha; pa.one_minus_alpha_f = (float)(1.0 - prm.alpha);
  pa.rmax_f = rmax_f; pa.undirected = prm.undirected; pa.vmark = vmark;
  pa.hub_deg = prm.hub_degree;
  pa.co_f = prm.cofrac >= 1.0 ? rmax_f : (float)(prm.rmax * std::max(prm.cofrac, 0.0));
  pa.heavy_w = P.heavy_w; pa.heavy_item = P.heavy_item;
  pa.heavy_count = P.counters + 2; pa.heavy_cap = P.heavy_cap;
  pa.units = P.units; pa.unit_count = P.counters + 3; pa.unit_cap = P.unit_cap;
  pa.overflow = P.counters + 4; pa.stats = P.stats;
  CollectArgs &ca = J.ca;
  ca.tflag = P.tflag; ca.pend = P.pend; ca.nwords = P.nwords; ca.n = P.n; ca.chunks = P.chunks;
  ca.nsrc = P.nsrc; ca.sp = P.sp; ca.r = P.r; ca.deg = A.deg; ca.rmax_f = rmax_f;
  ca.cap = P.cap; ca.overflow = P.counters + 4;
  ca.hub_deg = prm.hub_degree;
  J.gpush = grid_for((int64_t)1 << 30, 256, 8);
  J.gcol = grid_for(ceil_div(P.nwords, 64) * 256, 256, 8);
  J.level = std::max(1, prm.levels) - 1;
  J.done = false;
  J.rounds = 0;
  J.kernel_ms = 0;
  return TSVD_OK;
}

// Threshold schedule: residues above rmax * ratio^k are pushed first, k
// descending to 0. Lower residues wait in the pending set, so a vertex
// collects more before it is pushed; the last level is the plain rmax test
// and leaves the same invariant (every eligible residue <= rmax).
float level_theta(const PprParams &prm, int level, float rmax_f) {
  const float theta = largest_float_not_above(prm.rmax * std::pow(prm.ratio, (double)level));
  return std::max(theta, rmax_f);
}

// Launches `count` rounds on the job's stream (asynchronous).
tsvd_status job_rounds(PushJob &J, int count) {
  PprState &P = *J.P;
  cudaStream_t st = J.st;
  for (int k = 0; k < count; ++k) {
    const int cur = P.cur, nxt = 1 - P.cur;
    J.pa.front = P.front[cur];
    J.pa.front_count = P.counters + cur;
    TSVD_CUDA(cudaMemsetAsync(P.counters + 2, 0, 2 * sizeof(int32_t), st));
    TSVD_CUDA(cudaMemsetAsync(P.counters + nxt, 0, sizeof(int32_t), st));
    TSVD_CUDA(cudaEventRecord(P.kev[2 * k], st));
    push_kernel<<<J.gpush, 256, 0, st>>>(J.pa);
    TSVD_LAUNCH_CHECK();
    push_heavy_kernel<<<J.gpush, 256, 0, st>>>(J.pa);
    TSVD_LAUNCH_CHECK();
    TSVD_CUDA(cudaEventRecord(P.kev[2 * k + 1], st));
    J.ca.next = P.front[nxt];
    J.ca.next_count = P.counters + nxt;
    collect_kernel<<<J.gcol, 256, 0, st>>>(J.ca);
    TSVD_LAUNCH_CHECK();
    P.cur = nxt;
    ++J.rounds;
  }
  TSVD_CUDA(cudaMemcpyAsync(P.host_counters, P.counters, 8 * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
  return TSVD_OK;
}

// Waits for the job's launched rounds; ends the level when its frontier is
// empty, starting the next level (or finishing) as the schedule says.
tsvd_status job_poll(PushJob &J, int count, const PprParams &prm) {
  PprState &P = *J.P;
  TSVD_CUDA(cudaStreamSynchronize(J.st));
  for (int k = 0; k < count; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, P.kev[2 * k], P.kev[2 * k + 1]) == cudaSuccess) J.kernel_ms += ms;
  }
  if (P.host_counters[4]) return fail(TSVD_ERR_STATE, "push: frontier buffer overflow");
  if (P.host_counters[P.cur] != 0) {
    if (J.rounds >= prm.max_rounds)
      return fail(TSVD_ERR_TIMEOUT, "push: %lld rounds without convergence", (long long)J.rounds);
    return TSVD_OK;
  }
  if (J.level == 0) {
    J.done = true;
    return TSVD_OK;
  }
  // the frontier of this level is empty: re-examine parked pairs at the next
  --J.level;
  J.pa.theta_f = J.ca.theta_f = level_theta(prm, J.level, J.pa.rmax_f);
  unpark_kernel<<<grid_for(P.nwords, 256, 8), 256, 0, J.st>>>(P.tflag, P.pend, P.nwords);
  TSVD_LAUNCH_CHECK();
  TSVD_CUDA(cudaMemsetAsync(P.counters + P.cur, 0, sizeof(int32_t), J.st));
  J.ca.next = P.front[P.cur];
  J.ca.next_count = P.counters + P.cur;
  collect_kernel<<<J.gcol, 256, 0, J.st>>>(J.ca);
  TSVD_LAUNCH_CHECK();
  return TSVD_OK;
}

tsvd_status job_finish(PushJob &J, PushStats *out) {
  PprState &P = *J.P;
  unsigned long long slots[kStatSlots * 4], hs[4] = {0, 0, 0, 0};
  TSVD_CUDA(cudaMemcpyAsync(slots, P.stats, sizeof slots, cudaMemcpyDeviceToHost, J.st));
  TSVD_CUDA(cudaStreamSynchronize(J.st));
  for (int k = 0; k < kStatSlots * 4; ++k) hs[k % 4] += slots[k];
  if (out) {
    out->rounds = J.rounds;
    out->pushes = (int64_t)hs[0];
    out->edge_updates = (int64_t)hs[1];
    out->items = (int64_t)hs[2];
    out->item_edges = (int64_t)hs[3];
    out->kernel_ms = J.kernel_ms;
  }
  P.seeded = false;
  return TSVD_OK;
}

}  // namespace

tsvd_status ppr_push(PprState &P, const Adjacency &A, const PprParams &prm, uint8_t *vmark,
                     cudaStream_t st, PushStats *out) {
  PushJob J;
  TSVD_TRY(job_begin(J, P, A, prm, vmark, st));
  J.pa.theta_f = J.ca.theta_f = level_theta(prm, J.level, J.pa.rmax_f);
  const int check_every = std::min(8, prm.check_every > 0 ? prm.check_every : 4);
  while (!J.done) {
    TSVD_TRY(job_rounds(J, check_every));
    TSVD_TRY(job_poll(J, check_every, prm));
  }
  return job_finish(J, out);
}

}  // namespace tsvd
