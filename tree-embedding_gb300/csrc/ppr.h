// PPR store: device state and kernel argument blocks.
#pragma once
#include "internal.h"

namespace tsvd {

// Sources per chunk. The kChunk sources of one chunk of one vertex share a
// 256-byte pair of lines; a warp holds them as one float2 per lane.
constexpr int kChunk = 64;

// Cell of (vertex v, source s) in the chunk-major r / p arrays: the lines of
// one chunk are contiguous over the n vertices.
__host__ __device__ __forceinline__ int64_t ppr_cell(int32_t v, int32_t s, int32_t n) {
  return ((int64_t)(s >> 6) * n + v) * kChunk + (s & (kChunk - 1));
}

constexpr int kStatSlots = 64;  // push counters are spread over this many slots

struct PprState {
  int32_t n = 0, nsrc = 0, sp = 0, chunks = 0;
  float *r = nullptr, *p = nullptr;  // [chunks][n][kChunk], see ppr_cell
  float *p_host = nullptr;           // p's host allocation when it is mapped pinned host memory
  uint32_t *tflag = nullptr;         // touched (vertex, chunk) bitset, chunk-major
  uint32_t *pend = nullptr;          // parked below the current threshold level
  int64_t nwords = 0;                // words of either bitset
  int2 *front[2] = {nullptr, nullptr};
  int64_t cap = 0;
  int cur = 0;
  bool seeded = false;
  float *heavy_w = nullptr;
  int2 *heavy_item = nullptr;
  int2 *units = nullptr;
  int32_t heavy_cap = 0, unit_cap = 0;
  int32_t *upd = nullptr;
  int32_t *counters = nullptr;
  int32_t *host_counters = nullptr;
  unsigned long long *stats = nullptr;  // [kStatSlots][4]
  cudaEvent_t kev[16] = {};  // scatter-kernel timing, two per round of a check interval
};

struct PprParams {
  double alpha = 0.2, rmax = 1e-7;
  int intdiv = 0;
  int undirected = 1;
  int check_every = 4;
  int64_t max_rounds = 100000;
  int levels = 1;       // threshold schedule: rmax * ratio^(levels-1) ... rmax
  double ratio = 8.0;
  double cofrac = 1.0;  // co-push residues above rmax * cofrac on pushed lines
  int32_t hub_degree = 0;  // > 0: the threshold schedule applies to deg >= hub_degree only
};

struct PushStats {
  int64_t rounds = 0, pushes = 0, edge_updates = 0, items = 0;
  double kernel_ms = 0;  // push_kernel + push_heavy_kernel device time
  int64_t item_edges = 0;  // sum of deg(v) over pushed (vertex, chunk) items
};

struct PushArgs {
  const int2 *front;
  const int32_t *front_count;
  float *r, *p;
  const int64_t *off;
  const int32_t *deg, *nbr;
  int32_t n, sp, nsrc, chunks;
  uint32_t *tflag, *pend;
  float alpha_f, one_minus_alpha_f, rmax_f, theta_f, co_f;
  int32_t hub_deg;  // > 0: theta_f applies to deg >= hub_deg only (rmax_f below)
  int undirected;
  uint8_t *vmark;
  float *heavy_w;
  int2 *heavy_item;
  int32_t *heavy_count;
  int32_t heavy_cap;
  int2 *units;
  int32_t *unit_count;
  int32_t unit_cap;
  int32_t *overflow;
  unsigned long long *stats;
};

struct CollectArgs {
  uint32_t *tflag, *pend;
  float theta_f;
  int32_t hub_deg;
  int64_t nwords;
  int32_t n, chunks, nsrc, sp;
  const float *r;
  const int32_t *deg;
  float rmax_f;
  int2 *next;
  int32_t *next_count;
  int64_t cap;
  int32_t *overflow;
};

struct RefreshArgs {
  int32_t n, chunks, nsrc, sp;
  const int64_t *off;
  const int32_t *deg, *former, *nbr;
  float *r, *p;
  uint32_t *tflag;
  int intdiv;
  float inv_alpha_f, oma_over_alpha_f;
};

// host_reserve: p in pinned host memory mapped into the device address space
// (the kernels reach it over NVLink-C2C); r always in device memory.
tsvd_status ppr_alloc(PprState &P, int32_t n, int32_t nsrc, int32_t sp, bool host_reserve);
void ppr_free(PprState &P);
tsvd_status ppr_refresh(PprState &P, const Adjacency &A, const int32_t *sources_dev,
                        bool from_scratch, const PprParams &prm, uint8_t *vmark,
                        cudaStream_t st);
tsvd_status ppr_push(PprState &P, const Adjacency &A, const PprParams &prm, uint8_t *vmark,
                     cudaStream_t st, PushStats *out);

}  // namespace tsvd
