// PPR store: device state and kernel argument blocks.
#pragma once
#include "internal.h"

namespace tsvd {

struct PprState {
  int32_t n = 0, nsrc = 0, sp = 0, chunks = 0;
  float *r = nullptr, *p = nullptr;  // [n][sp]
  uint32_t *tflag = nullptr;         // touched (vertex, chunk) bitset
  int64_t nwords = 0;
  int2 *front[2] = {nullptr, nullptr};
  int64_t cap = 0;
  int cur = 0;
  bool seeded = false;
  float *heavy_w = nullptr;
  int2 *heavy_item = nullptr;
  uint32_t *heavy_mask = nullptr;
  int2 *units = nullptr;
  int32_t heavy_cap = 0, unit_cap = 0;
  int32_t *upd = nullptr;
  int32_t *counters = nullptr;
  int32_t *host_counters = nullptr;
  unsigned long long *stats = nullptr;
};

struct PprParams {
  double alpha = 0.2, rmax = 1e-7;
  int intdiv = 0;
  int undirected = 1;
  int check_every = 4;
  int64_t max_rounds = 100000;
};

struct PushStats {
  int64_t rounds = 0, pushes = 0, edge_updates = 0;
};

struct PushArgs {
  const int2 *front;
  const int32_t *front_count;
  float *r, *p;
  const int64_t *off;
  const int32_t *deg, *nbr;
  int32_t sp, nsrc, chunks;
  uint32_t *tflag;
  float alpha_f, one_minus_alpha_f, rmax_f;
  int undirected;
  uint8_t *vmark;
  float *heavy_w;
  int2 *heavy_item;
  uint32_t *heavy_mask;
  int32_t *heavy_count;
  int32_t heavy_cap;
  int2 *units;
  int32_t *unit_count;
  int32_t unit_cap;
  int32_t *overflow;
  unsigned long long *stats;
};

struct CollectArgs {
  uint32_t *tflag;
  int64_t nwords;
  int32_t chunks, nsrc, sp;
  const float *r;
  const int32_t *deg;
  float rmax_f;
  int2 *next;
  int32_t *next_count;
  int64_t cap;
  int32_t *overflow;
};

struct RefreshArgs {
  const int32_t *upd;
  const int32_t *nupd;
  int32_t chunks, nsrc, sp;
  const int64_t *off;
  const int32_t *deg, *former, *nbr;
  float *r, *p;
  uint32_t *tflag;
  int intdiv;
  float inv_alpha_f, oma_over_alpha_f;
};

tsvd_status ppr_alloc(PprState &P, int32_t n, int32_t nsrc, int32_t sp);
void ppr_free(PprState &P);
tsvd_status ppr_refresh(PprState &P, const Adjacency &A, const int32_t *sources_dev,
                        bool from_scratch, const PprParams &prm, uint8_t *vmark,
                        cudaStream_t st);
tsvd_status ppr_push(PprState &P, const Adjacency &A, const PprParams &prm, uint8_t *vmark,
                     cudaStream_t st, PushStats *out);

}  // namespace tsvd
