/*
 * Synthetic workload generator of the oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A second, independent statement of the seeded inputs the product draws
 * (R-MAT edge lists, the snapshot split and the source sample), so that the
 * CPU reference arm of bench.py and the tests can build the same workload
 * without loading the product library. tests/test_oracle_synth.py checks that
 * both produce identical bytes. The counter-based streams are the shared
 * Philox4x32-10 specification in philox_gauss.h.
 *
 *   R-MAT: for candidate i, ceil(scale / 4) Philox calls (counter i, stream 1,
 *   call index) give `scale` 32-bit words; word x picks the quadrant
 *   (x < a: (0,0), < a+b: (0,1), < a+b+c: (1,0), else (1,1)) bit by bit from
 *   the most significant. Candidates outside [0, n), self-loops and (for
 *   undirected graphs) unordered duplicates are dropped; the first
 *   occurrence of each pair in candidate order is kept, the first m of those
 *   in candidate order are the edges. Vertex ids are then relabelled by a
 *   seeded Fisher-Yates permutation (stream 2) and the edge list is shuffled
 *   (stream 3) into its uniform-random timestamp order.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "../tree-embedding_gb300/csrc/philox_gauss.h"

enum { kStreamRmat = 1, kStreamRelabel = 2, kStreamShuffle = 3, kStreamSample = 4 };

static uint64_t os_rand_u64(uint64_t seed, uint32_t stream, uint64_t idx) {
  tsvd_philox4 r = tsvd_philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32), stream, 0x53594e54u,
                                      (uint32_t)seed, (uint32_t)(seed >> 32));
  return ((uint64_t)r.v[0] << 32) | r.v[1];
}

static uint64_t os_bounded(uint64_t r, uint64_t n) {
  return (uint64_t)(((unsigned __int128)r * n) >> 64);
}

typedef struct {
  uint64_t *cand;
  uint64_t lo, hi, step, off;
  int32_t n, scale, directed;
  uint64_t ta, tab, tabc, seed;
} gen_job;

static void *gen_run(void *arg) {
  gen_job *J = (gen_job *)arg;
  const int calls = (J->scale + 3) / 4;
  for (uint64_t i = J->lo + J->off; i < J->hi; i += J->step) {
    uint64_t u = 0, v = 0;
    for (int cl = 0; cl < calls; ++cl) {
      tsvd_philox4 r = tsvd_philox4x32_10((uint32_t)i, (uint32_t)(i >> 32), kStreamRmat,
                                          (uint32_t)cl, (uint32_t)J->seed,
                                          (uint32_t)(J->seed >> 32));
      for (int w = 0; w < 4 && cl * 4 + w < J->scale; ++w) {
        uint64_t x = r.v[w];
        uint64_t row = x >= J->tab;
        uint64_t col = (x >= J->ta && x < J->tab) || x >= J->tabc;
        u = (u << 1) | row;
        v = (v << 1) | col;
      }
    }
    if (u >= (uint64_t)J->n || v >= (uint64_t)J->n || u == v) {
      J->cand[i] = ~0ull;
      continue;
    }
    if (!J->directed && u > v) {
      uint64_t t = u;
      u = v;
      v = t;
    }
    J->cand[i] = (u << 32) | v;
  }
  return NULL;
}

/* Stable LSD radix sort of candidate indices by their keys (8-bit digits over
 * the bits the keys use): equal keys stay in candidate order. */
static int sort_by_key(const uint64_t *key, uint32_t *idx, uint64_t cnt, int key_bits) {
  uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (cnt ? cnt : 1));
  uint64_t *kcur = (uint64_t *)malloc(sizeof(uint64_t) * (cnt ? cnt : 1));
  uint64_t *ktmp = (uint64_t *)malloc(sizeof(uint64_t) * (cnt ? cnt : 1));
  if (!tmp || !kcur || !ktmp) {
    free(tmp);
    free(kcur);
    free(ktmp);
    return -1;
  }
  uint64_t any_bits = 0;
  for (uint64_t i = 0; i < cnt; ++i) {
    kcur[i] = key[idx[i]];
    any_bits |= kcur[i];
  }
  for (int shift = 0; shift < key_bits; shift += 8) {
    if (((any_bits >> shift) & 0xffu) == 0) continue;  /* every key has digit 0 here */
    uint64_t hist[257];
    memset(hist, 0, sizeof hist);
    for (uint64_t i = 0; i < cnt; ++i) hist[((kcur[i] >> shift) & 0xffu) + 1]++;
    for (int b = 0; b < 256; ++b) hist[b + 1] += hist[b];
    for (uint64_t i = 0; i < cnt; ++i) {
      uint64_t pos = hist[(kcur[i] >> shift) & 0xffu]++;
      tmp[pos] = idx[i];
      ktmp[pos] = kcur[i];
    }
    memcpy(idx, tmp, sizeof(uint32_t) * cnt);
    memcpy(kcur, ktmp, sizeof(uint64_t) * cnt);
  }
  free(tmp);
  free(kcur);
  free(ktmp);
  return 0;
}

static int cmp_u32(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : x > y;
}

static void fisher_yates_u32(uint32_t *v, uint64_t len, uint64_t seed, uint32_t stream) {
  for (uint64_t i = len; i > 1; --i) {
    uint64_t j = os_bounded(os_rand_u64(seed, stream, i), i);
    uint32_t t = v[i - 1];
    v[i - 1] = v[j];
    v[j] = t;
  }
}

static void fisher_yates_u64(uint64_t *v, uint64_t len, uint64_t seed, uint32_t stream) {
  for (uint64_t i = len; i > 1; --i) {
    uint64_t j = os_bounded(os_rand_u64(seed, stream, i), i);
    uint64_t t = v[i - 1];
    v[i - 1] = v[j];
    v[j] = t;
  }
}

/* Returns 0 on success, -1 on bad arguments or when m unique edges could not
 * be drawn, -2 on allocation failure. edges_out: 2 m int32. */
int or_rmat_edges(int32_t n, int64_t m, double a, double b, double c, int32_t directed,
                  uint64_t seed, int32_t threads, int32_t *edges_out) {
  if (n < 2 || m < 0 || !edges_out || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
  int scale = 0;
  while ((1ll << scale) < n) ++scale;
  const double two32 = 4294967296.0;
  const uint64_t ta = (uint64_t)llround(a * two32), tab = (uint64_t)llround((a + b) * two32),
                 tabc = (uint64_t)llround((a + b + c) * two32);
  if (threads < 1) threads = 1;
  if (threads > 64) threads = 64;
  uint64_t want = (uint64_t)m + (uint64_t)m / 3 + 1024, have = 0;
  uint64_t *cand = NULL;
  uint32_t *uniq = NULL;
  uint64_t nuniq = 0;
  for (int attempt = 0; attempt < 12; ++attempt) {
    uint64_t *nc = (uint64_t *)realloc(cand, sizeof(uint64_t) * want);
    if (!nc) {
      free(cand);
      return -2;
    }
    cand = nc;
    pthread_t th[64];
    gen_job jobs[64];
    for (int t = 0; t < threads; ++t) {
      gen_job J = {cand, have, want, (uint64_t)threads, (uint64_t)t, n, scale, directed,
                   ta, tab, tabc, seed};
      jobs[t] = J;
      pthread_create(&th[t], NULL, gen_run, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    have = want;
    /* valid candidates in candidate order, then sorted by key (stably) */
    uint32_t *idx = (uint32_t *)malloc(sizeof(uint32_t) * have);
    if (!idx) {
      free(cand);
      return -2;
    }
    uint64_t cnt = 0;
    for (uint64_t i = 0; i < have; ++i)
      if (cand[i] != ~0ull) idx[cnt++] = (uint32_t)i;
    if (sort_by_key(cand, idx, cnt, 2 * 32) != 0) {
      free(idx);
      free(cand);
      return -2;
    }
    nuniq = 0;
    for (uint64_t k = 0; k < cnt; ++k)
      if (k == 0 || cand[idx[k]] != cand[idx[k - 1]]) idx[nuniq++] = idx[k];
    free(uniq);
    uniq = idx;
    if ((int64_t)nuniq >= m) break;
    want = want + want / 2;
  }
  if ((int64_t)nuniq < m) {
    free(uniq);
    free(cand);
    return -1;
  }
  qsort(uniq, nuniq, sizeof(uint32_t), cmp_u32);
  uint32_t *perm = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint64_t *edges = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(m ? m : 1));
  if (!perm || !edges) {
    free(perm);
    free(edges);
    free(uniq);
    free(cand);
    return -2;
  }
  for (int32_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
  fisher_yates_u32(perm, (uint64_t)n, seed, kStreamRelabel);
  for (int64_t e = 0; e < m; ++e) {
    uint64_t key = cand[uniq[e]];
    edges[e] = ((uint64_t)perm[key >> 32] << 32) | perm[key & 0xffffffffu];
  }
  fisher_yates_u64(edges, (uint64_t)m, seed, kStreamShuffle);
  for (int64_t e = 0; e < m; ++e) {
    edges_out[2 * e] = (int32_t)(edges[e] >> 32);
    edges_out[2 * e + 1] = (int32_t)(edges[e] & 0xffffffffu);
  }
  free(perm);
  free(edges);
  free(uniq);
  free(cand);
  return 0;
}

/* k distinct vertices drawn uniformly (partial Fisher-Yates, stream 4) from
 * those that appear in the m pairs, ascending. Returns 0, or -1. */
int or_sample_sources(int32_t n, const int32_t *edges, int64_t m, int32_t k, uint64_t seed,
                      int32_t *out) {
  if (n < 1 || k < 1 || !edges || !out || m < 0) return -1;
  uint8_t *seen = (uint8_t *)calloc((size_t)n, 1);
  if (!seen) return -1;
  for (int64_t e = 0; e < 2 * m; ++e) {
    if (edges[e] < 0 || edges[e] >= n) {
      free(seen);
      return -1;
    }
    seen[edges[e]] = 1;
  }
  uint32_t *pool = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint64_t np = 0;
  for (int32_t v = 0; v < n; ++v)
    if (seen[v]) pool[np++] = (uint32_t)v;
  free(seen);
  if ((int64_t)np < k) {
    free(pool);
    return -1;
  }
  for (int32_t i = 0; i < k; ++i) {
    uint64_t j = i + os_bounded(os_rand_u64(seed, kStreamSample, (uint64_t)i), np - i);
    uint32_t t = pool[i];
    pool[i] = pool[j];
    pool[j] = t;
  }
  qsort(pool, (size_t)k, sizeof(uint32_t), cmp_u32);
  for (int32_t i = 0; i < k; ++i) out[i] = (int32_t)pool[i];
  free(pool);
  return 0;
}

/* "u v" lines, one pair per line, final newline (the reference's delta-file
 * format). Returns 0, or -1 when the file cannot be written. */
int or_write_edges_text(const char *path, const int32_t *edges, int64_t m) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  char buf[1 << 16];
  size_t pos = 0;
  for (int64_t e = 0; e < m; ++e) {
    if (pos > sizeof buf - 32) {
      fwrite(buf, 1, pos, f);
      pos = 0;
    }
    pos += (size_t)snprintf(buf + pos, sizeof buf - pos, "%d %d\n", edges[2 * e], edges[2 * e + 1]);
  }
  fwrite(buf, 1, pos, f);
  return fclose(f) == 0 ? 0 : -1;
}
