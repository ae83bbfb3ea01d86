/*
 * CPU oracle — TEST INFRASTRUCTURE ONLY. Nothing in the product library links
 * or calls this file; tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it as the checker.
 *
 * A plain-C restatement of the reference's dense-path graph store, dynamic
 * PPR refresh and per-source FIFO forward push, keeping the reference's
 * visiting order and its float-state / double-arithmetic expression types so
 * that results are bit-identical to the reference code compiled from its own
 * sources (oracle/build_ref.sh builds that into oracle/_ref/).
 *
 *   graph insert ....... Code/Graph_dynamic.h:119-238 (Graph), :530-605 (UGraph)
 *   refresh ............ Code/ppr_computation_store_dynamic.h:2035-2121 (undirected),
 *                        :3811-3898 (directed out-lists), :4133-4228 (in-lists);
 *                        exact-division variant: :6500-6535 (sparse path)
 *   push ............... Code/ppr_computation_store_dynamic.h:1394-1498 (undirected),
 *                        :2945-3030 (directed), :3356-3437 (transpose)
 *   queue .............. Code/my_queue.h (FIFO; the reference never wraps within one push)
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared -pthread (see oracle/build_oracle.sh).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* The Gaussian test matrix is specified once (Philox4x32-10 + Box-Muller
 * with bit-reproducible float arithmetic) and shared with the device. */
#include "../tree-embedding_gb300/csrc/philox_gauss.h"

void or_gaussian_matrix(uint64_t seed, uint32_t stream, int64_t nrows, int32_t ncols,
                        double *out /* row-major nrows x ncols */) {
  for (int64_t i = 0; i < nrows; ++i)
    for (int32_t j = 0; j < ncols; ++j)
      out[i * ncols + j] = tsvd_gauss_entry(seed, stream, (uint32_t)i, (uint32_t)j);
}

/* ------------------------------------------------------------------ graph */
typedef struct {
  int32_t *v;
  int32_t len, cap;
} or_list;

typedef struct {
  int32_t n;
  int32_t directed;
  or_list *adj[2];        /* [0]: out-list (or the undirected list), [1]: in-list */
  int32_t *deg[2];
  int32_t *former[2];
  int64_t m;
} or_graph;

static int list_push(or_list *l, int32_t x) {
  if (l->len == l->cap) {
    int32_t nc = l->cap ? 2 * l->cap : 4;
    int32_t *nv = (int32_t *)realloc(l->v, (size_t)nc * sizeof(int32_t));
    if (!nv) return -1;
    l->v = nv;
    l->cap = nc;
  }
  l->v[l->len++] = x;
  return 0;
}

or_graph *or_graph_new(int32_t n, int32_t directed) {
  or_graph *g = (or_graph *)calloc(1, sizeof(or_graph));
  if (!g) return NULL;
  g->n = n;
  g->directed = directed;
  for (int d = 0; d < (directed ? 2 : 1); ++d) {
    g->adj[d] = (or_list *)calloc((size_t)n, sizeof(or_list));
    g->deg[d] = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    g->former[d] = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    if (!g->adj[d] || !g->deg[d] || !g->former[d]) return NULL;
  }
  return g;
}

void or_graph_free(or_graph *g) {
  if (!g) return;
  for (int d = 0; d < 2; ++d) {
    if (g->adj[d]) {
      for (int32_t i = 0; i < g->n; ++i) free(g->adj[d][i].v);
      free(g->adj[d]);
    }
    free(g->deg[d]);
    free(g->former[d]);
  }
  free(g);
}

/* Appends one delta file's edges in file order: former degrees are taken
 * first (Graph_dynamic.h:549-551), then each pair appends `to` to `from`'s
 * list and (undirected) `from` to `to`'s list (:590-596); directed graphs
 * append to the out-list of `from` and the in-list of `to` (:221-231). */
int or_graph_insert(or_graph *g, const int32_t *edges, int64_t m) {
  int nd = g->directed ? 2 : 1;
  for (int d = 0; d < nd; ++d) memcpy(g->former[d], g->deg[d], (size_t)g->n * 4);
  for (int64_t e = 0; e < m; ++e) {
    int32_t a = edges[2 * e], b = edges[2 * e + 1];
    if (a < 0 || b < 0 || a >= g->n || b >= g->n) return -2;
    if (list_push(&g->adj[0][a], b)) return -1;
    if (g->directed) {
      if (list_push(&g->adj[1][b], a)) return -1;
    } else {
      if (list_push(&g->adj[0][b], a)) return -1;
    }
    g->m++;
  }
  for (int d = 0; d < nd; ++d)
    for (int32_t i = 0; i < g->n; ++i) g->deg[d][i] = g->adj[d][i].len;
  return 0;
}

int or_graph_degrees(const or_graph *g, int32_t dir, int32_t *deg, int32_t *former) {
  if (dir < 0 || dir > 1 || !g->deg[dir]) return -1;
  if (deg) memcpy(deg, g->deg[dir], (size_t)g->n * 4);
  if (former) memcpy(former, g->former[dir], (size_t)g->n * 4);
  return 0;
}

/* CSR copy of the adjacency (insertion order); returns the entry count. */
int64_t or_graph_adjacency(const or_graph *g, int32_t dir, int64_t *offsets, int32_t *nbrs) {
  if (dir < 0 || dir > 1 || !g->adj[dir]) return -1;
  int64_t pos = 0;
  for (int32_t i = 0; i < g->n; ++i) {
    if (offsets) offsets[i] = pos;
    const or_list *l = &g->adj[dir][i];
    if (nbrs) memcpy(nbrs + pos, l->v, (size_t)l->len * 4);
    pos += l->len;
  }
  if (offsets) offsets[g->n] = pos;
  return pos;
}

/* -------------------------------------------------------------- PPR state */
typedef struct {
  int32_t n, s;
  int32_t *sources;
  float *r, *p;      /* |S| x N, row per source (the reference's float** rows) */
  uint8_t *flag;     /* |S| x N queued flags */
  int32_t **queue;   /* per-source FIFO storage */
  int64_t *qcap, *qhead, *qtail;
  int64_t pushes, edge_updates;
} or_ppr;

or_ppr *or_ppr_new(int32_t n, int32_t s, const int32_t *sources) {
  or_ppr *st = (or_ppr *)calloc(1, sizeof(or_ppr));
  if (!st) return NULL;
  st->n = n;
  st->s = s;
  size_t tot = (size_t)n * (size_t)s;
  st->sources = (int32_t *)malloc((size_t)s * 4);
  st->r = (float *)calloc(tot, sizeof(float));
  st->p = (float *)calloc(tot, sizeof(float));
  st->flag = (uint8_t *)calloc(tot, 1);
  st->queue = (int32_t **)calloc((size_t)s, sizeof(int32_t *));
  st->qcap = (int64_t *)calloc((size_t)s, 8);
  st->qhead = (int64_t *)calloc((size_t)s, 8);
  st->qtail = (int64_t *)calloc((size_t)s, 8);
  if (!st->sources || !st->r || !st->p || !st->flag || !st->queue || !st->qcap ||
      !st->qhead || !st->qtail)
    return NULL;
  memcpy(st->sources, sources, (size_t)s * 4);
  return st;
}

void or_ppr_free(or_ppr *st) {
  if (!st) return;
  for (int32_t k = 0; k < st->s; ++k) free(st->queue[k]);
  free(st->queue);
  free(st->qcap);
  free(st->qhead);
  free(st->qtail);
  free(st->sources);
  free(st->r);
  free(st->p);
  free(st->flag);
  free(st);
}

float *or_ppr_residue(or_ppr *st) { return st->r; }
float *or_ppr_reserve(or_ppr *st) { return st->p; }
int64_t or_ppr_pushes(or_ppr *st) { return st->pushes; }
int64_t or_ppr_edge_updates(or_ppr *st) { return st->edge_updates; }

static void q_push(or_ppr *st, int32_t k, int32_t v) {
  if (st->qtail[k] == st->qcap[k]) {
    int64_t nc = st->qcap[k] ? 2 * st->qcap[k] : 64;
    st->queue[k] = (int32_t *)realloc(st->queue[k], (size_t)nc * 4);
    st->qcap[k] = nc;
  }
  st->queue[k][st->qtail[k]++] = v;
}

typedef struct {
  or_ppr *st;
  const or_graph *g;
  int32_t dir, iter, dyn_start, intdiv;
  double alpha, rmax;
  int32_t k0, k1;
  int64_t pushes, edge_updates;
} or_job;

/* Refresh for sources [k0, k1): reference loop order i -> slot j -> source k. */
static void *refresh_job(void *arg) {
  or_job *J = (or_job *)arg;
  or_ppr *st = J->st;
  const or_graph *g = J->g;
  const int32_t n = st->n;
  const double alpha = J->alpha, rmax = J->rmax;
  if (J->iter < J->dyn_start) {
    for (int32_t k = J->k0; k < J->k1; ++k) {
      float *r = st->r + (size_t)k * n, *p = st->p + (size_t)k * n;
      uint8_t *fl = st->flag + (size_t)k * n;
      memset(r, 0, (size_t)n * 4);
      memset(p, 0, (size_t)n * 4);
      memset(fl, 0, (size_t)n);
      st->qhead[k] = st->qtail[k] = 0;
      int32_t src = st->sources[k];
      r[src] = 1;
      fl[src] = 1;
      q_push(st, k, src);
    }
    return NULL;
  }
  const or_list *adj = g->adj[J->dir];
  const int32_t *former = g->former[J->dir], *deg = g->deg[J->dir];
  for (int32_t i = 0; i < n; ++i) {
    for (int32_t j = former[i]; j < deg[i]; ++j) {
      int32_t to = adj[i].v[j];
      for (int32_t k = J->k0; k < J->k1; ++k) {
        float *r = st->r + (size_t)k * n, *p = st->p + (size_t)k * n;
        uint8_t *fl = st->flag + (size_t)k * n;
        if (j == 0) {
          /* First slot of a formerly dangling vertex: p(i) = 0, nothing to
           * rescale. The reference skips it (ppr:2086-2093), which leaves the
           * residue the vertex collected while dangling unpushed although it
           * can now push; the exact mode queues it like any other residue. */
          if (!J->intdiv && r[i] > rmax && !fl[i]) { q_push(st, k, i); fl[i] = 1; }
          continue;
        }
        if (J->intdiv) {
          p[i] *= (j + 1) / j;
          r[i] -= p[i] / (j + 1) / alpha;
          r[to] += (1 - alpha) * p[i] / (j + 1) / alpha;
        } else {
          p[i] *= (double)(j + 1.0) / (double)j;
          r[i] -= p[i] / (double)(j + 1.0) / alpha;
          r[to] += (1 - alpha) * p[i] / (double)(j + 1.0) / alpha;
        }
        if (r[i] > rmax && !fl[i]) { q_push(st, k, i); fl[i] = 1; }
        if (r[to] > rmax && !fl[to]) { q_push(st, k, to); fl[to] = 1; }
      }
    }
  }
  return NULL;
}

/* FIFO forward push per source with the "nodegree" threshold r(v) > rmax. */
static void *push_job(void *arg) {
  or_job *J = (or_job *)arg;
  or_ppr *st = J->st;
  const or_graph *g = J->g;
  const int32_t n = st->n;
  const double alpha = J->alpha, rmax = J->rmax;
  const int undirected = !g->directed;
  const or_list *adj = g->adj[J->dir];
  const int32_t *deg = g->deg[J->dir];
  int64_t pushes = 0, upd = 0;
  for (int32_t k = J->k0; k < J->k1; ++k) {
    float *r = st->r + (size_t)k * n, *p = st->p + (size_t)k * n;
    uint8_t *fl = st->flag + (size_t)k * n;
    int32_t src = st->sources[k];
    while (st->qhead[k] < st->qtail[k]) {
      int32_t v = st->queue[k][st->qhead[k]];
      if (deg[v] == 0) {
        fl[v] = 0;
        if (undirected) p[v] = alpha * r[v]; /* ppr:1433-1441 */
        st->qhead[k]++;
        continue;
      }
      if (r[v] > rmax) {
        const int32_t dv = deg[v];
        const int32_t *nb = adj[v].v;
        for (int32_t j = 0; j < dv; ++j) {
          int32_t u = nb[j];
          r[u] += (1 - alpha) * r[v] / dv;
          if (deg[u] == 0) {
            if (undirected) { /* ppr:1451-1455 (unreachable without isolated targets) */
              p[u] += alpha * r[u];
              r[src] += (1 - alpha) * r[u];
            }
            continue;
          }
          if (r[u] > rmax && !fl[u]) { q_push(st, k, u); fl[u] = 1; }
        }
        p[v] += alpha * r[v];
        r[v] = 0;
        pushes++;
        upd += dv;
      }
      fl[v] = 0;
      st->qhead[k]++;
    }
    st->qhead[k] = st->qtail[k] = 0;
  }
  J->pushes = pushes;
  J->edge_updates = upd;
  return NULL;
}

static void run_jobs(or_ppr *st, const or_graph *g, int32_t dir, int32_t iter,
                     int32_t dyn_start, int32_t intdiv, double alpha, double rmax,
                     int32_t nthreads, void *(*fn)(void *)) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > st->s) nthreads = st->s;
  or_job *jobs = (or_job *)calloc((size_t)nthreads, sizeof(or_job));
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  /* Source ranges as the drivers split them (Tree_u_NC.cpp:529-537). */
  int32_t per = st->s / nthreads;
  for (int32_t t = 0; t < nthreads; ++t) {
    or_job *J = &jobs[t];
    J->st = st; J->g = g; J->dir = dir; J->iter = iter; J->dyn_start = dyn_start;
    J->intdiv = intdiv; J->alpha = alpha; J->rmax = rmax;
    J->k0 = t * per;
    J->k1 = (t == nthreads - 1) ? st->s : (t + 1) * per;
    if (nthreads == 1) fn(J); else pthread_create(&th[t], NULL, fn, J);
  }
  if (nthreads > 1)
    for (int32_t t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  for (int32_t t = 0; t < nthreads; ++t) {
    st->pushes += jobs[t].pushes;
    st->edge_updates += jobs[t].edge_updates;
  }
  free(jobs);
  free(th);
}

void or_ppr_refresh(or_ppr *st, const or_graph *g, int32_t dir, int32_t iter,
                    int32_t dyn_start, double alpha, double rmax, int32_t intdiv,
                    int32_t nthreads) {
  run_jobs(st, g, dir, iter, dyn_start, intdiv, alpha, rmax, nthreads, refresh_job);
}

void or_ppr_push(or_ppr *st, const or_graph *g, int32_t dir, double alpha, double rmax,
                 int32_t nthreads) {
  st->pushes = 0;
  st->edge_updates = 0;
  run_jobs(st, g, dir, 0, 0, 0, alpha, rmax, nthreads, push_job);
}
