// Session: the per-snapshot refresh of Code/Tree_{u,d}_{NC,LP}.cpp
// (Tree_u_NC.cpp:507-866, Tree_d_NC.cpp:566-1140) on one GPU, plus the
// C-ABI entry points declared in include/tsvd.h.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "blocks.h"
#include "factor.h"
#include "internal.h"
#include "plain.h"
#include "ppr.h"

// ------------------------------------------------------------------ errors
namespace tsvd {
static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static thread_local char g_err[1024] = "";
tsvd_status fail(tsvd_status s, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return s;
}
}  // namespace tsvd

extern "C" const char *tsvd_last_error(void) { return tsvd::g_err; }
extern "C" const char *tsvd_status_string(tsvd_status s) {
  switch (s) {
    case TSVD_OK: return "ok";
    case TSVD_ERR_INVALID: return "invalid argument";
    case TSVD_ERR_OOM: return "out of memory";
    case TSVD_ERR_DEVICE: return "device error";
    case TSVD_ERR_TIMEOUT: return "timeout";
    case TSVD_ERR_STATE: return "bad state";
    case TSVD_ERR_IO: return "i/o error";
    case TSVD_ERR_NUMERIC: return "numeric error";
  }
  return "unknown";
}
extern "C" const char *tsvd_version(void) { return "tsvd-gb300 0.1 sm_103a"; }
extern "C" int64_t tsvd_launch_count(void) { return tsvd::g_launches.load(); }

using namespace tsvd;

// ------------------------------------------------------------------ session
struct tsvd_session {
  tsvd_config cfg{};
  std::vector<int32_t> sources;
  int n = 0, S = 0, sp = 0, nparts = 0, col_dim = 0, h = 0, d = 0, l = 0, q = 0;
  int directed = 0;
  cudaStream_t st = nullptr;
  Adjacency adj[2];
  InsertScratch ins;
  PprState ppr[2];
  uint8_t *vmark = nullptr;
  int32_t *sources_dev = nullptr;
  int32_t *colmap = nullptr, *ncols_dev = nullptr, *ncols_old_dev = nullptr;
  std::vector<int32_t> ncols_h, ncols_old_h;
  __half *atbuf[2] = {nullptr, nullptr};
  std::vector<int> atcur;
  __half **at_ptrs_dev = nullptr;  // [2][nparts]: old, new
  double *norm2_dev = nullptr, *diff2_dev = nullptr;
  unsigned long long *nnz_dev = nullptr, *stored_dev = nullptr;
  std::vector<double> norm2_h, diff2_h, norm2_acc, resid;
  std::vector<int64_t> nnz_h, stored_h;
  std::vector<uint8_t> dirty_h;
  std::vector<int> factor_now;
  int total_nodes = 0, leaf_start = 0;
  float *tree_b = nullptr, *tree_sigma = nullptr;
  float *embedding = nullptr;
  bool has_embedding = false;
  FrpcaWork fw;
  int32_t *edges_dev = nullptr;
  int64_t edges_cap = 0;
  uint32_t *keys = nullptr, *vals = nullptr;
  int64_t kv_cap = 0;
  int32_t *bad_dev = nullptr;
  int iter = 0;
  tsvd_step_stats last{};
  cudaEvent_t ev[8]{};
  // pipelined runs: the factor stage of snapshot k runs on st2 while the
  // graph insert, refresh and push of snapshot k+1 run on st
  cudaStream_t st2 = nullptr;
  cudaEvent_t pev[2][8]{};        // per snapshot (two in flight): [0..3] insert..log, [4..7] factor
  float *emb_stage = nullptr;     // pinned host copy of one embedding
  // LP right factor (cfg.lp_right_factor)
  float *lp_v = nullptr;          // [n][kLp]: row b*col_dim + c = V of block b's column c
  float *lp_u = nullptr;          // [nparts][S][d]: the root factor each V_b was made with
  std::vector<int> lp_iter;       // snapshot of each block's V_b (-1: never)
  int32_t *lp_valid_dev = nullptr;
  int32_t *colpos = nullptr;      // [n]: compacted column of a vertex in its block (-1: none)
  int32_t *src_row = nullptr;     // [n]: row of a source vertex in U (-1: not a source)
  int32_t *pairs_dev = nullptr;
  double *scores_dev = nullptr;
  int64_t pairs_cap = 0;
  // plain form (allocated on its first snapshot)
  int form = TSVD_FORM_MIXED;
  PlainPpr plain[2];
  PlainBlockWork pbw;
  // block-path autotuner and the sparse batch's CSR / CSC (mixed form)
  std::vector<PlainBlockWork> sbw;
  bool tuned = false;
  double tune_density = 0.0;
  cudaEvent_t tev[2]{};           // the autotuner's trial timings

  size_t node_elems() const { return (size_t)S * d; }
  float *node_b(int i) { return tree_b + (size_t)i * node_elems(); }
  float *node_sigma(int i) { return tree_sigma + (size_t)i * d; }
  __half *at_block(int which, int b) { return atbuf[which] + (size_t)b * col_dim * sp; }
};

namespace {

__global__ void expand_edges_kernel(const int32_t *__restrict__ e, int64_t m, int32_t n,
                                    int directed, uint32_t *__restrict__ k0,
                                    uint32_t *__restrict__ v0, uint32_t *__restrict__ k1,
                                    uint32_t *__restrict__ v1, int32_t *__restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t a = e[2 * i], b = e[2 * i + 1];
    if (a < 0 || b < 0 || a >= n || b >= n) {
      *bad = 1;
      a = 0;
      b = 0;
    }
    if (directed) {
      k0[i] = (uint32_t)a; v0[i] = (uint32_t)b;   // out-list of a
      k1[i] = (uint32_t)b; v1[i] = (uint32_t)a;   // in-list of b
    } else {
      k0[2 * i] = (uint32_t)a; v0[2 * i] = (uint32_t)b;
      k0[2 * i + 1] = (uint32_t)b; v0[2 * i + 1] = (uint32_t)a;
    }
  }
}

// One warp per (source i, vertex j) pair: U_b[row(i)] . V[j] in fp64, times
// the degree product when asked; invalid pairs set *bad.
__global__ void lp_score_kernel(const int32_t *__restrict__ pairs, int64_t m,
                                const int32_t *__restrict__ src_row,
                                const int32_t *__restrict__ colpos, int32_t n, int32_t col_dim,
                                int32_t nparts, const float *__restrict__ lp_v,
                                const float *__restrict__ lp_u, const int32_t *__restrict__ valid,
                                int d, int S, const int32_t *__restrict__ deg_i,
                                const int32_t *__restrict__ deg_j, int degree_scaled,
                                double *__restrict__ scores, int32_t *__restrict__ bad) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = gw; k < m; k += nw) {
    const int32_t i = pairs[2 * k], j = pairs[2 * k + 1];
    const int32_t row = (i >= 0 && i < n) ? src_row[i] : -1;
    if (row < 0 || j < 0 || j >= n) {
      if (lane == 0) {
        scores[k] = 0.0;
        *bad = 1;
      }
      continue;
    }
    const int32_t b = min(j / col_dim, nparts - 1);
    const int32_t c = colpos[j];
    double acc = 0.0;
    if (valid[b] && c >= 0) {
      const float *u = lp_u + ((size_t)b * S + row) * d;
      const float *v = lp_v + ((size_t)b * col_dim + c) * kLp;
      for (int t = lane; t < d; t += 32) acc += (double)u[t] * (double)v[t];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (degree_scaled) acc *= (double)deg_i[i] * (double)deg_j[j];
    if (lane == 0) scores[k] = acc;
  }
}

bool is_power_of(int n, int h) {
  if (h < 2) return false;
  while (n > 1 && n % h == 0) n /= h;
  return n == 1;
}

float ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace

extern "C" void tsvd_config_default(tsvd_config *c) {
  std::memset(c, 0, sizeof *c);
  c->alpha = 0.5;  // run.sh
  c->rmax = 1e-7;
  c->n_parts = 64;
  c->hierarchy_n = 2;
  c->rank_d = 128;
  c->oversample = 5;
  c->passes_q = 12;
  c->dynamic_ppr_start_iter = 100;
  c->lazy_update_start_iter = 100;
  c->delta = 0.3;
  c->transform = TSVD_TRANSFORM_LOG10_NC;
  c->dirty_rule = TSVD_DIRTY_REFERENCE;
  c->dirty_frac = 0.01;
  c->root_scaling = TSVD_ROOT_SQRT_SIGMA;
  c->refresh_mode = TSVD_REFRESH_EXACT;
  c->seed = 20231;
  c->device = 0;
  c->max_push_rounds = 0;
  c->push_levels = 1;
  c->push_ratio = 8.0;
  c->push_cofrac = 0.85;  // measured best on the 2.7M-vertex directed workload (0.5: +3.5 %)
}

static tsvd_status session_alloc(tsvd_session *s) {
  const tsvd_config &c = s->cfg;
  TSVD_CUDA(cudaSetDevice(c.device));
  // Launches are checked with cudaGetLastError: an error another component
  // left in that slot (a library's handled failure, the caller's own code)
  // must not be reported as ours.
  cudaGetLastError();
  // The factor stream of a pipelined run gets the lowest priority: its
  // blocks fill the SMs the insert and push leave idle instead of delaying
  // the insert's short dependent kernels.
  int prio_low = 0, prio_high = 0;
  TSVD_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  TSVD_CUDA(cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, prio_high));
  TSVD_CUDA(cudaStreamCreateWithPriority(&s->st2, cudaStreamNonBlocking, prio_low));
  for (auto &e : s->ev) TSVD_CUDA(cudaEventCreate(&e));
  for (auto &e : s->tev) TSVD_CUDA(cudaEventCreate(&e));
  for (auto &set : s->pev)
    for (auto &e : set) TSVD_CUDA(cudaEventCreate(&e));
  const int ndir = s->directed ? 2 : 1;
  for (int dd = 0; dd < ndir; ++dd) {
    Adjacency &A = s->adj[dd];
    A.n = s->n;
    TSVD_CUDA(cudaMalloc(&A.off, sizeof(int64_t) * (s->n + 1)));
    TSVD_CUDA(cudaMemset(A.off, 0, sizeof(int64_t) * (s->n + 1)));
    TSVD_CUDA(cudaMalloc(&A.deg, sizeof(int32_t) * s->n));
    TSVD_CUDA(cudaMemset(A.deg, 0, sizeof(int32_t) * s->n));
    TSVD_CUDA(cudaMalloc(&A.former, sizeof(int32_t) * s->n));
    TSVD_CUDA(cudaMemset(A.former, 0, sizeof(int32_t) * s->n));
    TSVD_TRY(ppr_alloc(s->ppr[dd], s->n, s->S, s->sp, c.ppr_host_reserve != 0));
  }
  TSVD_CUDA(cudaMalloc(&s->vmark, s->n));
  TSVD_CUDA(cudaMemset(s->vmark, 0, s->n));
  TSVD_CUDA(cudaMalloc(&s->sources_dev, sizeof(int32_t) * s->S));
  TSVD_CUDA(cudaMemcpy(s->sources_dev, s->sources.data(), sizeof(int32_t) * s->S,
                       cudaMemcpyHostToDevice));
  TSVD_CUDA(cudaMalloc(&s->colmap, sizeof(int32_t) * s->n));
  TSVD_CUDA(cudaMalloc(&s->ncols_dev, sizeof(int32_t) * s->nparts));
  TSVD_CUDA(cudaMalloc(&s->ncols_old_dev, sizeof(int32_t) * s->nparts));
  TSVD_CUDA(cudaMemset(s->ncols_dev, 0, sizeof(int32_t) * s->nparts));
  TSVD_CUDA(cudaMemset(s->ncols_old_dev, 0, sizeof(int32_t) * s->nparts));
  s->ncols_h.assign(s->nparts, 0);
  s->ncols_old_h.assign(s->nparts, 0);
  const size_t at_elems = (size_t)s->n * s->sp;
  // the last block is wider: col_dim*(nparts-1) + last = n, fits in n*sp
  for (int w = 0; w < 2; ++w) {
    TSVD_CUDA(cudaMalloc(&s->atbuf[w], at_elems * sizeof(__half)));
  }
  s->atcur.assign(s->nparts, 0);
  TSVD_CUDA(cudaMalloc(&s->at_ptrs_dev, sizeof(__half *) * 2 * s->nparts));
  TSVD_CUDA(cudaMalloc(&s->norm2_dev, sizeof(double) * s->nparts));
  TSVD_CUDA(cudaMalloc(&s->diff2_dev, sizeof(double) * s->nparts));
  TSVD_CUDA(cudaMalloc(&s->nnz_dev, sizeof(unsigned long long) * s->nparts));
  TSVD_CUDA(cudaMalloc(&s->stored_dev, sizeof(unsigned long long) * s->nparts));
  s->norm2_h.assign(s->nparts, 0);
  s->diff2_h.assign(s->nparts, 0);
  s->norm2_acc.assign(s->nparts, 0);
  s->resid.assign(s->nparts, 0);
  s->nnz_h.assign(s->nparts, 0);
  s->stored_h.assign(s->nparts, 0);
  s->dirty_h.assign(s->nparts, 0);
  // tree: complete h-ary tree with nparts leaves (ppr:225-245)
  int levels = 1;
  for (int t = s->nparts; t > 1; t /= s->h) ++levels;
  int64_t total = 0, pw = 1;
  for (int i = 0; i < levels; ++i, pw *= s->h) total += pw;
  s->total_nodes = (int)total;
  s->leaf_start = s->total_nodes - s->nparts;
  TSVD_CUDA(cudaMalloc(&s->tree_b, sizeof(float) * s->node_elems() * s->total_nodes));
  TSVD_CUDA(cudaMemset(s->tree_b, 0, sizeof(float) * s->node_elems() * s->total_nodes));
  TSVD_CUDA(cudaMalloc(&s->tree_sigma, sizeof(float) * s->d * s->total_nodes));
  TSVD_CUDA(cudaMemset(s->tree_sigma, 0, sizeof(float) * s->d * s->total_nodes));
  TSVD_CUDA(cudaMalloc(&s->embedding, sizeof(float) * s->node_elems()));
  TSVD_CUDA(cudaMemset(s->embedding, 0, sizeof(float) * s->node_elems()));
  TSVD_CUDA(cudaMallocHost(&s->emb_stage, sizeof(float) * s->node_elems()));
  TSVD_CUDA(cudaMalloc(&s->bad_dev, sizeof(int32_t)));
  if (c.lp_right_factor) {
    TSVD_CUDA(cudaMalloc(&s->lp_v, sizeof(float) * s->n * kLp));
    TSVD_CUDA(cudaMemset(s->lp_v, 0, sizeof(float) * s->n * kLp));
    TSVD_CUDA(cudaMalloc(&s->lp_u, sizeof(float) * s->node_elems() * s->nparts));
    TSVD_CUDA(cudaMemset(s->lp_u, 0, sizeof(float) * s->node_elems() * s->nparts));
    TSVD_CUDA(cudaMalloc(&s->lp_valid_dev, sizeof(int32_t) * s->nparts));
    TSVD_CUDA(cudaMemset(s->lp_valid_dev, 0, sizeof(int32_t) * s->nparts));
    s->lp_iter.assign(s->nparts, -1);
    TSVD_CUDA(cudaMalloc(&s->colpos, sizeof(int32_t) * s->n));
    TSVD_CUDA(cudaMemset(s->colpos, 0xFF, sizeof(int32_t) * s->n));
    std::vector<int32_t> rows(s->n, -1);
    for (int k = 0; k < s->S; ++k) rows[s->sources[k]] = k;
    TSVD_CUDA(cudaMalloc(&s->src_row, sizeof(int32_t) * s->n));
    TSVD_CUDA(cudaMemcpy(s->src_row, rows.data(), sizeof(int32_t) * s->n, cudaMemcpyHostToDevice));
  }
  const int last_w = s->n - (s->nparts - 1) * s->col_dim;
  TSVD_TRY(frpca_work_alloc(s->fw, s->nparts, std::max(last_w, s->col_dim), s->sp, s->l, s->d));
  return TSVD_OK;
}

static void session_release(tsvd_session *s) {
  if (!s) return;
  cudaSetDevice(s->cfg.device);
  if (s->st) cudaStreamSynchronize(s->st);
  if (s->st2) cudaStreamSynchronize(s->st2);
  for (int dd = 0; dd < 2; ++dd) {
    adjacency_free(s->adj[dd]);
    if (s->ppr[dd].r) ppr_free(s->ppr[dd]);
  }
  cudaFree(s->ins.buf);
  cudaFree(s->vmark); cudaFree(s->sources_dev); cudaFree(s->colmap);
  cudaFree(s->ncols_dev); cudaFree(s->ncols_old_dev);
  cudaFree(s->atbuf[0]); cudaFree(s->atbuf[1]); cudaFree(s->at_ptrs_dev);
  cudaFree(s->norm2_dev); cudaFree(s->diff2_dev); cudaFree(s->nnz_dev); cudaFree(s->stored_dev);
  cudaFree(s->tree_b); cudaFree(s->tree_sigma); cudaFree(s->embedding);
  cudaFree(s->edges_dev); cudaFree(s->keys); cudaFree(s->vals); cudaFree(s->bad_dev);
  cudaFree(s->lp_v); cudaFree(s->lp_u); cudaFree(s->lp_valid_dev); cudaFree(s->colpos);
  cudaFree(s->src_row); cudaFree(s->pairs_dev); cudaFree(s->scores_dev);
  frpca_work_free(s->fw);
  for (int dd = 0; dd < 2; ++dd)
    if (s->plain[dd].cbits) plain_free(s->plain[dd]);
  plain_block_free(s->pbw);
  for (auto &w : s->sbw) plain_block_free(w);
  cudaFreeHost(s->emb_stage);
  for (auto &e : s->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : s->tev)
    if (e) cudaEventDestroy(e);
  for (auto &set : s->pev)
    for (auto &e : set)
      if (e) cudaEventDestroy(e);
  if (s->st) cudaStreamDestroy(s->st);
  if (s->st2) cudaStreamDestroy(s->st2);
  cudaGetLastError();  // nothing from teardown may surface in a later launch check
}

extern "C" tsvd_status tsvd_session_create(const tsvd_config *cfg, tsvd_session **out) {
  if (!cfg || !out) return fail(TSVD_ERR_INVALID, "null argument");
  *out = nullptr;
  const tsvd_config &c = *cfg;
  if (c.n_vertices < 2 || c.n_sources < 1 || !c.sources)
    return fail(TSVD_ERR_INVALID, "need n_vertices >= 2 and at least one source");
  if (!(c.alpha > 0 && c.alpha < 1) || !(c.rmax > 0))
    return fail(TSVD_ERR_INVALID, "alpha must be in (0,1) and rmax > 0");
  if (c.n_parts < 1 || c.n_parts > c.n_vertices)
    return fail(TSVD_ERR_INVALID, "n_parts=%d", c.n_parts);
  if (c.hierarchy_n < 2 || !is_power_of(c.n_parts, c.hierarchy_n) || c.n_parts < c.hierarchy_n)
    return fail(TSVD_ERR_INVALID,
                "n_parts (%d) must be a power of hierarchy_n (%d), at least one merge",
                c.n_parts, c.hierarchy_n);
  if (c.rank_d < 1 || c.oversample < 0 || c.rank_d + c.oversample > kLp)
    return fail(TSVD_ERR_INVALID, "rank_d + oversample must be <= %d", kLp);
  if (c.hierarchy_n > 16 || (int64_t)c.hierarchy_n * c.rank_d > 2048)
    return fail(TSVD_ERR_INVALID, "need hierarchy_n <= 16 and hierarchy_n * rank_d <= 2048");
  if (c.passes_q < 1) return fail(TSVD_ERR_INVALID, "passes_q must be >= 1");
  if (c.transform < 0 || c.transform > 2 || c.dirty_rule < 0 || c.dirty_rule > 2)
    return fail(TSVD_ERR_INVALID, "bad transform or dirty rule");
  if (c.form != TSVD_FORM_MIXED && c.form != TSVD_FORM_PLAIN)
    return fail(TSVD_ERR_INVALID, "form must be TSVD_FORM_MIXED or TSVD_FORM_PLAIN");
  if (c.block_path < TSVD_BLOCKS_DENSE || c.block_path > TSVD_BLOCKS_AUTO)
    return fail(TSVD_ERR_INVALID, "block_path must be one of TSVD_BLOCKS_*");
  if (c.lp_right_factor && c.root_scaling != TSVD_ROOT_U)
    return fail(TSVD_ERR_INVALID, "lp_right_factor needs root_scaling TSVD_ROOT_U (LP drivers)");
  std::vector<int32_t> src(c.sources, c.sources + c.n_sources);
  {
    std::vector<int32_t> chk = src;
    std::sort(chk.begin(), chk.end());
    for (size_t i = 0; i < chk.size(); ++i) {
      if (chk[i] < 0 || chk[i] >= c.n_vertices)
        return fail(TSVD_ERR_INVALID, "source %d out of range", chk[i]);
      if (i && chk[i] == chk[i - 1]) return fail(TSVD_ERR_INVALID, "duplicate source %d", chk[i]);
    }
  }
  tsvd_session *s = new tsvd_session;
  s->cfg = c;
  s->cfg.sources = nullptr;
  s->sources = src;
  s->n = c.n_vertices;
  s->S = c.n_sources;
  s->sp = (int)round_up(s->S, kRowPad);
  s->nparts = c.n_parts;
  s->col_dim = c.n_vertices / c.n_parts;
  s->h = c.hierarchy_n;
  s->d = c.rank_d;
  s->l = c.rank_d + c.oversample;
  s->q = c.passes_q;
  s->directed = c.directed ? 1 : 0;
  s->form = c.form;
  tsvd_status st = session_alloc(s);
  if (st != TSVD_OK) {
    std::string msg = tsvd_last_error();
    session_release(s);
    delete s;
    return fail(st, "%s", msg.c_str());
  }
  *out = s;
  return TSVD_OK;
}

// Device bytes a session with this configuration holds once expected_edges
// pairs are inserted (the allocations of session_alloc, ppr_alloc and
// frpca_work_alloc; the adjacency with its 50 % slack; one insert's sort
// buffers). Used by the serving layer to admit tenants by HBM footprint.
extern "C" tsvd_status tsvd_session_footprint(const tsvd_config *c, int64_t expected_edges,
                                              int64_t *bytes) {
  if (!c || !bytes || c->n_vertices < 1 || c->n_sources < 1 || c->n_parts < 1 ||
      expected_edges < 0)
    return fail(TSVD_ERR_INVALID, "footprint: bad arguments");
  const double n = c->n_vertices, sp = (double)round_up(c->n_sources, kRowPad);
  const double S = c->n_sources, d = c->rank_d, P = c->n_parts;
  const double chunks = sp / 64.0, dirs = c->directed ? 2 : 1;
  const double entries = (c->directed ? 1.0 : 2.0) * expected_edges;  // per direction list
  double b = 0;
  b += dirs * (8 * (n + 1) + 8 * n + 1.5 * 4 * entries);            // adjacency
  b += 16.0 * expected_edges / 8 + 16.0 * entries;                     // insert staging, sort
  const double state = 4 * n * sp;
  b += dirs * (state * (c->ppr_host_reserve ? 1 : 2));                 // r (+ p)
  b += dirs * (2 * n * chunks / 8 + 2 * 8 * n * chunks + 4 * n);       // bitsets, frontiers
  b += dirs * ((1 << 20) * 64 * 4.0 + (1 << 20) * 8.0 + (1 << 22) * 8.0);  // hub units
  b += 2 * 2 * n * sp + 13 * n;                                         // A^T blocks, maps
  int levels = 1;
  for (int t = c->n_parts; t > 1 && c->hierarchy_n > 1; t /= c->hierarchy_n) ++levels;
  double nodes = 0, pw = 1;
  for (int i = 0; i < levels; ++i, pw *= c->hierarchy_n) nodes += pw;
  b += nodes * S * d * 4 + nodes * d * 4 + S * d * 4;                   // tree factors
  const double rows_max = n - (P - 1) * std::floor(n / P) + 1;
  b += P * rows_max * kLp * 8 + P * sp * 256 * 4;                      // X hi/lo, Z
  b += P * sp * kLp * 8 + P * 65536 * (8 + 4 + 24) + P * 2048 * 4;     // Y, Q, G, V, refine
  b += (std::min(P * std::ceil(std::max(rows_max, sp) / 128), 2048.0) + P) * 65536 * 8;  // Grams
  b += P * 30.0 * 255 * 128 * 8;                                        // Jacobi rotation logs
  if (c->lp_right_factor) b += n * kLp * 4 + P * S * d * 4 + 8 * n;
  *bytes = (int64_t)(b * 1.05) + (64ll << 20);
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_destroy(tsvd_session *s) {
  if (!s) return TSVD_OK;
  session_release(s);
  delete s;
  return TSVD_OK;
}

// ------------------------------------------------------------------ stages
static PprParams ppr_params(const tsvd_session *s) {
  PprParams p;
  p.alpha = s->cfg.alpha;
  p.rmax = s->cfg.rmax;
  p.intdiv = s->cfg.refresh_mode == TSVD_REFRESH_INTDIV;
  p.undirected = !s->directed;
  p.max_rounds = s->cfg.max_push_rounds > 0 ? s->cfg.max_push_rounds : 1000000;
  p.levels = std::max(1, s->cfg.push_levels);
  p.ratio = s->cfg.push_ratio > 1.0 ? s->cfg.push_ratio : 8.0;
  p.cofrac = s->cfg.push_cofrac;
  p.hub_degree = std::max(0, s->cfg.push_hub_degree);
  return p;
}

static tsvd_status insert_device(tsvd_session *s, const int32_t *edges_dev, int64_t m) {
  const int64_t entries = s->directed ? m : 2 * m;
  if (entries > s->kv_cap) {
    cudaFree(s->keys);
    cudaFree(s->vals);
    s->keys = s->vals = nullptr;
    s->kv_cap = 0;
    int64_t cap = std::max<int64_t>(entries, 1024);
    // directed keeps both lists: [0, m) out, [cap, cap+m) in
    TSVD_CUDA(cudaMalloc(&s->keys, sizeof(uint32_t) * cap * 2));
    TSVD_CUDA(cudaMalloc(&s->vals, sizeof(uint32_t) * cap * 2));
    s->kv_cap = cap;
  }
  TSVD_CUDA(cudaMemsetAsync(s->bad_dev, 0, sizeof(int32_t), s->st));
  if (m > 0) {
    expand_edges_kernel<<<grid_for(m, 256), 256, 0, s->st>>>(
        edges_dev, m, s->n, s->directed, s->keys, s->vals, s->keys + s->kv_cap,
        s->vals + s->kv_cap, s->bad_dev);
    TSVD_LAUNCH_CHECK();
  }
  int32_t bad = 0;
  TSVD_CUDA(cudaMemcpyAsync(&bad, s->bad_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  if (bad) return fail(TSVD_ERR_INVALID, "edge endpoint outside [0, %d)", s->n);
  TSVD_TRY(adjacency_append(s->adj[0], s->keys, s->vals, entries, s->ins, s->st));
  if (s->directed)
    TSVD_TRY(adjacency_append(s->adj[1], s->keys + s->kv_cap, s->vals + s->kv_cap, m, s->ins,
                              s->st));
  s->last.edges_inserted = m;
  return TSVD_OK;
}

// Column map, log transform and block norms of the converged PPR state
// (launch and read-back; the dirty decision is materialize_decide).
static tsvd_status materialize_launch(tsvd_session *s) {
  const int P = s->nparts;
  TSVD_TRY(colmap_update(s->vmark, s->colmap, s->colpos, s->ncols_dev, s->n, s->col_dim, P, s->st));
  TSVD_CUDA(cudaMemcpyAsync(s->ncols_h.data(), s->ncols_dev, sizeof(int32_t) * P,
                            cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  std::vector<__half *> ptrs(2 * P);
  for (int b = 0; b < P; ++b) {
    ptrs[b] = s->at_block(s->atcur[b], b);
    ptrs[P + b] = s->at_block(1 - s->atcur[b], b);
  }
  TSVD_CUDA(cudaMemcpyAsync(s->at_ptrs_dev, ptrs.data(), sizeof(__half *) * 2 * P,
                            cudaMemcpyHostToDevice, s->st));
  MaterializeArgs a;
  a.p1 = s->ppr[0].p;
  a.p2 = s->directed ? s->ppr[1].p : nullptr;
  a.colmap = s->colmap;
  a.ncols = s->ncols_dev;
  a.ncols_old = s->ncols_old_dev;
  a.at_old = s->at_ptrs_dev;
  a.at_new = s->at_ptrs_dev + P;
  a.n = s->n;
  a.sp = s->sp;
  a.nsrc = s->S;
  a.col_dim = s->col_dim;
  a.transform = s->cfg.transform;
  a.rmin_f = (float)s->cfg.rmax;
  a.inv_rmin_f = (float)(1.0 / s->cfg.rmax);
  a.n_f = (float)s->n;
  a.norm2 = s->norm2_dev;
  a.diff2 = s->diff2_dev;
  a.nnz = s->nnz_dev;
  a.stored = s->stored_dev;
  int32_t max_nc = 0;
  for (int32_t x : s->ncols_h) max_nc = std::max(max_nc, x);
  TSVD_CUDA(cudaEventRecord(s->ev[6], s->st));
  TSVD_TRY(materialize_blocks(a, P, max_nc, s->st));
  TSVD_CUDA(cudaEventRecord(s->ev[7], s->st));
  std::vector<unsigned long long> nn(P), ss(P);
  TSVD_CUDA(cudaMemcpyAsync(s->norm2_h.data(), s->norm2_dev, sizeof(double) * P, cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaMemcpyAsync(s->diff2_h.data(), s->diff2_dev, sizeof(double) * P, cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaMemcpyAsync(nn.data(), s->nnz_dev, sizeof(unsigned long long) * P, cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaMemcpyAsync(ss.data(), s->stored_dev, sizeof(unsigned long long) * P, cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  s->last.ms_materialize_kernel = ms_between(s->ev[6], s->ev[7]);
  for (int b = 0; b < P; ++b) {
    s->nnz_h[b] = (int64_t)nn[b];
    s->stored_h[b] = (int64_t)ss[b];
  }
  return TSVD_OK;
}
// Lazy-update decision (ppr:2700-2729) or unconditional refresh
// (Tree_u_NC.cpp:642-668). The reference rule reads the residuals of the
// previous factorization, so a pipelined run calls this only after the
// previous snapshot's factor stage has finished.
static tsvd_status materialize_decide(tsvd_session *s, int iter) {
  const int P = s->nparts;
  const bool with_norm = iter >= s->cfg.lazy_update_start_iter;
  s->factor_now.clear();
  int ndirty = 0;
  for (int b = 0; b < P; ++b) {
    bool dirty = true;
    if (with_norm) {
      const double a_norm = std::sqrt(std::max(s->norm2_h[b], 0.0));
      const double ei = std::sqrt(std::max(s->diff2_h[b], 0.0));
      switch (s->cfg.dirty_rule) {
        case TSVD_DIRTY_REFERENCE:
          dirty = !(s->resid[b] + ei < s->cfg.delta * std::sqrt(2.0) * a_norm);
          break;
        case TSVD_DIRTY_FROBENIUS:
          dirty = ei > s->cfg.dirty_frac * a_norm;
          break;
        default:
          dirty = true;
      }
    }
    s->dirty_h[b] = dirty ? 1 : 0;
    if (!dirty) continue;
    ++ndirty;
    // accept: the new matrix becomes the reference for the next comparison
    s->atcur[b] = 1 - s->atcur[b];
    s->ncols_old_h[b] = s->ncols_h[b];
    s->norm2_acc[b] = s->norm2_h[b];
    if (s->stored_h[b] > 0) s->factor_now.push_back(b);  // nonZeros() == 0 blocks are skipped
  }
  TSVD_CUDA(cudaMemcpyAsync(s->ncols_old_dev, s->ncols_old_h.data(), sizeof(int32_t) * P,
                            cudaMemcpyHostToDevice, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  s->last.dirty_blocks = ndirty;
  return TSVD_OK;
}

static tsvd_status stage_materialize(tsvd_session *s, int iter) {
  TSVD_TRY(materialize_launch(s));
  return materialize_decide(s, iter);
}

// What the factor stage of one snapshot needs from the host-side block
// state, copied when the snapshot's dirty decision is made: a pipelined run
// changes that state for the next snapshot while this one is factorized.
struct FactorJob {
  int iter = 0;
  std::vector<int> factor_now;     // dirty blocks with stored entries
  std::vector<int> atcur;          // accepted buffer of every block
  std::vector<int32_t> ncols;      // compacted columns of every block
  std::vector<uint8_t> dirty;
  std::vector<double> norm2_acc;   // ||A_b||^2 of the accepted matrices
  tsvd_step_stats stats{};
};

static void make_job(const tsvd_session *s, int iter, FactorJob &job) {
  job.iter = iter;
  job.factor_now = s->factor_now;
  job.atcur = s->atcur;
  job.ncols = s->ncols_h;
  job.dirty = s->dirty_h;
  job.norm2_acc = s->norm2_acc;
  job.stats = s->last;
}

// The sparse path of the mixed form: block b's accepted half-precision A^T
// compressed into CSR / CSC (the tensor-core path's values, exactly).
static BlockSource at_source(const tsvd_session *s, const FactorJob &job, int b) {
  BlockSource src;
  src.at = const_cast<tsvd_session *>(s)->at_block(job.atcur[b], b);
  src.colmap = s->colmap + (size_t)b * s->col_dim;
  src.ncols = job.ncols[b];
  src.n = s->n;
  src.sp = s->sp;
  src.nsrc = s->S;
  return src;
}

// Block-path autotuner (TSVD_BLOCKS_AUTO), run at the first factorization:
// up to three dirty blocks spanning the density range are factorized alone
// through both paths, timed with events (the faster of two runs each). Dense cost is modelled per stored
// cell (Sp x n_c: every pass streams the half-precision A^T), sparse cost per
// non-zero (the SpMM gathers) plus per stored cell (the CSR / CSC build reads
// the block once per pass of the build); the crossover density follows.
static tsvd_status tune_block_paths(tsvd_session *s, const FactorJob &job,
                                    const std::vector<FrpcaProblem> &probs, cudaStream_t st) {
  const int nf = (int)job.factor_now.size();
  std::vector<int> order(nf);
  std::vector<double> dens(nf);
  for (int i = 0; i < nf; ++i) {
    const int b = job.factor_now[i];
    order[i] = i;
    dens[i] = (double)s->nnz_h[b] / std::max(1.0, (double)s->S * job.ncols[b]);
  }
  std::sort(order.begin(), order.end(), [&](int a, int b) { return dens[a] > dens[b]; });
  std::vector<int> pick;
  for (int q : {0, nf / 2, nf - 1})
    if (std::find(pick.begin(), pick.end(), order[q]) == pick.end()) pick.push_back(order[q]);
  cudaEvent_t e0 = s->tev[0], e1 = s->tev[1];
  double sd = 0, sc = 0;                      // dense: time over cells
  double a11 = 0, a12 = 0, a22 = 0, r1 = 0, r2 = 0;  // sparse: least squares in (nnz, cells)
  if (s->sbw.empty()) s->sbw.resize(1);
  for (int i : pick) {
    const int b = job.factor_now[i];
    FrpcaProblem P = probs[i];
    P.b_out = nullptr;  // a trial: results dropped
    P.sigma_out = nullptr;
    const double cells = (double)s->sp * job.ncols[b], nnz = (double)s->nnz_h[b];
    double ss = 0;
    // each path runs twice and the faster run counts: the first call of a
    // path pays one-time set-up (kernel attributes, the tensor-map encoder's
    // lookup) that would bias the choice against it
    double td = 1e30, ts = 1e30;
    for (int rep = 0; rep < 2; ++rep) {
      P.sparse = nullptr;
      TSVD_CUDA(cudaEventRecord(e0, st));
      TSVD_TRY(frpca_batch(s->fw, &P, 1, s->q, s->cfg.seed, s->S, st, &ss));
      TSVD_CUDA(cudaEventRecord(e1, st));
      TSVD_CUDA(cudaEventSynchronize(e1));
      td = std::min(td, (double)ms_between(e0, e1));
      TSVD_CUDA(cudaEventRecord(e0, st));
      TSVD_TRY(plain_block_build(s->sbw[0], at_source(s, job, b), s->nnz_h[b], st));
      P.sparse = &s->sbw[0].blk;
      TSVD_TRY(frpca_batch(s->fw, &P, 1, s->q, s->cfg.seed, s->S, st, &ss));
      TSVD_CUDA(cudaEventRecord(e1, st));
      TSVD_CUDA(cudaEventSynchronize(e1));
      ts = std::min(ts, (double)ms_between(e0, e1));
    }
    sd += td;
    sc += cells;
    a11 += nnz * nnz; a12 += nnz * cells; a22 += cells * cells;
    r1 += nnz * ts; r2 += cells * ts;
  }
  const double cd = sd / std::max(sc, 1.0);
  double c1, c2;
  const double det = a11 * a22 - a12 * a12;
  if (pick.size() >= 2 && std::fabs(det) > 1e-12 * a11 * a22) {
    c1 = (r1 * a22 - r2 * a12) / det;
    c2 = (a11 * r2 - a12 * r1) / det;
  } else {
    c1 = r1 / std::max(a11, 1.0);  // one point: all of it per non-zero
    c2 = 0;
  }
  c1 = std::max(c1, 1e-30);
  c2 = std::max(c2, 0.0);
  // sparse is cheaper while c1 rho S + c2 < cd (per stored cell, rho S / Sp ~ rho)
  s->tune_density = std::max(0.0, (cd - c2) / c1) * ((double)s->sp / s->S);
  s->tuned = true;
  return TSVD_OK;
}

// Mixed form with TSVD_BLOCKS_SPARSE / TSVD_BLOCKS_AUTO: one batch of dense
// blocks on the tensor cores and one batch of sparse blocks through SpMM.
// Factorizes the dirty blocks with those below density `threshold` (or all,
// for TSVD_BLOCKS_SPARSE) through SpMM and the rest on the tensor cores.
static tsvd_status factorize_split(tsvd_session *s, FactorJob &job,
                                   std::vector<FrpcaProblem> &probs, std::vector<double> &ssum,
                                   double threshold, cudaStream_t st, int *nsparse) {
  const int nf = (int)job.factor_now.size();
  std::vector<int> di, si;
  for (int i = 0; i < nf; ++i) {
    const int b = job.factor_now[i];
    const double rho = (double)s->nnz_h[b] / std::max(1.0, (double)s->S * job.ncols[b]);
    const bool sparse = s->cfg.block_path == TSVD_BLOCKS_SPARSE || rho < threshold;
    (sparse ? si : di).push_back(i);
  }
  if (!di.empty()) {
    std::vector<FrpcaProblem> pd;
    for (int i : di) pd.push_back(probs[i]);
    std::vector<double> sd(di.size());
    TSVD_TRY(frpca_batch(s->fw, pd.data(), (int)pd.size(), s->q, s->cfg.seed, s->S, st, sd.data()));
    for (size_t k = 0; k < di.size(); ++k) ssum[di[k]] = sd[k];
  }
  if (!si.empty()) {
    if (s->sbw.size() < si.size()) s->sbw.resize(si.size());
    std::vector<FrpcaProblem> ps;
    for (size_t k = 0; k < si.size(); ++k) {
      const int b = job.factor_now[si[k]];
      TSVD_TRY(plain_block_build(s->sbw[k], at_source(s, job, b), s->nnz_h[b], st));
      FrpcaProblem P = probs[si[k]];
      P.sparse = &s->sbw[k].blk;
      ps.push_back(P);
    }
    std::vector<double> sv(si.size());
    TSVD_TRY(frpca_batch(s->fw, ps.data(), (int)ps.size(), s->q, s->cfg.seed, s->S, st, sv.data()));
    for (size_t k = 0; k < si.size(); ++k) ssum[si[k]] = sv[k];
  }
  *nsparse = (int)si.size();
  return TSVD_OK;
}

// Mixed form with TSVD_BLOCKS_SPARSE / TSVD_BLOCKS_AUTO: one batch of dense
// blocks on the tensor cores and one batch of sparse blocks through SpMM.
// The single-block trials of the autotuner see the tensor-core path at a
// fraction of the GPU, while the real batch fills it; so at the first
// factorization the split they suggest is timed against the whole batch on
// the tensor cores, and the faster of the two is kept.
static tsvd_status factorize_two_paths(tsvd_session *s, FactorJob &job,
                                       std::vector<FrpcaProblem> &probs,
                                       std::vector<double> &ssum, cudaStream_t st) {
  int nsparse = 0;
  if (s->cfg.block_path == TSVD_BLOCKS_AUTO && !s->tuned) {
    TSVD_TRY(tune_block_paths(s, job, probs, st));
    if (s->tune_density > 0) {
      cudaEvent_t e0 = s->tev[0], e1 = s->tev[1];
      TSVD_CUDA(cudaEventRecord(e0, st));
      TSVD_TRY(factorize_split(s, job, probs, ssum, s->tune_density, st, &nsparse));
      TSVD_CUDA(cudaEventRecord(e1, st));
      TSVD_CUDA(cudaEventSynchronize(e1));
      const double t_split = ms_between(e0, e1);
      if (nsparse > 0) {
        TSVD_CUDA(cudaEventRecord(e0, st));
        TSVD_TRY(factorize_split(s, job, probs, ssum, 0.0, st, &nsparse));
        TSVD_CUDA(cudaEventRecord(e1, st));
        TSVD_CUDA(cudaEventSynchronize(e1));
        const double t_dense = ms_between(e0, e1);
        if (t_dense <= t_split) {
          s->tune_density = 0.0;  // this batch (now factorized) stays on the tensor cores
        } else {
          TSVD_TRY(factorize_split(s, job, probs, ssum, s->tune_density, st, &nsparse));
        }
      }
      job.stats.sparse_blocks = nsparse;
      job.stats.tune_density = s->tune_density;
      return TSVD_OK;
    }
  }
  TSVD_TRY(factorize_split(s, job, probs, ssum, s->tune_density, st, &nsparse));
  job.stats.sparse_blocks = nsparse;
  job.stats.tune_density = s->tune_density;
  return TSVD_OK;
}

static tsvd_status stage_factorize(tsvd_session *s, FactorJob &job, cudaStream_t st) {
  const int nf = (int)job.factor_now.size();
  job.stats.factorized_blocks = nf;
  if (nf == 0) return TSVD_OK;
  std::vector<FrpcaProblem> probs(nf);
  for (int i = 0; i < nf; ++i) {
    int b = job.factor_now[i];
    FrpcaProblem &P = probs[i];
    P.block = b;
    P.at = s->at_block(job.atcur[b], b);
    P.ncols = job.ncols[b];
    P.colmap = s->colmap + (size_t)b * s->col_dim;
    P.col_base = b * s->col_dim;
    P.b_out = s->node_b(s->leaf_start + b);
    P.sigma_out = s->node_sigma(s->leaf_start + b);
    P.u_out = nullptr;
    P.v_out = nullptr;
  }
  std::vector<double> ssum(nf);
  if (s->form == TSVD_FORM_PLAIN) {
    // every dirty block on its own: FP32 CSR / CSC from the reserve, then
    // frPCA with SpMM products
    for (int i = 0; i < nf; ++i) {
      const int b = job.factor_now[i];
      BlockSource src;
      src.p1 = s->ppr[0].p;
      src.p2 = s->directed ? s->ppr[1].p : nullptr;
      src.colmap = s->colmap + (size_t)b * s->col_dim;
      src.ncols = job.ncols[b];
      src.n = s->n;
      src.sp = s->sp;
      src.nsrc = s->S;
      src.transform = s->cfg.transform;
      src.rmin_f = (float)s->cfg.rmax;
      src.inv_rmin_f = (float)(1.0 / s->cfg.rmax);
      src.n_f = (float)s->n;
      TSVD_TRY(plain_block_build(s->pbw, src, s->nnz_h[b], st));
      probs[i].sparse = &s->pbw.blk;
      TSVD_TRY(frpca_batch(s->fw, &probs[i], 1, s->q, s->cfg.seed, s->S, st, &ssum[i]));
      job.stats.eig_refine_sweeps = std::max(job.stats.eig_refine_sweeps, s->fw.last_refine_sweeps);
    }
  } else if (s->cfg.block_path == TSVD_BLOCKS_DENSE) {
    TSVD_TRY(frpca_batch(s->fw, probs.data(), nf, s->q, s->cfg.seed, s->S, st, ssum.data()));
  } else {
    TSVD_TRY(factorize_two_paths(s, job, probs, ssum, st));
  }
  job.stats.eig_sweeps_frpca = s->fw.last_sweeps;
  job.stats.eig_refine_sweeps = std::max(job.stats.eig_refine_sweeps, s->fw.last_refine_sweeps);
  // Residual ||A - U S V^T||_F = sqrt(||A||^2 - sum sigma^2) for an orthonormal
  // basis (the reference forms the dense product, Tree_u_NC.cpp:158-204).
  if (job.iter >= s->cfg.lazy_update_start_iter - 1)
    for (int i = 0; i < nf; ++i) {
      int b = job.factor_now[i];
      s->resid[b] = std::sqrt(std::max(job.norm2_acc[b] - ssum[i], 0.0));
    }
  return TSVD_OK;
}

static tsvd_status stage_merge(tsvd_session *s, FactorJob &job, cudaStream_t st) {
  job.stats.merged_nodes = 0;
  if (job.factor_now.empty()) return TSVD_OK;
  const int h = s->h;
  std::vector<int> level;
  for (int b : job.factor_now) {
    int par = (s->leaf_start + b - 1) / h;
    if (std::find(level.begin(), level.end(), par) == level.end()) level.push_back(par);
  }
  std::sort(level.begin(), level.end());
  while (!level.empty()) {
    const bool root = level.size() == 1 && level[0] == 0;
    std::vector<MergeProblem> probs(level.size());
    for (size_t i = 0; i < level.size(); ++i) {
      int p = level[i];
      for (int c = 0; c < h; ++c) probs[i].children[c] = s->node_b(p * h + 1 + c);
      probs[i].out = root ? s->embedding : s->node_b(p);
      probs[i].sigma_out = s->node_sigma(p);
    }
    int mode = 0;
    if (root) mode = s->cfg.root_scaling == TSVD_ROOT_U ? 2 : 1;
    if (s->form == TSVD_FORM_PLAIN) {
      for (auto &pr : probs) TSVD_TRY(merge_batch(s->fw, &pr, 1, h, s->S, mode, st));
    } else {
      TSVD_TRY(merge_batch(s->fw, probs.data(), (int)probs.size(), h, s->S, mode, st));
    }
    job.stats.eig_sweeps_merge = std::max(job.stats.eig_sweeps_merge, s->fw.last_sweeps);
    job.stats.merge_subspace_iters = std::max(job.stats.merge_subspace_iters, s->fw.wide_iters);
    job.stats.eig_refine_sweeps = std::max(job.stats.eig_refine_sweeps, s->fw.last_refine_sweeps);
    job.stats.merged_nodes += (int)probs.size();
    if (root) {
      TSVD_CUDA(cudaMemcpyAsync(s->node_b(0), s->embedding, sizeof(float) * s->node_elems(),
                                cudaMemcpyDeviceToDevice, st));
      s->has_embedding = true;
      break;
    }
    std::vector<int> next;
    for (int p : level) {
      int par = (p - 1) / h;
      if (std::find(next.begin(), next.end(), par) == next.end()) next.push_back(par);
    }
    std::sort(next.begin(), next.end());
    level.swap(next);
  }
  TSVD_CUDA(cudaStreamSynchronize(st));
  return TSVD_OK;
}

// LP right factor of the blocks refreshed in this snapshot (Tree_u_LP.cpp:
// 1024-1044: the blocks whose update record is this iteration), with this
// snapshot's root factor U, which is kept beside them for scoring.
static tsvd_status stage_lp(tsvd_session *s, const FactorJob &job, cudaStream_t st) {
  if (!s->cfg.lp_right_factor || !s->has_embedding) return TSVD_OK;
  std::vector<LpProblem> probs;
  std::vector<int> blocks;
  for (int b = 0; b < s->nparts; ++b) {
    if (!job.dirty[b]) continue;
    LpProblem p;
    p.at = s->at_block(job.atcur[b], b);
    p.ncols = job.ncols[b];
    p.v_out = s->lp_v + (size_t)b * s->col_dim * kLp;
    probs.push_back(p);
    blocks.push_back(b);
  }
  if (probs.empty()) return TSVD_OK;
  TSVD_TRY(lp_right_batch(s->fw, probs.data(), (int)probs.size(), s->embedding, s->S, s->d, st));
  std::vector<int32_t> valid(s->nparts);
  for (int b : blocks) {
    TSVD_CUDA(cudaMemcpyAsync(s->lp_u + (size_t)b * s->node_elems(), s->embedding,
                              sizeof(float) * s->node_elems(), cudaMemcpyDeviceToDevice, st));
    s->lp_iter[b] = job.iter;
  }
  for (int b = 0; b < s->nparts; ++b) valid[b] = s->lp_iter[b] >= 0;
  TSVD_CUDA(cudaMemcpyAsync(s->lp_valid_dev, valid.data(), sizeof(int32_t) * s->nparts,
                            cudaMemcpyHostToDevice, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  return TSVD_OK;
}

// Refresh + push of one PPR state (the reverse one of a directed graph with
// dir = 1). Running the two directions on two streams, round-interleaved, was
// measured no faster: both are DRAM-bound through most of their rounds.
static tsvd_status stage_ppr(tsvd_session *s, int iter, int dir) {
  const bool scratch = iter < s->cfg.dynamic_ppr_start_iter;
  PprParams prm = ppr_params(s);
  PushStats ps;
  if (s->form == TSVD_FORM_PLAIN) {
    if (!s->plain[dir].cbits)
      TSVD_TRY(plain_alloc(s->plain[dir], s->n, s->sp, s->cfg.plain_frontier_cap));
    TSVD_TRY(plain_refresh(s->plain[dir], s->ppr[dir], s->adj[dir], s->sources_dev, scratch, prm,
                           s->st));
    TSVD_TRY(plain_push(s->plain[dir], s->ppr[dir], s->adj[dir], prm, s->vmark, s->st, &ps));
  } else {
    TSVD_TRY(ppr_refresh(s->ppr[dir], s->adj[dir], s->sources_dev, scratch, prm, s->vmark, s->st));
    TSVD_TRY(ppr_push(s->ppr[dir], s->adj[dir], prm, s->vmark, s->st, &ps));
  }
  s->last.push_rounds += ps.rounds;
  s->last.pushes += ps.pushes;
  s->last.push_edge_updates += ps.edge_updates;
  s->last.push_items += ps.items;
  s->last.ms_push_kernels += ps.kernel_ms;
  s->last.push_item_edges += ps.item_edges;
  return TSVD_OK;
}

static tsvd_status stage_edges_to_device(tsvd_session *s, const int32_t *edges, int64_t m);

// Graph insert (after the copy of host edges, when on_device is false),
// refresh + push and materialization of one snapshot on the main stream;
// ea[0..3] mark its stage boundaries. after_insert (optional) runs once the
// insert is issued. Snapshots before lazy_update_start_iter - 1 only grow the
// graph (Tree_u_NC.cpp:516): they return with *skipped set.
static tsvd_status stage_front(tsvd_session *s, const int32_t *edges, bool on_device, int64_t m,
                               cudaEvent_t *ea, bool *skipped,
                               const std::function<tsvd_status()> &after_insert = nullptr) {
  const int iter = ++s->iter;
  std::memset(&s->last, 0, sizeof s->last);
  s->last.iter = iter;
  *skipped = false;
  TSVD_CUDA(cudaEventRecord(ea[0], s->st));
  if (!on_device) {
    TSVD_TRY(stage_edges_to_device(s, edges, m));
    edges = s->edges_dev;
  }
  TSVD_TRY(insert_device(s, edges, m));
  TSVD_CUDA(cudaEventRecord(ea[1], s->st));
  if (after_insert) TSVD_TRY(after_insert());
  if (s->cfg.lazy_update_start_iter != 100 && iter < s->cfg.lazy_update_start_iter - 1) {
    s->last.skipped = 1;
    TSVD_CUDA(cudaStreamSynchronize(s->st));
    s->last.ms_insert = s->last.ms_total = ms_between(ea[0], ea[1]);
    *skipped = true;
    return TSVD_OK;
  }
  TSVD_TRY(stage_ppr(s, iter, 0));
  if (s->directed) TSVD_TRY(stage_ppr(s, iter, 1));
  TSVD_CUDA(cudaEventRecord(ea[2], s->st));
  TSVD_TRY(materialize_launch(s));
  TSVD_CUDA(cudaEventRecord(ea[3], s->st));
  return TSVD_OK;
}

// Factorization, merge and LP right factor of one snapshot on stream st,
// then (when out is given) the read-back of its embedding, widened to double
// (|S| x d; zeros before the first embedding). eb[0..3] mark the stage
// boundaries. Returns with st drained.
static tsvd_status stage_back(tsvd_session *s, FactorJob &job, cudaStream_t st, cudaEvent_t *eb,
                              double *out) {
  TSVD_CUDA(cudaEventRecord(eb[0], st));
  TSVD_TRY(stage_factorize(s, job, st));
  TSVD_CUDA(cudaEventRecord(eb[1], st));
  TSVD_TRY(stage_merge(s, job, st));
  TSVD_CUDA(cudaEventRecord(eb[2], st));
  if (s->cfg.lp_right_factor) TSVD_TRY(stage_lp(s, job, st));
  const size_t E = s->node_elems();
  if (out && s->has_embedding)
    TSVD_CUDA(cudaMemcpyAsync(s->emb_stage, s->embedding, sizeof(float) * E,
                              cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaEventRecord(eb[3], st));
  TSVD_CUDA(cudaEventSynchronize(eb[3]));
  if (out) {
    if (s->has_embedding)
      for (size_t i = 0; i < E; ++i) out[i] = s->emb_stage[i];
    else
      std::fill(out, out + E, 0.0);
  }
  return TSVD_OK;
}

// Stage times of a finished snapshot. ms_total is its latency: from the
// start of its graph insert to the end of its factor stage.
static void finish_stats(tsvd_step_stats &st, cudaEvent_t *ea, cudaEvent_t *eb) {
  st.ms_insert = ms_between(ea[0], ea[1]);
  st.ms_push = ms_between(ea[1], ea[2]);
  st.ms_log = ms_between(ea[2], ea[3]);
  st.ms_frpca = ms_between(eb[0], eb[1]);
  st.ms_merge = ms_between(eb[1], eb[2]);
  st.ms_lp = ms_between(eb[2], eb[3]);
  st.ms_total = ms_between(ea[0], eb[3]);
}

static tsvd_status step_device(tsvd_session *s, const int32_t *edges, bool on_device, int64_t m) {
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  cudaGetLastError();  // not ours: see session_alloc
  bool skipped = false;
  TSVD_TRY(stage_front(s, edges, on_device, m, s->ev, &skipped));
  if (skipped) return TSVD_OK;
  TSVD_TRY(materialize_decide(s, s->iter));
  FactorJob job;
  make_job(s, s->iter, job);
  TSVD_TRY(stage_back(s, job, s->st, s->ev + 4, nullptr));
  finish_stats(job.stats, s->ev, s->ev + 4);
  s->last = job.stats;
  return TSVD_OK;
}

// The current embedding, widened to double, into out (|S| x d); zeros before
// the first one. Drains st.
static tsvd_status embedding_to_host(tsvd_session *s, cudaStream_t st, double *out) {
  const size_t E = s->node_elems();
  if (!s->has_embedding) {
    std::fill(out, out + E, 0.0);
    return TSVD_OK;
  }
  TSVD_CUDA(cudaMemcpyAsync(s->emb_stage, s->embedding, sizeof(float) * E, cudaMemcpyDeviceToHost, st));
  TSVD_CUDA(cudaStreamSynchronize(st));
  for (size_t i = 0; i < E; ++i) out[i] = s->emb_stage[i];
  return TSVD_OK;
}

static tsvd_status reserve_edges(tsvd_session *s, int64_t m) {
  if (m > s->edges_cap) {
    cudaFree(s->edges_dev);
    s->edges_dev = nullptr;
    s->edges_cap = 0;
    int64_t cap = std::max<int64_t>(m, 1024);
    TSVD_CUDA(cudaMalloc(&s->edges_dev, sizeof(int32_t) * 2 * cap));
    s->edges_cap = cap;
  }
  return TSVD_OK;
}

static tsvd_status stage_edges_to_device(tsvd_session *s, const int32_t *edges, int64_t m) {
  TSVD_TRY(reserve_edges(s, m));
  if (m > 0)
    TSVD_CUDA(cudaMemcpyAsync(s->edges_dev, edges, sizeof(int32_t) * 2 * m, cudaMemcpyHostToDevice,
                              s->st));
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_step(tsvd_session *s, const int32_t *edges, int64_t m) {
  if (!s || (m > 0 && !edges) || m < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  return step_device(s, edges, false, m);
}

extern "C" tsvd_status tsvd_session_step_device(tsvd_session *s, const int32_t *edges_dev,
                                                int64_t m) {
  if (!s || (m > 0 && !edges_dev) || m < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  return step_device(s, edges_dev, true, m);
}

// Snapshots [0, count): snapshot k's edges are the pairs [offsets[k],
// offsets[k+1]) of `edges` (device memory when on_device). The factor stage
// of snapshot k (frPCA, merge, LP right factor) runs on a worker thread and
// the low-priority second stream, started once the insert of snapshot k+1 is
// issued (the insert's short dependent kernels run on an idle GPU), while
// this thread refreshes, pushes and materializes snapshot k+1. The two
// overlap without sharing buffers: the materialization of k+1 writes only
// the candidate block buffers, which the factor stage of k does not read,
// and the dirty decision of k+1 (which reads the residuals of k) waits for
// the factor stage of k. A failing snapshot still lets the factor stage of
// the one before it finish, so the session stays consistent.
static tsvd_status run_snapshots(tsvd_session *s, const int32_t *edges, bool on_device,
                                 const int64_t *offsets, int32_t count, double *emb_out,
                                 tsvd_step_stats *stats_out) {
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  cudaGetLastError();  // not ours: see session_alloc
  if (s->form == TSVD_FORM_PLAIN)
    return fail(TSVD_ERR_INVALID,
                "the plain form reads the reserve in its factor stage: one snapshot per call");
  int64_t max_m = 0;
  for (int k = 0; k < count; ++k) {
    const int64_t m = offsets[k + 1] - offsets[k];
    if (m < 0 || offsets[k] < 0) return fail(TSVD_ERR_INVALID, "offsets must not decrease");
    max_m = std::max(max_m, m);
  }
  if (max_m > 0 && !edges) return fail(TSVD_ERR_INVALID, "null edges");
  if (!on_device) TSVD_TRY(reserve_edges(s, max_m));  // no reallocation while the worker runs
  const size_t E = s->node_elems();
  FactorJob jobs[2];
  std::thread worker;
  tsvd_status wst = TSVD_OK;
  std::string wmsg;
  int prepared = -1;  // snapshot whose factor job is built but not started
  int pending = -1;   // snapshot whose factor job is running
  auto launch = [&]() -> tsvd_status {
    if (prepared < 0) return TSVD_OK;
    const int k = prepared;
    prepared = -1;
    cudaEvent_t *ea = s->pev[k & 1];
    if (cudaStreamWaitEvent(s->st2, ea[3], 0) != cudaSuccess)
      return fail(TSVD_ERR_DEVICE, "cudaStreamWaitEvent failed");
    FactorJob *job = &jobs[k & 1];
    double *out = emb_out ? emb_out + k * E : nullptr;
    wst = TSVD_OK;
    try {
      worker = std::thread([s, job, &wst, &wmsg, ea, out]() {
        tsvd_status r = cudaSetDevice(s->cfg.device) == cudaSuccess
                            ? TSVD_OK
                            : fail(TSVD_ERR_DEVICE, "cudaSetDevice failed on the factor thread");
        if (r == TSVD_OK) r = stage_back(s, *job, s->st2, ea + 4, out);
        if (r != TSVD_OK) wmsg = tsvd_last_error();
        wst = r;
      });
    } catch (...) {
      return fail(TSVD_ERR_STATE, "could not start the factor thread");
    }
    pending = k;
    return TSVD_OK;
  };
  auto join = [&]() -> tsvd_status {
    if (worker.joinable()) worker.join();
    if (pending < 0) return TSVD_OK;
    const int k = pending;
    pending = -1;
    if (wst != TSVD_OK) return fail(wst, "%s", wmsg.c_str());
    FactorJob &job = jobs[k & 1];
    finish_stats(job.stats, s->pev[k & 1], s->pev[k & 1] + 4);
    s->last = job.stats;
    if (stats_out) stats_out[k] = job.stats;
    return TSVD_OK;
  };
  tsvd_status st = TSVD_OK;
  for (int k = 0; k < count; ++k) {
    const int64_t m = offsets[k + 1] - offsets[k];
    const int32_t *e = edges ? edges + 2 * offsets[k] : nullptr;
    cudaEvent_t *ea = s->pev[k & 1];
    bool skipped = false;
    if ((st = stage_front(s, e, on_device, m, ea, &skipped, launch)) != TSVD_OK) break;
    const tsvd_step_stats front = s->last;
    if ((st = join()) != TSVD_OK) break;  // the factor stage of snapshot k - 1
    s->last = front;
    if (skipped) {
      if (stats_out) stats_out[k] = s->last;
      if (emb_out && (st = embedding_to_host(s, s->st, emb_out + k * E)) != TSVD_OK) break;
      continue;
    }
    if ((st = materialize_decide(s, s->iter)) != TSVD_OK) break;
    make_job(s, s->iter, jobs[k & 1]);
    prepared = k;
  }
  // the last prepared job (also after a failure: its blocks are accepted)
  tsvd_status ls = launch();
  if (ls != TSVD_OK && st == TSVD_OK) st = ls;
  const tsvd_status js = join();
  return st != TSVD_OK ? st : js;
}

extern "C" tsvd_status tsvd_session_run(tsvd_session *s, const int32_t *edges,
                                        const int64_t *offsets, int32_t count, double *embeddings,
                                        tsvd_step_stats *stats) {
  if (!s || !offsets || count < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  return run_snapshots(s, edges, false, offsets, count, embeddings, stats);
}

extern "C" tsvd_status tsvd_session_run_device(tsvd_session *s, const int32_t *edges_dev,
                                               const int64_t *offsets, int32_t count,
                                               double *embeddings, tsvd_step_stats *stats) {
  if (!s || !offsets || count < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  return run_snapshots(s, edges_dev, true, offsets, count, embeddings, stats);
}

extern "C" tsvd_status tsvd_session_embedding(tsvd_session *s, double *out) {
  if (!s || !out) return fail(TSVD_ERR_INVALID, "null argument");
  if (!s->has_embedding) return fail(TSVD_ERR_STATE, "no embedding yet");
  std::vector<float> tmp(s->node_elems());
  TSVD_CUDA(cudaMemcpyAsync(tmp.data(), s->embedding, sizeof(float) * tmp.size(),
                            cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_embedding_device(tsvd_session *s, const float **out) {
  if (!s || !out) return fail(TSVD_ERR_INVALID, "null argument");
  if (!s->has_embedding) return fail(TSVD_ERR_STATE, "no embedding yet");
  *out = s->embedding;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_set_form(tsvd_session *s, int32_t form) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  if (form != TSVD_FORM_MIXED && form != TSVD_FORM_PLAIN)
    return fail(TSVD_ERR_INVALID, "form must be TSVD_FORM_MIXED or TSVD_FORM_PLAIN");
  s->form = form;
  s->cfg.form = form;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_stream(tsvd_session *s, void **stream) {
  if (!s || !stream) return fail(TSVD_ERR_INVALID, "null argument");
  *stream = (void *)s->st;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_session_last_stats(tsvd_session *s, tsvd_step_stats *out) {
  if (!s || !out) return fail(TSVD_ERR_INVALID, "null argument");
  *out = s->last;
  return TSVD_OK;
}

// ------------------------------------------------------------------ granular API
extern "C" tsvd_status tsvd_graph_insert(tsvd_session *s, const int32_t *edges, int64_t m) {
  if (!s || (m > 0 && !edges) || m < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  TSVD_TRY(stage_edges_to_device(s, edges, m));
  return insert_device(s, s->edges_dev, m);
}

extern "C" tsvd_status tsvd_ppr_refresh(tsvd_session *s, int32_t iter, int32_t transpose) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  if (transpose && !s->directed) return fail(TSVD_ERR_INVALID, "transpose on undirected graph");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  PprParams prm = ppr_params(s);
  const int dir = transpose ? 1 : 0;
  const bool scratch = iter < s->cfg.dynamic_ppr_start_iter;
  if (s->form == TSVD_FORM_PLAIN) {
    if (!s->plain[dir].cbits)
      TSVD_TRY(plain_alloc(s->plain[dir], s->n, s->sp, s->cfg.plain_frontier_cap));
    return plain_refresh(s->plain[dir], s->ppr[dir], s->adj[dir], s->sources_dev, scratch, prm,
                         s->st);
  }
  return ppr_refresh(s->ppr[dir], s->adj[dir], s->sources_dev, scratch, prm, s->vmark, s->st);
}

extern "C" tsvd_status tsvd_ppr_push(tsvd_session *s, int32_t transpose) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  if (transpose && !s->directed) return fail(TSVD_ERR_INVALID, "transpose on undirected graph");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  PprParams prm = ppr_params(s);
  const int dir = transpose ? 1 : 0;
  PushStats ps;
  if (s->form == TSVD_FORM_PLAIN) {
    if (!s->plain[dir].cbits) return fail(TSVD_ERR_STATE, "push before refresh");
    TSVD_TRY(plain_push(s->plain[dir], s->ppr[dir], s->adj[dir], prm, s->vmark, s->st, &ps));
  } else {
    TSVD_TRY(ppr_push(s->ppr[dir], s->adj[dir], prm, s->vmark, s->st, &ps));
  }
  s->last.push_rounds += ps.rounds;
  s->last.pushes += ps.pushes;
  s->last.push_edge_updates += ps.edge_updates;
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_blocks_materialize(tsvd_session *s, int32_t iter, uint8_t *dirty) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  s->iter = iter;
  TSVD_TRY(stage_materialize(s, iter));
  if (dirty) std::memcpy(dirty, s->dirty_h.data(), s->nparts);
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_blocks_factorize(tsvd_session *s, int32_t iter) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  FactorJob job;
  make_job(s, iter, job);
  TSVD_TRY(stage_factorize(s, job, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  s->last.factorized_blocks = job.stats.factorized_blocks;
  s->last.eig_sweeps_frpca = job.stats.eig_sweeps_frpca;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_tree_merge(tsvd_session *s) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  FactorJob job;
  make_job(s, s->iter, job);
  TSVD_TRY(stage_merge(s, job, s->st));
  s->last.merged_nodes = job.stats.merged_nodes;
  s->last.eig_sweeps_merge = job.stats.eig_sweeps_merge;
  return TSVD_OK;
}

// ------------------------------------------------------------------ inspection
extern "C" tsvd_status tsvd_graph_degrees(tsvd_session *s, int32_t dir, int32_t *deg,
                                          int32_t *former) {
  if (!s || dir < 0 || dir > (s->directed ? 1 : 0)) return fail(TSVD_ERR_INVALID, "bad dir");
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  if (deg) TSVD_CUDA(cudaMemcpy(deg, s->adj[dir].deg, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost));
  if (former)
    TSVD_CUDA(cudaMemcpy(former, s->adj[dir].former, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost));
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_graph_adjacency(tsvd_session *s, int32_t dir, int64_t *offsets,
                                            int32_t *nbrs, int64_t cap) {
  if (!s || dir < 0 || dir > (s->directed ? 1 : 0)) return fail(TSVD_ERR_INVALID, "bad dir");
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  const Adjacency &A = s->adj[dir];
  std::vector<int32_t> deg(s->n);
  std::vector<int64_t> off(s->n + 1);
  TSVD_CUDA(cudaMemcpy(deg.data(), A.deg, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost));
  TSVD_CUDA(cudaMemcpy(off.data(), A.off, sizeof(int64_t) * (s->n + 1), cudaMemcpyDeviceToHost));
  std::vector<int32_t> all((size_t)std::max<int64_t>(A.cap_total, 1));
  if (A.cap_total > 0)
    TSVD_CUDA(cudaMemcpy(all.data(), A.nbr, sizeof(int32_t) * A.cap_total, cudaMemcpyDeviceToHost));
  int64_t pos = 0;
  for (int v = 0; v < s->n; ++v) {
    if (offsets) offsets[v] = pos;
    if (nbrs) {
      if (pos + deg[v] > cap) return fail(TSVD_ERR_INVALID, "adjacency buffer too small");
      std::memcpy(nbrs + pos, all.data() + off[v], sizeof(int32_t) * deg[v]);
    }
    pos += deg[v];
  }
  if (offsets) offsets[s->n] = pos;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_ppr_state(tsvd_session *s, int32_t transpose, int32_t which,
                                      float *out) {
  if (!s || !out || (transpose && !s->directed)) return fail(TSVD_ERR_INVALID, "bad arguments");
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  const PprState &P = s->ppr[transpose ? 1 : 0];
  std::vector<float> tmp((size_t)s->n * s->sp);
  TSVD_CUDA(cudaMemcpy(tmp.data(), which ? P.p : P.r, sizeof(float) * tmp.size(),
                       cudaMemcpyDefault));  // p may be mapped host memory
  for (int v = 0; v < s->n; ++v)
    for (int k = 0; k < s->S; ++k) out[(size_t)k * s->n + v] = tmp[ppr_cell(v, k, s->n)];
  return TSVD_OK;
}

namespace {
// out[i][v] = state cell (v, rows[i]) for the listed source rows
__global__ void gather_rows_kernel(const float *__restrict__ x, const int32_t *__restrict__ rows,
                                   int32_t count, int32_t n, float *__restrict__ out) {
  const int64_t total = (int64_t)count * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = (int32_t)(i / n), v = (int32_t)(i % n);
    out[i] = x[ppr_cell(v, rows[k], n)];
  }
}
}  // namespace

extern "C" tsvd_status tsvd_ppr_state_rows(tsvd_session *s, int32_t transpose, int32_t which,
                                           const int32_t *rows, int32_t count, float *out) {
  if (!s || !out || !rows || count < 1 || (transpose && !s->directed))
    return fail(TSVD_ERR_INVALID, "bad arguments");
  for (int32_t i = 0; i < count; ++i)
    if (rows[i] < 0 || rows[i] >= s->S) return fail(TSVD_ERR_INVALID, "row %d out of range", rows[i]);
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  const PprState &P = s->ppr[transpose ? 1 : 0];
  int32_t *drows = nullptr;
  float *dout = nullptr;
  TSVD_CUDA(cudaMalloc(&drows, sizeof(int32_t) * count));
  if (cudaMalloc(&dout, sizeof(float) * (size_t)count * s->n) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(drows);
    return fail(TSVD_ERR_OOM, "ppr_state_rows: %d rows", count);
  }
  tsvd_status st = TSVD_OK;
  if (cudaMemcpyAsync(drows, rows, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s->st) !=
      cudaSuccess)
    st = fail(TSVD_ERR_DEVICE, "ppr_state_rows: copy");
  if (st == TSVD_OK) {
    gather_rows_kernel<<<grid_for((int64_t)count * s->n, 256), 256, 0, s->st>>>(
        which ? P.p : P.r, drows, count, s->n, dout);
    count_launch();
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)count * s->n, cudaMemcpyDeviceToHost,
                        s->st) != cudaSuccess ||
        cudaStreamSynchronize(s->st) != cudaSuccess)
      st = fail(TSVD_ERR_DEVICE, "ppr_state_rows: gather");
  }
  cudaFree(drows);
  cudaFree(dout);
  return st;
}

extern "C" tsvd_status tsvd_block_info(tsvd_session *s, double *norm_a, double *norm_diff,
                                       double *resid, int64_t *nnz, uint8_t *dirty) {
  if (!s) return fail(TSVD_ERR_INVALID, "null session");
  for (int b = 0; b < s->nparts; ++b) {
    if (norm_a) norm_a[b] = std::sqrt(std::max(s->norm2_h[b], 0.0));
    if (norm_diff) norm_diff[b] = std::sqrt(std::max(s->diff2_h[b], 0.0));
    if (resid) resid[b] = s->resid[b];
    if (nnz) nnz[b] = s->nnz_h[b];
    if (dirty) dirty[b] = s->dirty_h[b];
  }
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_tree_factor(tsvd_session *s, int32_t node, double *out,
                                        double *sigma) {
  if (!s || node < 0 || node >= s->total_nodes) return fail(TSVD_ERR_INVALID, "bad node");
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  if (out) {
    std::vector<float> tmp(s->node_elems());
    TSVD_CUDA(cudaMemcpy(tmp.data(), s->node_b(node), sizeof(float) * tmp.size(),
                         cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
  }
  if (sigma) {
    std::vector<float> tmp(s->d);
    TSVD_CUDA(cudaMemcpy(tmp.data(), s->node_sigma(node), sizeof(float) * s->d,
                         cudaMemcpyDeviceToHost));
    for (int i = 0; i < s->d; ++i) sigma[i] = tmp[i];
  }
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_block_dense(tsvd_session *s, int32_t b, float *out) {
  if (!s || !out || b < 0 || b >= s->nparts) return fail(TSVD_ERR_INVALID, "bad block");
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  const int nb = b == s->nparts - 1 ? s->n - (s->nparts - 1) * s->col_dim : s->col_dim;
  const int nc = s->ncols_old_h[b];
  std::vector<__half> at((size_t)std::max(nc, 1) * s->sp);
  std::vector<int32_t> cm(std::max(nc, 1));
  if (nc > 0) {
    TSVD_CUDA(cudaMemcpy(at.data(), s->at_block(s->atcur[b], b), sizeof(__half) * nc * s->sp,
                         cudaMemcpyDeviceToHost));
    TSVD_CUDA(cudaMemcpy(cm.data(), s->colmap + (size_t)b * s->col_dim, sizeof(int32_t) * nc,
                         cudaMemcpyDeviceToHost));
  }
  std::memset(out, 0, sizeof(float) * (size_t)s->S * nb);
  for (int c = 0; c < nc; ++c) {
    int col = cm[c] - b * s->col_dim;
    for (int k = 0; k < s->S; ++k)
      out[(size_t)k * nb + col] = __half2float(at[(size_t)c * s->sp + k]);
  }
  return TSVD_OK;
}

// ------------------------------------------------------------------ link prediction
extern "C" tsvd_status tsvd_lp_right_factor(tsvd_session *s, float *v_out) {
  if (!s || !v_out) return fail(TSVD_ERR_INVALID, "null argument");
  if (!s->cfg.lp_right_factor) return fail(TSVD_ERR_STATE, "session built without lp_right_factor");
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  std::memset(v_out, 0, sizeof(float) * (size_t)s->n * s->d);
  std::vector<float> v;
  std::vector<int32_t> cm;
  for (int b = 0; b < s->nparts; ++b) {
    const int nc = s->ncols_h[b];
    if (s->lp_iter[b] < 0 || nc == 0) continue;
    v.resize((size_t)nc * kLp);
    cm.resize(nc);
    TSVD_CUDA(cudaMemcpy(v.data(), s->lp_v + (size_t)b * s->col_dim * kLp,
                         sizeof(float) * v.size(), cudaMemcpyDeviceToHost));
    TSVD_CUDA(cudaMemcpy(cm.data(), s->colmap + (size_t)b * s->col_dim, sizeof(int32_t) * nc,
                         cudaMemcpyDeviceToHost));
    for (int c = 0; c < nc; ++c)
      std::memcpy(v_out + (size_t)cm[c] * s->d, v.data() + (size_t)c * kLp, sizeof(float) * s->d);
  }
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_lp_scores(tsvd_session *s, const int32_t *pairs, int64_t m,
                                      int32_t degree_scaled, double *scores) {
  if (!s || (m > 0 && (!pairs || !scores)) || m < 0) return fail(TSVD_ERR_INVALID, "bad arguments");
  if (!s->cfg.lp_right_factor) return fail(TSVD_ERR_STATE, "session built without lp_right_factor");
  if (m == 0) return TSVD_OK;
  TSVD_CUDA(cudaSetDevice(s->cfg.device));
  if (m > s->pairs_cap) {
    cudaFree(s->pairs_dev);
    cudaFree(s->scores_dev);
    s->pairs_dev = nullptr;
    s->scores_dev = nullptr;
    s->pairs_cap = 0;
    TSVD_CUDA(cudaMalloc(&s->pairs_dev, sizeof(int32_t) * 2 * m));
    TSVD_CUDA(cudaMalloc(&s->scores_dev, sizeof(double) * m));
    s->pairs_cap = m;
  }
  TSVD_CUDA(cudaMemcpyAsync(s->pairs_dev, pairs, sizeof(int32_t) * 2 * m, cudaMemcpyHostToDevice,
                            s->st));
  TSVD_CUDA(cudaMemsetAsync(s->bad_dev, 0, sizeof(int32_t), s->st));
  const int32_t *deg_i = s->adj[0].deg;
  const int32_t *deg_j = s->directed ? s->adj[1].deg : s->adj[0].deg;
  lp_score_kernel<<<grid_for(m * 32, 256, 8), 256, 0, s->st>>>(
      s->pairs_dev, m, s->src_row, s->colpos, s->n, s->col_dim, s->nparts, s->lp_v, s->lp_u,
      s->lp_valid_dev, s->d, s->S, deg_i, deg_j, degree_scaled, s->scores_dev, s->bad_dev);
  TSVD_LAUNCH_CHECK();
  int32_t bad = 0;
  TSVD_CUDA(cudaMemcpyAsync(scores, s->scores_dev, sizeof(double) * m, cudaMemcpyDeviceToHost,
                            s->st));
  TSVD_CUDA(cudaMemcpyAsync(&bad, s->bad_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, s->st));
  TSVD_CUDA(cudaStreamSynchronize(s->st));
  if (bad) return fail(TSVD_ERR_INVALID, "a pair's first vertex is not a source or a vertex is out of range");
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_lp_precision(const double *scores, const uint8_t *positive, int64_t m,
                                         int64_t k, double *precision) {
  if (!precision || m < 0 || k < 1 || k > m || (m > 0 && (!scores || !positive)))
    return fail(TSVD_ERR_INVALID, "need 1 <= k <= m");
  std::vector<int64_t> idx(m);
  for (int64_t i = 0; i < m; ++i) idx[i] = i;
  auto before = [&](int64_t a, int64_t b) {
    return scores[a] > scores[b] || (scores[a] == scores[b] && a < b);
  };
  std::nth_element(idx.begin(), idx.begin() + (k - 1), idx.end(), before);
  int64_t hit = 0;
  for (int64_t i = 0; i < k; ++i) hit += positive[idx[i]] ? 1 : 0;
  *precision = (double)hit / (double)k;
  return TSVD_OK;
}
