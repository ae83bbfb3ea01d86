// Serving layer: many tenants (graphs with their source subsets) resident on
// one GPU, edge-update batches and embedding queries taken as they arrive.
//
// No counterpart in the reference, whose drivers (Code/Tree_u_NC.cpp:296-911)
// refresh one graph from a fixed list of delta files. Here:
//   * a tenant is one session (its CSR, PPR state, block factors and tree on
//     the device); it is admitted when its estimated footprint
//     (tsvd_session_footprint) fits in the HBM budget left, and its measured
//     footprint (free device memory before and after) is charged to the
//     budget until it is removed;
//   * requests queue per tenant in arrival order (a session takes one caller
//     at a time); `slots` worker threads each take the oldest waiting request
//     whose tenant is idle, so a request that arrives while others run starts
//     as soon as a slot and its tenant are free, and different tenants' work
//     overlaps on the device (every session has its own stream);
//   * an update runs one snapshot (tsvd_session_step); a query copies the
//     tenant's embedding as of every update submitted before it;
//   * latency = completion - submission (queueing included); the server keeps
//     every update's latency for p50 / p99 and the edges applied.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "status.h"
#include "tsvd.h"

using tsvd::fail;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int32_t tenant = 0;
  int kind = 0;  // 0 update, 1 query
  std::vector<int32_t> edges;
  double *out = nullptr;
  Clock::time_point t_submit, t_start, t_end;
  tsvd_status status = TSVD_OK;
  std::string error;
  bool done = false;
};

struct Tenant {
  tsvd_session *s = nullptr;
  int64_t charged = 0;
  bool busy = false;
  bool alive = false;
  std::deque<int64_t> queue;
  int64_t edges_applied = 0;
  int64_t updates_done = 0;
};

}  // namespace

struct tsvd_server {
  int device = 0;
  int64_t budget = 0, used = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<Tenant> tenants;
  std::unordered_map<int64_t, Request> reqs;
  std::deque<int64_t> order;  // waiting request ids, arrival order
  int64_t next_id = 1;
  bool stop = false;
  std::vector<std::thread> workers;
  std::vector<double> lat_ms;  // completed updates
  int64_t edges_total = 0;
  Clock::time_point t_first{}, t_last{};
  bool any = false;
};

namespace {

// The oldest waiting request whose tenant is idle (called with mu held).
bool take(tsvd_server *sv, int64_t *id) {
  for (auto it = sv->order.begin(); it != sv->order.end(); ++it) {
    Request &r = sv->reqs[*it];
    Tenant &t = sv->tenants[r.tenant];
    if (t.busy || t.queue.empty() || t.queue.front() != *it) continue;
    *id = *it;
    sv->order.erase(it);
    t.queue.pop_front();
    t.busy = true;
    return true;
  }
  return false;
}

void worker_loop(tsvd_server *sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    int64_t id = 0;
    sv->cv_work.wait(lk, [&] { return sv->stop || take(sv, &id); });
    if (sv->stop && id == 0) return;
    Request &r = sv->reqs[id];
    Tenant &t = sv->tenants[r.tenant];
    tsvd_session *s = t.s;
    r.t_start = Clock::now();
    lk.unlock();
    tsvd_status st;
    if (r.kind == 0)
      st = tsvd_session_step(s, r.edges.data(), (int64_t)(r.edges.size() / 2));
    else
      st = tsvd_session_embedding(s, r.out);
    std::string err = st == TSVD_OK ? std::string() : std::string(tsvd_last_error());
    lk.lock();
    Request &q = sv->reqs[id];
    q.t_end = Clock::now();
    q.status = st;
    q.error = err;
    q.done = true;
    Tenant &tt = sv->tenants[q.tenant];
    tt.busy = false;
    if (q.kind == 0 && st == TSVD_OK) {
      tt.edges_applied += (int64_t)(q.edges.size() / 2);
      tt.updates_done += 1;
      sv->edges_total += (int64_t)(q.edges.size() / 2);
      sv->lat_ms.push_back(std::chrono::duration<double, std::milli>(q.t_end - q.t_submit).count());
      sv->t_last = q.t_end;
    }
    std::vector<int32_t>().swap(q.edges);
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double x = p / 100.0 * (double)(v.size() - 1);
  const size_t i = (size_t)x;
  const double f = x - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" tsvd_status tsvd_server_create(int32_t device, int64_t hbm_budget_bytes, int32_t slots,
                                          tsvd_server **out) {
  if (!out || slots < 1 || slots > 64) return fail(TSVD_ERR_INVALID, "server: 1 <= slots <= 64");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess)
    return fail(TSVD_ERR_DEVICE, "server: device %d", device);
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return fail(TSVD_ERR_DEVICE, "server: meminfo");
  tsvd_server *sv = new tsvd_server;
  sv->device = device;
  // default budget: what is free now, less 4 GB for the runtime and staging
  sv->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes
                                    : std::max<int64_t>(0, (int64_t)fr - (4ll << 30));
  try {
    for (int i = 0; i < slots; ++i) sv->workers.emplace_back(worker_loop, sv);
  } catch (...) {
    {
      std::lock_guard<std::mutex> g(sv->mu);
      sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto &w : sv->workers) w.join();
    delete sv;
    return fail(TSVD_ERR_STATE, "server: could not start the worker threads");
  }
  *out = sv;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_add_tenant(tsvd_server *sv, const tsvd_config *cfg,
                                              int64_t expected_edges, int32_t *tenant) {
  if (!sv || !cfg || !tenant) return fail(TSVD_ERR_INVALID, "server: null argument");
  tsvd_config c = *cfg;
  c.device = sv->device;
  int64_t est = 0;
  if (tsvd_session_footprint(&c, expected_edges, &est) != TSVD_OK) return TSVD_ERR_INVALID;
  std::lock_guard<std::mutex> g(sv->mu);  // one admission at a time: the memory delta is ours
  if (sv->used + est > sv->budget)
    return fail(TSVD_ERR_OOM, "server: tenant needs about %.2f GB, %.2f GB of the budget left",
                est / 1e9, (sv->budget - sv->used) / 1e9);
  cudaSetDevice(sv->device);
  size_t f0 = 0, f1 = 0, tot = 0;
  cudaMemGetInfo(&f0, &tot);
  tsvd_session *s = nullptr;
  tsvd_status st = tsvd_session_create(&c, &s);
  if (st != TSVD_OK) return st;
  cudaMemGetInfo(&f1, &tot);
  Tenant t;
  t.s = s;
  t.alive = true;
  // the larger of the estimate and what the creation took: buffers that grow
  // with the edges come later
  t.charged = std::max<int64_t>(est, (int64_t)f0 - (int64_t)f1);
  sv->used += t.charged;
  sv->tenants.push_back(std::move(t));
  *tenant = (int32_t)sv->tenants.size() - 1;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_remove_tenant(tsvd_server *sv, int32_t tenant) {
  if (!sv) return fail(TSVD_ERR_INVALID, "server: null");
  std::unique_lock<std::mutex> lk(sv->mu);
  if (tenant < 0 || tenant >= (int32_t)sv->tenants.size() || !sv->tenants[tenant].alive)
    return fail(TSVD_ERR_INVALID, "server: no tenant %d", tenant);
  Tenant &t = sv->tenants[tenant];
  sv->cv_done.wait(lk, [&] { return !t.busy && t.queue.empty(); });
  tsvd_session_destroy(t.s);
  t.s = nullptr;
  t.alive = false;
  sv->used -= t.charged;
  t.charged = 0;
  return TSVD_OK;
}

static tsvd_status submit(tsvd_server *sv, int32_t tenant, int kind, const int32_t *edges,
                          int64_t m, double *out, int64_t *request) {
  if (!sv || !request) return fail(TSVD_ERR_INVALID, "server: null argument");
  if (kind == 0 && (m < 0 || (m > 0 && !edges))) return fail(TSVD_ERR_INVALID, "server: edges");
  if (kind == 1 && !out) return fail(TSVD_ERR_INVALID, "server: null output");
  std::lock_guard<std::mutex> g(sv->mu);
  if (tenant < 0 || tenant >= (int32_t)sv->tenants.size() || !sv->tenants[tenant].alive)
    return fail(TSVD_ERR_INVALID, "server: no tenant %d", tenant);
  const int64_t id = sv->next_id++;
  Request &r = sv->reqs[id];
  r.id = id;
  r.tenant = tenant;
  r.kind = kind;
  if (kind == 0) r.edges.assign(edges, edges + 2 * m);
  r.out = out;
  r.t_submit = Clock::now();
  if (!sv->any) {
    sv->t_first = r.t_submit;
    sv->any = true;
  }
  sv->tenants[tenant].queue.push_back(id);
  sv->order.push_back(id);
  *request = id;
  sv->cv_work.notify_one();
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_submit_update(tsvd_server *sv, int32_t tenant,
                                                 const int32_t *edges, int64_t m,
                                                 int64_t *request) {
  return submit(sv, tenant, 0, edges, m, nullptr, request);
}

extern "C" tsvd_status tsvd_server_submit_query(tsvd_server *sv, int32_t tenant, double *out,
                                                int64_t *request) {
  return submit(sv, tenant, 1, nullptr, 0, out, request);
}

extern "C" tsvd_status tsvd_server_wait(tsvd_server *sv, int64_t request, double *latency_ms,
                                        double *service_ms) {
  if (!sv) return fail(TSVD_ERR_INVALID, "server: null");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(request);
  if (it == sv->reqs.end()) return fail(TSVD_ERR_INVALID, "server: no request %lld", (long long)request);
  sv->cv_done.wait(lk, [&] { return it->second.done; });
  const Request &r = it->second;
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r.t_end - r.t_submit).count();
  if (service_ms)
    *service_ms = std::chrono::duration<double, std::milli>(r.t_end - r.t_start).count();
  const tsvd_status st = r.status;
  const std::string err = r.error;
  sv->reqs.erase(it);
  if (st != TSVD_OK) return fail(st, "server request %lld: %s", (long long)request, err.c_str());
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_drain(tsvd_server *sv) {
  if (!sv) return fail(TSVD_ERR_INVALID, "server: null");
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv_done.wait(lk, [&] {
    if (!sv->order.empty()) return false;
    for (const Tenant &t : sv->tenants)
      if (t.busy) return false;
    return true;
  });
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_stats(tsvd_server *sv, tsvd_server_stats_t *out) {
  if (!sv || !out) return fail(TSVD_ERR_INVALID, "server: null argument");
  std::lock_guard<std::mutex> g(sv->mu);
  std::memset(out, 0, sizeof *out);
  out->updates = (int64_t)sv->lat_ms.size();
  out->edges = sv->edges_total;
  out->p50_ms = percentile(sv->lat_ms, 50);
  out->p99_ms = percentile(sv->lat_ms, 99);
  const double span = sv->any ? std::chrono::duration<double>(sv->t_last - sv->t_first).count() : 0;
  out->edges_per_s = span > 0 ? sv->edges_total / span : 0.0;
  out->hbm_budget = sv->budget;
  out->hbm_charged = sv->used;
  int32_t alive = 0;
  for (const Tenant &t : sv->tenants) alive += t.alive ? 1 : 0;
  out->tenants = alive;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_session(tsvd_server *sv, int32_t tenant, tsvd_session **out) {
  if (!sv || !out) return fail(TSVD_ERR_INVALID, "server: null argument");
  std::lock_guard<std::mutex> g(sv->mu);
  if (tenant < 0 || tenant >= (int32_t)sv->tenants.size() || !sv->tenants[tenant].alive)
    return fail(TSVD_ERR_INVALID, "server: no tenant %d", tenant);
  *out = sv->tenants[tenant].s;
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_server_destroy(tsvd_server *sv) {
  if (!sv) return TSVD_OK;
  tsvd_server_drain(sv);
  {
    std::lock_guard<std::mutex> g(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto &w : sv->workers) w.join();
  for (Tenant &t : sv->tenants)
    if (t.s) tsvd_session_destroy(t.s);
  delete sv;
  return TSVD_OK;
}
