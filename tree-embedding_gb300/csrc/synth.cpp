// Host-side synthetic inputs and edge-file ingestion.
//
// R-MAT graphs stand in for the reference's public datasets; the snapshot
// split follows the reference's "first snapshot + equal deltas" layout
// (config.txt lines 1.., Code/Tree_u_NC.cpp:338-351), and the subset sampler
// mirrors Code/Random_Sample_Points_NC.cpp (uniform among first-snapshot
// nodes, written sorted). The text reader reproduces Code/Graph_dynamic.h:
// 127-130 / 539-542, including (optionally) its repeat of the last pair.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "philox_gauss.h"
#include "status.h"

namespace {

constexpr uint32_t kStreamRmat = 1, kStreamRelabel = 2, kStreamShuffle = 3,
                   kStreamSample = 4;

uint64_t rand_u64(uint64_t seed, uint32_t stream, uint64_t idx) {
  tsvd_philox4 r = tsvd_philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32),
                                      stream, 0x53594e54u, (uint32_t)seed,
                                      (uint32_t)(seed >> 32));
  return ((uint64_t)r.v[0] << 32) | r.v[1];
}

// Unbiased-enough bounded draw: high 64 bits of a 128-bit product.
uint64_t bounded(uint64_t r, uint64_t n) {
  return (uint64_t)(((unsigned __int128)r * n) >> 64);
}

// Fisher-Yates driven by a counter stream (deterministic for a seed).
template <typename T>
void shuffle(std::vector<T> &v, uint64_t seed, uint32_t stream) {
  for (uint64_t i = v.size(); i > 1; --i) {
    uint64_t j = bounded(rand_u64(seed, stream, i), i);
    std::swap(v[i - 1], v[j]);
  }
}

unsigned hw_threads() {
  unsigned t = std::thread::hardware_concurrency();
  return t == 0 ? 1 : std::min(t, 64u);
}

}  // namespace

extern "C" tsvd_status tsvd_rmat_edges(int32_t n, int64_t m, double a, double b,
                                       double c, int32_t directed,
                                       uint64_t seed, int32_t *edges_out) {
  using tsvd::fail;
  if (n < 2 || m < 0 || !edges_out)
    return fail(TSVD_ERR_INVALID, "rmat: n=%d m=%lld", n, (long long)m);
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return fail(TSVD_ERR_INVALID, "rmat: bad quadrant probabilities");
  double max_pairs = directed ? (double)n * (n - 1) : (double)n * (n - 1) / 2;
  if ((double)m > 0.5 * max_pairs)
    return fail(TSVD_ERR_INVALID, "rmat: m too large for n");
  int scale = 0;
  while ((1ll << scale) < n) ++scale;
  const uint64_t two32 = 4294967296ull;
  const uint64_t ta = (uint64_t)std::llround(a * two32);
  const uint64_t tab = (uint64_t)std::llround((a + b) * two32);
  const uint64_t tabc = (uint64_t)std::llround((a + b + c) * two32);
  const int calls = (scale + 3) / 4;

  // Candidates in generation order; key = (u << 32) | v, 0xff.. = rejected.
  std::vector<uint64_t> cand;
  std::vector<uint64_t> uniq_idx;
  uint64_t want = (uint64_t)m + (uint64_t)m / 3 + 1024;
  for (int attempt = 0; attempt < 12; ++attempt) {
    uint64_t old = cand.size();
    cand.resize(want);
    unsigned T = hw_threads();
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; ++t) {
      th.emplace_back([&, t]() {
        for (uint64_t i = old + t; i < want; i += T) {
          uint64_t u = 0, v = 0;
          for (int cl = 0; cl < calls; ++cl) {
            tsvd_philox4 r = tsvd_philox4x32_10(
                (uint32_t)i, (uint32_t)(i >> 32), kStreamRmat, (uint32_t)cl,
                (uint32_t)seed, (uint32_t)(seed >> 32));
            for (int w = 0; w < 4 && cl * 4 + w < scale; ++w) {
              uint64_t x = r.v[w];
              uint64_t bu = x >= tab ? 1 : 0;
              uint64_t bv = (x >= ta && x < tab) || x >= tabc ? 1 : 0;
              u = (u << 1) | bu;
              v = (v << 1) | bv;
            }
          }
          if (u >= (uint64_t)n || v >= (uint64_t)n || u == v) {
            cand[i] = ~0ull;
            continue;
          }
          if (!directed && u > v) std::swap(u, v);
          cand[i] = (u << 32) | v;
        }
      });
    }
    for (auto &x : th) x.join();
    // First occurrence of each key, in generation order.
    std::vector<uint64_t> order(cand.size());
    for (uint64_t i = 0; i < order.size(); ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](uint64_t x, uint64_t y) {
      return cand[x] != cand[y] ? cand[x] < cand[y] : x < y;
    });
    uniq_idx.clear();
    for (uint64_t k = 0; k < order.size(); ++k) {
      uint64_t key = cand[order[k]];
      if (key == ~0ull) break;
      if (k > 0 && cand[order[k - 1]] == key) continue;
      uniq_idx.push_back(order[k]);
    }
    if ((int64_t)uniq_idx.size() >= m) break;
    want = want + want / 2;
  }
  if ((int64_t)uniq_idx.size() < m)
    return fail(TSVD_ERR_INVALID, "rmat: could not draw %lld unique edges",
                (long long)m);
  std::sort(uniq_idx.begin(), uniq_idx.end());
  uniq_idx.resize((size_t)m);

  std::vector<int32_t> perm((size_t)n);
  for (int32_t i = 0; i < n; ++i) perm[i] = i;
  shuffle(perm, seed, kStreamRelabel);

  std::vector<uint64_t> edges((size_t)m);
  for (int64_t e = 0; e < m; ++e) {
    uint64_t key = cand[uniq_idx[e]];
    uint32_t u = perm[key >> 32], v = perm[key & 0xffffffffu];
    edges[e] = ((uint64_t)u << 32) | v;
  }
  // Uniform random timestamps == a uniformly random order of the edges.
  shuffle(edges, seed, kStreamShuffle);
  for (int64_t e = 0; e < m; ++e) {
    edges_out[2 * e] = (int32_t)(edges[e] >> 32);
    edges_out[2 * e + 1] = (int32_t)(edges[e] & 0xffffffffu);
  }
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_snapshot_sizes(int64_t m, int32_t n_snapshots,
                                           double first_frac,
                                           int64_t *sizes_out) {
  if (m < 0 || n_snapshots < 1 || first_frac < 0 || first_frac > 1 ||
      !sizes_out)
    return tsvd::fail(TSVD_ERR_INVALID, "snapshot_sizes: bad arguments");
  int64_t first = n_snapshots == 1 ? m : (int64_t)std::llround(first_frac * (double)m);
  sizes_out[0] = first;
  int64_t rest = m - first;
  for (int32_t i = 1; i < n_snapshots; ++i) {
    int64_t k = n_snapshots - 1;
    sizes_out[i] = rest / k + ((i - 1) < rest % k ? 1 : 0);
  }
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_sample_sources(int32_t n, const int32_t *edges,
                                           int64_t m, int32_t k, uint64_t seed,
                                           int32_t *out) {
  if (n < 1 || k < 1 || !edges || !out || m < 0)
    return tsvd::fail(TSVD_ERR_INVALID, "sample_sources: bad arguments");
  std::vector<uint8_t> seen((size_t)n, 0);
  for (int64_t e = 0; e < 2 * m; ++e) {
    int32_t v = edges[e];
    if (v < 0 || v >= n)
      return tsvd::fail(TSVD_ERR_INVALID, "sample_sources: vertex %d out of range", v);
    seen[v] = 1;
  }
  std::vector<int32_t> pool;
  for (int32_t v = 0; v < n; ++v)
    if (seen[v]) pool.push_back(v);
  if ((int64_t)pool.size() < k)
    return tsvd::fail(TSVD_ERR_INVALID, "sample_sources: only %zu candidates for %d",
                      pool.size(), k);
  // Partial Fisher-Yates: the first k slots become the sample.
  for (int32_t i = 0; i < k; ++i) {
    uint64_t j = i + bounded(rand_u64(seed, kStreamSample, (uint64_t)i),
                             pool.size() - i);
    std::swap(pool[i], pool[j]);
  }
  std::sort(pool.begin(), pool.begin() + k);
  std::copy(pool.begin(), pool.begin() + k, out);
  return TSVD_OK;
}

extern "C" tsvd_status tsvd_read_edge_file(const char *path,
                                           int32_t compat_dup_last,
                                           int32_t **edges, int64_t *m) {
  if (!path || !edges || !m) return tsvd::fail(TSVD_ERR_INVALID, "read_edge_file: null");
  const size_t plen = std::strlen(path);
  if (plen > 4 && std::strcmp(path + plen - 4, ".bin") == 0) {
    // binary: raw int32 (from, to) pairs in host byte order
    FILE *fb = std::fopen(path, "rb");
    if (!fb) return tsvd::fail(TSVD_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
    std::fseek(fb, 0, SEEK_END);
    const long bytes = std::ftell(fb);
    std::fseek(fb, 0, SEEK_SET);
    if (bytes < 0 || bytes % 8) {
      std::fclose(fb);
      return tsvd::fail(TSVD_ERR_IO, "%s: size %ld is not a whole number of int32 pairs", path, bytes);
    }
    int32_t *out = (int32_t *)std::malloc(std::max<long>(bytes, 8));
    if (!out) {
      std::fclose(fb);
      return tsvd::fail(TSVD_ERR_OOM, "read_edge_file: malloc");
    }
    const size_t got = std::fread(out, 1, (size_t)bytes, fb);
    std::fclose(fb);
    if (got != (size_t)bytes) {
      std::free(out);
      return tsvd::fail(TSVD_ERR_IO, "%s: short read", path);
    }
    *edges = out;
    *m = bytes / 8;
    return TSVD_OK;
  }
  FILE *f = std::fopen(path, "rb");
  if (!f) return tsvd::fail(TSVD_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
  std::vector<char> buf;
  char tmp[1 << 16];
  size_t got;
  while ((got = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  std::fclose(f);
  std::vector<int32_t> vals;
  size_t i = 0, nb = buf.size();
  bool trailing_space_after_last = false;
  while (i < nb) {
    while (i < nb && std::isspace((unsigned char)buf[i])) ++i;
    if (i >= nb) break;
    bool neg = false;
    if (buf[i] == '-' || buf[i] == '+') { neg = buf[i] == '-'; ++i; }
    if (i >= nb || !std::isdigit((unsigned char)buf[i]))
      return tsvd::fail(TSVD_ERR_IO, "%s: not an integer at byte %zu", path, i);
    int64_t x = 0;
    while (i < nb && std::isdigit((unsigned char)buf[i])) {
      x = x * 10 + (buf[i] - '0');
      if (x > INT32_MAX) return tsvd::fail(TSVD_ERR_IO, "%s: id overflow", path);
      ++i;
    }
    vals.push_back((int32_t)(neg ? -x : x));
    trailing_space_after_last = (i < nb);  // anything after the number (whitespace)
  }
  if (vals.size() % 2)
    return tsvd::fail(TSVD_ERR_IO, "%s: odd number of integers", path);
  // The reference loop `while (infile.good()) { infile >> from >> to; push }`
  // runs once more after the last pair whenever the stream has not hit EOF,
  // i.e. when whitespace follows the last number, and pushes the stale pair.
  if (compat_dup_last && !vals.empty() && trailing_space_after_last) {
    int32_t a = vals[vals.size() - 2], b = vals[vals.size() - 1];
    vals.push_back(a);
    vals.push_back(b);
  }
  int32_t *out = (int32_t *)std::malloc(std::max<size_t>(1, vals.size()) * sizeof(int32_t));
  if (!out) return tsvd::fail(TSVD_ERR_OOM, "read_edge_file: malloc");
  std::copy(vals.begin(), vals.end(), out);
  *edges = out;
  *m = (int64_t)(vals.size() / 2);
  return TSVD_OK;
}

extern "C" void tsvd_free(void *p) { std::free(p); }

extern "C" float tsvd_gaussian(uint64_t seed, uint32_t stream, uint32_t row,
                               uint32_t col) {
  return tsvd_gauss_entry(seed, stream, row, col);
}

extern "C" tsvd_status tsvd_write_edge_file_binary(const char *path, const int32_t *edges,
                                                   int64_t m) {
  if (!path || (m > 0 && !edges) || m < 0) return tsvd::fail(TSVD_ERR_INVALID, "write_edge_file: bad arguments");
  FILE *f = std::fopen(path, "wb");
  if (!f) return tsvd::fail(TSVD_ERR_IO, "cannot create %s: %s", path, std::strerror(errno));
  const size_t want = (size_t)m * 2 * sizeof(int32_t);
  const size_t put = want ? std::fwrite(edges, 1, want, f) : 0;
  const int rc = std::fclose(f);
  if (put != want || rc != 0) return tsvd::fail(TSVD_ERR_IO, "%s: short write", path);
  return TSVD_OK;
}
