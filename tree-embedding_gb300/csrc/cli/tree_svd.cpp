// tree_svd — command-line drop-in for the reference drivers Tree_u_NC,
// Tree_d_NC, Tree_u_LP and Tree_d_LP (Code/Tree_u_NC.cpp:296-911 and
// siblings), running the snapshot loop on the GPU through libtsvd_gb300.
//
//   tree_svd <u_nc|d_nc|u_lp|d_lp> queryname EBpath alpha pass rmax NUMTHREAD \
//            nParts hierarchy_n N dynamic_ppr_start_iter lazy_update_start_iter delta \
//            [--compat] [--device K] [--npy]
//   tree_svd split <nc|lp> queryname round_index [--batch B] [--count C] [--compat]
//
// While the GPU runs a snapshot, the next snapshot's file is read and parsed
// on a host thread. --npy also writes the embeddings as <output>.npy
// (float64, ((T-1)*|S|) x 128). `split` is the batch splitter of
// Code/split_edges_NC.cpp / split_edges_LP.cpp: snapshots before round_index
// are kept, the edges from round_index on are re-cut into files of B edges
// (10,000), at most C of them (100), under DY_[LP_]Dataset/<queryname>_batch/.
//
// Same positional arguments (Tree_u_NC.cpp:301-322; NUMTHREAD is accepted and
// ignored), same inputs (DY_Dataset/<queryname>/config.txt: line 0 the subset
// file, then one edge file per snapshot, :338-372) and the same output file
// name and CSV layout (:877-909): ((T-1)*|S|) x 128 values, ", " separated,
// six significant digits. --compat reproduces the reference's reader (last
// pair of a file repeated when whitespace follows it) and its integer-division
// refresh; without it the exact refresh is used.
//
// The LP modes follow Tree_u_LP.cpp / Tree_d_LP.cpp instead: inputs from
// DY_LP_Dataset/<queryname>/ (config.txt and the <queryname>-Pos_LP_Test.txt /
// -Neg_LP_Test.txt pairs, :473, :617-638), the LOG10_LP transform, the root
// factor U, and after every snapshot the right factor of the refreshed blocks
// and "link prediction precision: P", the share of positive pairs among the
// sample_m best-scored test pairs (:1040-1122); no embedding file is written.
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "tsvd.h"

static int die(const char *what, tsvd_status st) {
  std::fprintf(stderr, "tree_svd: %s: %s (%s)\n", what, tsvd_status_string(st), tsvd_last_error());
  return 1;
}

// Code/split_edges_NC.cpp:21-131 (and the LP twin with DY_LP_Dataset).
static int split_main(int argc, char **argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s split <nc|lp> queryname round_index [--batch B] [--count C] "
                         "[--compat]\n", argv[0]);
    return 2;
  }
  const bool lp = std::string(argv[2]) == "lp";
  const std::string root = lp ? "DY_LP_Dataset/" : "DY_Dataset/";
  const std::string q = argv[3], bq = q + "_batch";
  const int round_index = std::atoi(argv[4]);
  int64_t per = 10000, count = 100;
  bool compat = false;
  for (int i = 5; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--batch") && i + 1 < argc) per = std::atoll(argv[++i]);
    else if (!std::strcmp(argv[i], "--count") && i + 1 < argc) count = std::atoll(argv[++i]);
    else if (!std::strcmp(argv[i], "--compat")) compat = true;
  }
  std::vector<std::string> shots;
  {
    std::ifstream cfg((root + q + "/config.txt").c_str());
    if (!cfg) {
      std::fprintf(stderr, "tree_svd: cannot read %s%s/config.txt\n", root.c_str(), q.c_str());
      return 1;
    }
    std::string line;
    while (std::getline(cfg, line)) shots.push_back(line);
  }
  if (round_index < 0 || round_index > (int)shots.size() || per < 1 || count < 1) {
    std::fprintf(stderr, "tree_svd: bad round_index / batch / count\n");
    return 2;
  }
  ::mkdir((root + bq).c_str(), 0755);
  std::ofstream oc((root + bq + "/config.txt").c_str());
  for (int i = 0; i < round_index; ++i) oc << shots[i] << "\n";
  std::vector<int32_t> pending;
  int64_t written = 0;
  for (size_t f = round_index; f < shots.size() && written < count; ++f) {
    int32_t *e = nullptr;
    int64_t m = 0;
    tsvd_status st = tsvd_read_edge_file(shots[f].c_str(), compat ? 1 : 0, &e, &m);
    if (st != TSVD_OK) return die(shots[f].c_str(), st);
    pending.insert(pending.end(), e, e + 2 * m);
    tsvd_free(e);
    while ((int64_t)pending.size() >= 2 * per && written < count) {
      ++written;
      const std::string name = "./" + root + bq + "/" + bq + "-Train-" +
                               std::to_string(round_index) + "-" + std::to_string(written) + ".txt";
      std::ofstream out(name.c_str());
      for (int64_t i = 0; i < per; ++i) out << pending[2 * i] << " " << pending[2 * i + 1] << "\n";
      oc << name << "\n";
      pending.erase(pending.begin(), pending.begin() + 2 * per);
    }
  }
  if (written < count)
    std::printf("We have read all consecutive edges, but there are not enough edges till the end!\n");
  std::printf("wrote %lld batches of %lld edges\n", (long long)written, (long long)per);
  return 0;
}

static bool write_npy(const std::string &path, const std::vector<double> &a, size_t rows,
                      size_t cols) {
  std::ofstream os(path.c_str(), std::ios::binary);
  if (!os) return false;
  std::string hdr = "{'descr': '<f8', 'fortran_order': False, 'shape': (" + std::to_string(rows) +
                    ", " + std::to_string(cols) + "), }";
  while ((10 + hdr.size() + 1) % 64) hdr += ' ';
  hdr += '\n';
  const unsigned short hl = (unsigned short)hdr.size();
  os.write("\x93NUMPY\x01\x00", 8);
  os.put((char)(hl & 0xff));
  os.put((char)(hl >> 8));
  os << hdr;
  os.write(reinterpret_cast<const char *>(a.data()), (std::streamsize)(rows * cols * sizeof(double)));
  return (bool)os;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !std::strcmp(argv[1], "split")) return split_main(argc, argv);
  if (argc < 14) {
    std::fprintf(stderr,
                 "usage: %s <u_nc|d_nc|u_lp|d_lp> queryname EBpath alpha pass rmax NUMTHREAD "
                 "nParts hierarchy_n N dynamic_ppr_start_iter lazy_update_start_iter delta "
                 "[--compat] [--device K]\n",
                 argv[0]);
    return 2;
  }
  const std::string mode = argv[1];
  const bool directed = mode[0] == 'd';
  const bool lp = mode.size() >= 4 && mode.substr(2) == "lp";
  const std::string queryname = argv[2], ebpath = argv[3];
  char *endp;
  const double alpha = std::strtod(argv[4], &endp);
  const int pass = (int)std::strtod(argv[5], &endp);
  const double rmax = std::strtod(argv[6], &endp);
  const int nparts = (int)std::strtod(argv[8], &endp);
  const int hn = (int)std::strtod(argv[9], &endp);
  const int nv = (int)std::strtod(argv[10], &endp);
  const int dyn = (int)std::strtod(argv[11], &endp);
  const int lazy = (int)std::strtod(argv[12], &endp);
  const double delta = std::strtod(argv[13], &endp);
  bool compat = false, npy = false;
  int device = 0;
  for (int i = 14; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--compat")) compat = true;
    else if (!std::strcmp(argv[i], "--npy")) npy = true;
    else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) device = std::atoi(argv[++i]);
  }
  const std::string dataset = std::string(lp ? "DY_LP_Dataset/" : "DY_Dataset/") + queryname + "/";
  std::vector<std::string> shots;
  {
    std::ifstream cfg((dataset + "config.txt").c_str());
    if (!cfg) {
      std::fprintf(stderr, "tree_svd: cannot read %sconfig.txt\n", dataset.c_str());
      return 1;
    }
    std::string line;
    while (std::getline(cfg, line)) shots.push_back(line);
  }
  if (shots.size() < 2) {
    std::fprintf(stderr, "tree_svd: config.txt needs a subset file and at least one snapshot\n");
    return 1;
  }
  std::vector<int32_t> sources;
  {
    std::ifstream sf(shots[0].c_str());
    int v;
    while (sf >> v) sources.push_back(v);
  }
  const int d = 128;
  tsvd_config c;
  tsvd_config_default(&c);
  c.n_vertices = nv;
  c.directed = directed;
  c.n_sources = (int32_t)sources.size();
  c.sources = sources.data();
  c.alpha = alpha;
  c.rmax = rmax;
  c.n_parts = nparts;
  c.hierarchy_n = hn;
  c.rank_d = d;
  c.passes_q = pass;
  c.dynamic_ppr_start_iter = dyn;
  c.lazy_update_start_iter = lazy;
  c.delta = delta;
  c.transform = lp ? TSVD_TRANSFORM_LOG10_LP : TSVD_TRANSFORM_LOG10_NC;
  c.root_scaling = lp ? TSVD_ROOT_U : TSVD_ROOT_SQRT_SIGMA;
  c.refresh_mode = compat ? TSVD_REFRESH_INTDIV : TSVD_REFRESH_EXACT;
  c.device = device;
  c.lp_right_factor = lp ? 1 : 0;
  // LP test pairs: both files as sets, positives first (Tree_u_LP.cpp:617-638);
  // sample_m counts every read of the positive file, including the repeated
  // last pair of the reference's reader under --compat.
  std::vector<int32_t> test_pairs;
  std::vector<uint8_t> test_pos;
  int64_t sample_m = 0;
  if (lp) {
    std::vector<std::pair<int32_t, int32_t>> pos, neg;
    for (int f = 0; f < 2; ++f) {
      const std::string path = dataset + queryname + (f ? "-Neg_LP_Test.txt" : "-Pos_LP_Test.txt");
      int32_t *e = nullptr;
      int64_t m = 0;
      tsvd_status rs = tsvd_read_edge_file(path.c_str(), compat ? 1 : 0, &e, &m);
      if (rs != TSVD_OK) return die(path.c_str(), rs);
      auto &dst = f ? neg : pos;
      for (int64_t i = 0; i < m; ++i) dst.emplace_back(e[2 * i], e[2 * i + 1]);
      if (!f) sample_m = m;
      tsvd_free(e);
      std::sort(dst.begin(), dst.end());
      dst.erase(std::unique(dst.begin(), dst.end()), dst.end());
    }
    for (int f = 0; f < 2; ++f)
      for (auto &p : f ? neg : pos) {
        test_pairs.push_back(p.first);
        test_pairs.push_back(p.second);
        test_pos.push_back(f == 0 || std::binary_search(pos.begin(), pos.end(), p) ? 1 : 0);
      }
  }
  tsvd_session *s = nullptr;
  tsvd_status st = tsvd_session_create(&c, &s);
  if (st != TSVD_OK) return die("session", st);
  const size_t S = sources.size();
  const int T = (int)shots.size();
  std::vector<double> all((size_t)(T - 1) * S * d, 0.0), emb(S * d, 0.0);
  bool have = false;
  // the next snapshot's file is read on a host thread while the GPU works
  struct Loaded {
    int32_t *edges = nullptr;
    int64_t m = 0;
    tsvd_status st = TSVD_OK;
  };
  auto load = [&](int it, Loaded *out) {
    out->st = tsvd_read_edge_file(shots[it].c_str(), compat ? 1 : 0, &out->edges, &out->m);
  };
  Loaded cur, nxt;
  load(1, &cur);
  for (int it = 1; it < T; ++it) {
    std::thread reader;
    if (it + 1 < T) reader = std::thread(load, it + 1, &nxt);
    if (cur.st != TSVD_OK) {
      if (reader.joinable()) reader.join();
      return die(shots[it].c_str(), cur.st);
    }
    st = tsvd_session_step(s, cur.edges, cur.m);
    tsvd_free(cur.edges);
    cur.edges = nullptr;
    if (reader.joinable()) reader.join();
    if (st != TSVD_OK) return die("step", st);
    cur = nxt;
    nxt = Loaded();
    tsvd_step_stats ss;
    tsvd_session_last_stats(s, &ss);
    std::printf("Iter = %d, edges %lld, pushes %lld, dirty %d, time = %.3f ms\n", it,
                (long long)ss.edges_inserted, (long long)ss.pushes, ss.dirty_blocks, ss.ms_total);
    if (tsvd_session_embedding(s, emb.data()) == TSVD_OK) have = true;
    if (have) std::copy(emb.begin(), emb.end(), all.begin() + (size_t)(it - 1) * S * d);
    const int64_t np = (int64_t)test_pos.size();
    if (lp && have && np > 0) {
      std::vector<double> score(np);
      st = tsvd_lp_scores(s, test_pairs.data(), np, 0, score.data());
      if (st != TSVD_OK) return die("lp scores", st);
      double prec = 0;
      st = tsvd_lp_precision(score.data(), test_pos.data(), np, std::min(sample_m, np), &prec);
      if (st != TSVD_OK) return die("lp precision", st);
      std::printf("link prediction precision: %g\n", prec);
    }
  }
  tsvd_session_destroy(s);
  if (lp) return 0;
  // Tree_u_NC.cpp:877-896
  int residue_order = 0;
  if (rmax * 10000 == 1) residue_order = 5;
  else if (rmax * 100000 == 1) residue_order = 6;
  else if (rmax * 1000000 == 1) residue_order = 7;
  else if (rmax * 10000000 == 1) residue_order = 8;
  else if (rmax * 1000000000 == 1) residue_order = 10;
  const std::string out = ebpath + queryname + std::to_string(delta) + "_" +
                          std::to_string(residue_order) + "_" + std::to_string(nparts) + "_" +
                          std::to_string(hn) + "_" + "De_svd_" + (directed ? "d" : "u") +
                          "_Dppr_parallel_bound_nodegree_U.csv";
  std::ofstream os(out.c_str());
  if (!os) {
    std::fprintf(stderr, "tree_svd: cannot write %s\n", out.c_str());
    return 1;
  }
  const size_t rows = (size_t)(T - 1) * S;
  for (size_t r = 0; r < rows; ++r) {
    for (int j = 0; j < d; ++j) {
      if (j) os << ", ";
      os << all[r * d + j];
    }
    if (r + 1 < rows) os << "\n";
  }
  std::printf("wrote %s\n", out.c_str());
  if (npy) {
    if (!write_npy(out + ".npy", all, rows, d)) {
      std::fprintf(stderr, "tree_svd: cannot write %s.npy\n", out.c_str());
      return 1;
    }
    std::printf("wrote %s.npy\n", out.c_str());
  }
  return 0;
}
