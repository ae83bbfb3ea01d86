// TEST INFRASTRUCTURE ONLY: a thin C wrapper around the reference's own
// dense-path code, compiled from the reference sources where they lie by
// oracle/build_ref.sh into oracle/_ref/libtsvd_ref.so. Used to pin the
// oracle (oracle/oracle_ppr.c) bit-for-bit; never linked into the product.
//
// Compiled reference pieces:
//   Code/Graph_dynamic.h                (UGraph / Graph and their inserts)
//   Code/my_queue.h                     (Queue)
//   Code/ppr_computation_store_dynamic.h lines 1394-1498, 2035-2121,
//     2945-3030, 3356-3437, 3811-3898, 4133-4228 (the six dense-path
//     refresh / push functions used by Tree_{u,d}_{NC,LP}.cpp), extracted at
//     build time because the rest of that header needs MKL, Eigen and emhash.
// The only reference type those functions touch beyond the graph and queue is
// d_row_tree_mkl::dense_mat_mapping[b](row, col) += x; a minimal stand-in with
// that member is defined below.
//
// Also compiled: the four log-transform + lazy-test functions of the same
// header (lines 2527-2561, 2598-2638, 2649-2732, 2742-2826). They use Eigen's
// SparseMatrix (sparseView of the dense block, InnerIterator, norm, a
// difference); Eigen is not in this image, so a minimal column-major sparse
// matrix with that interface is written below.
#include <algorithm>  // Graph_dynamic.h expects it first, as in the drivers
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "Graph_dynamic.h"
#include "my_queue.h"

using namespace std;

enum { ColMajor = 0 };

// Column-major compressed sparse matrix: the subset of Eigen::SparseMatrix the
// log functions use. Stored entries keep their order (rows ascending within a
// column); norm() sums the squares in that order.
template <typename T, int Options, typename Index>
class SparseMatrix {
 public:
  struct Storage {
    void squeeze() {}
  };
  int nrows = 0, ncols = 0;
  vector<Index> outer = vector<Index>(1, 0), inner;
  vector<T> val;

  void resize(int r, int c) {
    nrows = r;
    ncols = c;
    outer.assign((size_t)c + 1, 0);
    inner.clear();
    val.clear();
  }
  int outerSize() const { return ncols; }
  Storage data() { return Storage(); }
  double norm() const {
    double acc = 0;
    for (T x : val) acc += (double)x * (double)x;
    return std::sqrt(acc);
  }
  // this - o over the union of the two patterns; an empty (0 x 0) operand is zero
  SparseMatrix operator-(const SparseMatrix &o) const {
    const SparseMatrix &a = *this;
    SparseMatrix out;
    const int c = std::max(a.ncols, o.ncols);
    out.resize(std::max(a.nrows, o.nrows), c);
    for (int j = 0; j < c; ++j) {
      Index p = j < a.ncols ? a.outer[j] : 0, pe = j < a.ncols ? a.outer[j + 1] : 0;
      Index q = j < o.ncols ? o.outer[j] : 0, qe = j < o.ncols ? o.outer[j + 1] : 0;
      while (p < pe || q < qe) {
        if (q >= qe || (p < pe && a.inner[p] < o.inner[q])) {
          out.inner.push_back(a.inner[p]);
          out.val.push_back(a.val[p++]);
        } else if (p >= pe || o.inner[q] < a.inner[p]) {
          out.inner.push_back(o.inner[q]);
          out.val.push_back(-o.val[q++]);
        } else {
          out.inner.push_back(a.inner[p]);
          out.val.push_back(a.val[p++] - o.val[q++]);
        }
      }
      out.outer[j + 1] = (Index)out.val.size();
    }
    return out;
  }

  class InnerIterator {
   public:
    InnerIterator(SparseMatrix &m, int col) : m_(m), p_(m.outer[col]), end_(m.outer[col + 1]) {}
    explicit operator bool() const { return p_ < end_; }
    InnerIterator &operator++() {
      ++p_;
      return *this;
    }
    T value() const { return m_.val[p_]; }
    T &valueRef() { return m_.val[p_]; }
    Index row() const { return m_.inner[p_]; }

   private:
    SparseMatrix &m_;
    Index p_, end_;
  };
};

struct RefDenseBlock {
  int rows = 0, cols = 0;
  vector<double> v;
  double &operator()(int i, int j) { return v[(size_t)j * rows + i]; }
  // the non-zero entries, as Eigen's sparseView() keeps them
  SparseMatrix<double, 0, int> sparseView() const {
    SparseMatrix<double, 0, int> m;
    m.resize(rows, cols);
    for (int j = 0; j < cols; ++j) {
      for (int i = 0; i < rows; ++i) {
        const double x = v[(size_t)j * rows + i];
        if (x != 0.0) {
          m.inner.push_back(i);
          m.val.push_back(x);
        }
      }
      m.outer[j + 1] = (int)m.val.size();
    }
    return m;
  }
};

class d_row_tree_mkl {
 public:
  unordered_map<int, RefDenseBlock> dense_mat_mapping;
  unordered_map<int, SparseMatrix<double, 0, int>> mat_mapping;
  int row_dim = 0;
  vector<double> norm_B_Bid_difference_vec;
};

#include "ref_functions.inc"

namespace {

struct RefGraph {
  int directed = 0;
  int n = 0;
  UGraph *ug = nullptr;
  Graph *dg = nullptr;
};

struct RefPPR {
  int n = 0, S = 0, nparts = 0, col_dim = 0;
  double alpha = 0, rmax = 0;
  vector<int> sources, inner, indicator;
  unordered_map<int, int> row_index;
  vector<float *> r, p;
  vector<bool *> flags;
  vector<Queue> queues;
  d_row_tree_mkl tree;
  vector<long long int> nnz_record;
};

}  // namespace

extern "C" {

void *ref_graph_new(int n, int directed) {
  RefGraph *g = new RefGraph;
  g->directed = directed;
  g->n = n;
  if (directed) {
    g->dg = new Graph();
    g->dg->initializeDirectedDynamicGraph(n);
    // The reference relies on freshly mapped (zeroed) pointer arrays.
    memset(g->dg->inAdjList, 0, sizeof(int *) * n);
    memset(g->dg->outAdjList, 0, sizeof(int *) * n);
    memset(g->dg->BiggerInAdjList, 0, sizeof(int *) * n);
    memset(g->dg->BiggerOutAdjList, 0, sizeof(int *) * n);
  } else {
    g->ug = new UGraph();
    g->ug->initializeDynamicUGraph(n);
    memset(g->ug->AdjList, 0, sizeof(int *) * n);
    memset(g->ug->BiggerAdjList, 0, sizeof(int *) * n);
  }
  return g;
}

// Reads one delta file with the reference reader (including its handling of
// a trailing newline). Returns the number of pairs it appended.
long long ref_graph_insert_file(void *gp, const char *path) {
  RefGraph *g = (RefGraph *)gp;
  vector<pair<int, int>> ev;
  if (g->directed)
    g->dg->inputDirectedDynamicGraph(string(path), ev);
  else
    g->ug->inputDynamicGraph(string(path), ev);
  return (long long)ev.size();
}

void ref_graph_degrees(void *gp, int dir, int *deg, int *former) {
  RefGraph *g = (RefGraph *)gp;
  const int *d, *f;
  if (g->directed) {
    d = dir ? g->dg->indegree : g->dg->outdegree;
    f = dir ? g->dg->former_indegree : g->dg->former_outdegree;
  } else {
    d = g->ug->degree;
    f = g->ug->former_degree;
  }
  if (deg) memcpy(deg, d, sizeof(int) * g->n);
  if (former) memcpy(former, f, sizeof(int) * g->n);
}

long long ref_graph_adjacency(void *gp, int dir, long long *offsets, int *nbrs) {
  RefGraph *g = (RefGraph *)gp;
  long long pos = 0;
  for (int i = 0; i < g->n; ++i) {
    int d;
    int *row;
    if (g->directed) {
      d = dir ? g->dg->indegree[i] : g->dg->outdegree[i];
      row = dir ? g->dg->inAdjList[i] : g->dg->outAdjList[i];
    } else {
      d = g->ug->degree[i];
      row = g->ug->AdjList[i];
    }
    if (offsets) offsets[i] = pos;
    if (nbrs && d) memcpy(nbrs + pos, row, sizeof(int) * d);
    pos += d;
  }
  if (offsets) offsets[g->n] = pos;
  return pos;
}

void *ref_ppr_new(int n, int S, const int *sources, int nparts, double alpha,
                  double rmax) {
  RefPPR *st = new RefPPR;
  st->n = n;
  st->S = S;
  st->nparts = nparts;
  st->alpha = alpha;
  st->rmax = rmax;
  st->sources.assign(sources, sources + S);
  st->indicator.assign(n, -1);
  for (int i = 0; i < S; ++i) {
    st->row_index[sources[i]] = i;
    st->indicator[sources[i]] = 0;
  }
  // Column partition of Tree_u_NC.cpp:396-432.
  st->col_dim = n / nparts;
  int last = n - (nparts - 1) * st->col_dim;
  st->inner.assign(n, 0);
  for (int v = 0; v < n; ++v) {
    int b = v / st->col_dim;
    if (b >= nparts) b = nparts - 1;
    st->inner[v] = v - b * st->col_dim;
  }
  for (int b = 0; b < nparts; ++b) {
    RefDenseBlock &blk = st->tree.dense_mat_mapping[b];
    blk.rows = S;
    blk.cols = b == nparts - 1 ? last : st->col_dim;
    blk.v.assign((size_t)blk.rows * blk.cols, 0.0);
  }
  // Queue capacity of Tree_u_NC.cpp:454-488, bounded for small test graphs.
  long long upper = (long long)ceil(1 / rmax / alpha);
  long long cap = 2 * (upper + 2);
  long long bound = 64ll * n + 4096;
  if (cap > bound) cap = bound;
  for (int i = 0; i < S; ++i) {
    st->r.push_back((float *)calloc(n, sizeof(float)));
    st->p.push_back((float *)calloc(n, sizeof(float)));
    st->flags.push_back((bool *)calloc(n, sizeof(bool)));
    Queue q{(int *)malloc(sizeof(int) * cap), (int)cap, 0, 0};
    st->queues.push_back(q);
  }
  return st;
}

void ref_ppr_free(void *sp) {
  RefPPR *st = (RefPPR *)sp;
  for (int i = 0; i < st->S; ++i) {
    free(st->r[i]);
    free(st->p[i]);
    free(st->flags[i]);
    free(st->queues[i].arr);
  }
  delete st;
}

// One refresh + push. transpose selects the in-list variants (directed only).
void ref_ppr_step(void *sp, void *gp, int transpose, int iter, int dyn_start) {
  RefPPR *st = (RefPPR *)sp;
  RefGraph *g = (RefGraph *)gp;
  int S = st->S;
  float **r = st->r.data(), **p = st->p.data();
  bool **fl = st->flags.data();
  Queue *q = st->queues.data();
  if (!g->directed) {
    nodegree_DenseUndirected_Refresh_PPR_initialization(
        0, S, g->ug, st->rmax, st->alpha, st->sources, r, p, fl, q, iter, st->n,
        st->col_dim, st->nparts, st->inner, &st->tree, st->row_index,
        st->indicator, dyn_start);
    nodegree_DenseDynamicForwardPush(0, S, g->ug, st->rmax, st->alpha,
                                     st->sources, r, p, fl, q, st->row_index,
                                     st->col_dim, st->nparts, &st->tree,
                                     st->inner, st->indicator);
  } else if (!transpose) {
    nodegree_DenseDirected_Refresh_PPR_initialization(
        0, S, g->dg, st->rmax, st->rmax, st->alpha, st->sources, r, p, fl, q,
        st->col_dim, st->nparts, st->inner, iter, st->n, &st->tree, dyn_start);
    nodegree_DenseDirectedDynamicForwardPush(0, S, g->dg, st->rmax, st->rmax,
                                             st->alpha, st->sources, r, p, fl, q,
                                             st->col_dim, st->nparts, st->inner,
                                             &st->tree);
  } else {
    nodegree_DenseDirected_Refresh_PPR_initialization_Transpose(
        0, S, g->dg, st->rmax, st->rmax, st->alpha, st->sources, r, p, fl, q,
        st->col_dim, st->nparts, st->inner, iter, st->n, &st->tree, dyn_start);
    nodegree_DenseDirectedDynamicForwardPushTranspose(
        0, S, g->dg, st->rmax, st->rmax, st->alpha, st->sources, r, p, fl, q,
        st->col_dim, st->nparts, st->inner, &st->tree);
  }
}

// The same refresh + push, the way the reference's drivers run it
// (Code/Tree_u_NC.cpp:566-640): `threads` std::threads, each calling the
// entry points on its own contiguous range of sources.
void ref_ppr_step_mt(void *sp, void *gp, int transpose, int iter, int dyn_start, int threads) {
  RefPPR *st = (RefPPR *)sp;
  RefGraph *g = (RefGraph *)gp;
  const int S = st->S;
  if (threads < 1) threads = 1;
  if (threads > S) threads = S;
  float **r = st->r.data(), **p = st->p.data();
  bool **fl = st->flags.data();
  Queue *q = st->queues.data();
  vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    const int a = (int)((long long)S * t / threads), b = (int)((long long)S * (t + 1) / threads);
    pool.emplace_back([=]() {
      if (!g->directed) {
        nodegree_DenseUndirected_Refresh_PPR_initialization(
            a, b, g->ug, st->rmax, st->alpha, st->sources, r, p, fl, q, iter, st->n,
            st->col_dim, st->nparts, st->inner, &st->tree, st->row_index, st->indicator,
            dyn_start);
        nodegree_DenseDynamicForwardPush(a, b, g->ug, st->rmax, st->alpha, st->sources, r, p,
                                         fl, q, st->row_index, st->col_dim, st->nparts,
                                         &st->tree, st->inner, st->indicator);
      } else if (!transpose) {
        nodegree_DenseDirected_Refresh_PPR_initialization(
            a, b, g->dg, st->rmax, st->rmax, st->alpha, st->sources, r, p, fl, q, st->col_dim,
            st->nparts, st->inner, iter, st->n, &st->tree, dyn_start);
        nodegree_DenseDirectedDynamicForwardPush(a, b, g->dg, st->rmax, st->rmax, st->alpha,
                                                 st->sources, r, p, fl, q, st->col_dim,
                                                 st->nparts, st->inner, &st->tree);
      } else {
        nodegree_DenseDirected_Refresh_PPR_initialization_Transpose(
            a, b, g->dg, st->rmax, st->rmax, st->alpha, st->sources, r, p, fl, q, st->col_dim,
            st->nparts, st->inner, iter, st->n, &st->tree, dyn_start);
        nodegree_DenseDirectedDynamicForwardPushTranspose(a, b, g->dg, st->rmax, st->rmax,
                                                          st->alpha, st->sources, r, p, fl, q,
                                                          st->col_dim, st->nparts, st->inner,
                                                          &st->tree);
      }
    });
  }
  for (auto &th : pool) th.join();
}

// which: 0 residue, 1 reserve (|S| x N floats).
void ref_ppr_state(void *sp, int which, float *out) {
  RefPPR *st = (RefPPR *)sp;
  for (int i = 0; i < st->S; ++i)
    memcpy(out + (size_t)i * st->n, which ? st->p[i] : st->r[i],
           sizeof(float) * st->n);
}

// The accumulated dense_mat_mapping as |S| x N doubles.
void ref_ppr_dense(void *sp, double *out) {
  RefPPR *st = (RefPPR *)sp;
  for (int b = 0; b < st->nparts; ++b) {
    RefDenseBlock &blk = st->tree.dense_mat_mapping[b];
    for (int i = 0; i < blk.rows; ++i)
      for (int j = 0; j < blk.cols; ++j)
        out[(size_t)i * st->n + (size_t)b * st->col_dim + j] = blk(i, j);
  }
}

// The reference's log transform + lazy test of every block of the
// accumulated dense matrix: Log_sparse_matrix_entries[_LP] when with_norm is
// 0 (every block accepted), ..._with_norm_computation[_LP] otherwise, reading
// resid[b] as norm_B_Bid_difference_vec[b]. Outputs: the accepted log blocks
// (mat_mapping) as |S| x N doubles, the update record (-1: kept, iter:
// refreshed) and the nnz record.
void ref_log_blocks(void *sp, int lp, int with_norm, int iter, double delta,
                    const double *resid, double *accepted, int *record, long long *nnz) {
  RefPPR *st = (RefPPR *)sp;
  const int P = st->nparts;
  d_row_tree_mkl &t = st->tree;
  t.row_dim = st->S;
  t.norm_B_Bid_difference_vec.assign(resid, resid + P);
  st->nnz_record.resize(P, 0);
  unordered_map<int, vector<int>> vec_mapping;
  for (int b = 0; b < P; ++b) vec_mapping[b].resize(t.dense_mat_mapping[b].cols);
  vector<int> upd(P, 0);
  for (int b = 0; b < P; ++b) {
    if (!with_norm) {
      if (lp)
        Log_sparse_matrix_entries_LP(b, st->rmax, &t, vec_mapping, st->nnz_record);
      else
        Log_sparse_matrix_entries(b, st->rmax, &t, vec_mapping, st->nnz_record);
      upd[b] = iter;
    } else if (lp) {
      Log_sparse_matrix_entries_with_norm_computation_LP(b, st->rmax, &t, vec_mapping, upd, iter,
                                                         delta, st->S, 0, st->nnz_record);
    } else {
      Log_sparse_matrix_entries_with_norm_computation(b, st->rmax, &t, vec_mapping, upd, iter,
                                                      delta, st->S, 0, st->nnz_record);
    }
  }
  if (accepted) memset(accepted, 0, sizeof(double) * (size_t)st->S * st->n);
  for (int b = 0; b < P; ++b) {
    SparseMatrix<double, 0, int> &m = t.mat_mapping[b];
    if (accepted)
      for (int j = 0; j < m.ncols; ++j)
        for (int q = m.outer[j]; q < m.outer[j + 1]; ++q)
          accepted[(size_t)m.inner[q] * st->n + (size_t)b * st->col_dim + j] = m.val[q];
    if (record) record[b] = upd[b];
    if (nnz) nnz[b] = st->nnz_record[b];
  }
}

// Block b's accepted log matrix (mat_mapping[b], |S| x cols) as 0-based CSR:
// with null outputs, returns the entry count only.
long long ref_block_csr(void *sp, int b, int *rowptr, int *cols, double *vals) {
  RefPPR *st = (RefPPR *)sp;
  SparseMatrix<double, 0, int> &m = st->tree.mat_mapping[b];
  const long long nnz = (long long)m.val.size();
  if (!rowptr) return nnz;
  vector<int> cnt((size_t)st->S + 1, 0);
  for (int q = 0; q < (int)nnz; ++q) cnt[(size_t)m.inner[q] + 1]++;
  for (int i = 0; i < st->S; ++i) cnt[i + 1] += cnt[i];
  memcpy(rowptr, cnt.data(), sizeof(int) * ((size_t)st->S + 1));
  for (int j = 0; j < m.ncols; ++j)
    for (int q = m.outer[j]; q < m.outer[j + 1]; ++q) {
      const int pos = cnt[m.inner[q]]++;
      cols[pos] = j;
      vals[pos] = m.val[q];
    }
  return nnz;
}

}  // extern "C"
