"""Python binding (ctypes) of libtsvd_gb300.so — the C-ABI in include/tsvd.h.

The library is the product: every compute call goes to sm_103a kernels. If
the shared object is missing this module raises at import time instead of
falling back to anything else.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtsvd_gb300.so")

TRANSFORM_LOG10_NC, TRANSFORM_LOG10_LP, TRANSFORM_LN_N = 0, 1, 2
DIRTY_REFERENCE, DIRTY_FROBENIUS, DIRTY_ALL = 0, 1, 2
ROOT_SQRT_SIGMA, ROOT_U = 0, 1
REFRESH_EXACT, REFRESH_INTDIV = 0, 1
FORM_MIXED, FORM_PLAIN = 0, 1
BLOCKS_DENSE, BLOCKS_SPARSE, BLOCKS_AUTO = 0, 1, 2

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "device error",
          4: "timeout", 5: "bad state", 6: "i/o error", 7: "numeric error"}


class TsvdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [
        ("n_vertices", ctypes.c_int32), ("directed", ctypes.c_int32),
        ("n_sources", ctypes.c_int32), ("sources", ctypes.POINTER(ctypes.c_int32)),
        ("alpha", ctypes.c_double), ("rmax", ctypes.c_double),
        ("n_parts", ctypes.c_int32), ("hierarchy_n", ctypes.c_int32),
        ("rank_d", ctypes.c_int32), ("oversample", ctypes.c_int32),
        ("passes_q", ctypes.c_int32), ("dynamic_ppr_start_iter", ctypes.c_int32),
        ("lazy_update_start_iter", ctypes.c_int32), ("delta", ctypes.c_double),
        ("transform", ctypes.c_int32), ("dirty_rule", ctypes.c_int32),
        ("dirty_frac", ctypes.c_double), ("root_scaling", ctypes.c_int32),
        ("refresh_mode", ctypes.c_int32), ("seed", ctypes.c_uint64),
        ("device", ctypes.c_int32), ("max_push_rounds", ctypes.c_int32),
        ("push_levels", ctypes.c_int32), ("push_ratio", ctypes.c_double),
        ("push_cofrac", ctypes.c_double), ("lp_right_factor", ctypes.c_int32),
        ("ppr_host_reserve", ctypes.c_int32), ("form", ctypes.c_int32),
        ("block_path", ctypes.c_int32), ("plain_frontier_cap", ctypes.c_int32),
        ("push_hub_degree", ctypes.c_int32),
    ]


class StepStats(ctypes.Structure):
    _fields_ = [
        ("iter", ctypes.c_int32), ("skipped", ctypes.c_int32),
        ("edges_inserted", ctypes.c_int64), ("push_rounds", ctypes.c_int64),
        ("pushes", ctypes.c_int64), ("push_edge_updates", ctypes.c_int64),
        ("dirty_blocks", ctypes.c_int32), ("factorized_blocks", ctypes.c_int32),
        ("merged_nodes", ctypes.c_int32),
        ("ms_insert", ctypes.c_double), ("ms_refresh", ctypes.c_double),
        ("ms_push", ctypes.c_double), ("ms_log", ctypes.c_double),
        ("ms_frpca", ctypes.c_double), ("ms_merge", ctypes.c_double),
        ("ms_total", ctypes.c_double), ("push_items", ctypes.c_int64),
        ("ms_push_kernels", ctypes.c_double), ("ms_materialize_kernel", ctypes.c_double),
        ("push_item_edges", ctypes.c_int64), ("ms_lp", ctypes.c_double),
        ("eig_sweeps_frpca", ctypes.c_int32), ("eig_sweeps_merge", ctypes.c_int32),
        ("merge_subspace_iters", ctypes.c_int32), ("eig_refine_sweeps", ctypes.c_int32),
        ("sparse_blocks", ctypes.c_int32), ("tune_density", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p

_SIGS = {
    "tsvd_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "tsvd_last_error": (ctypes.c_char_p, []),
    "tsvd_version": (ctypes.c_char_p, []),
    "tsvd_launch_count": (ctypes.c_int64, []),
    "tsvd_session_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "tsvd_session_set_form": (ctypes.c_int, [_vp, ctypes.c_int32]),
    "tsvd_session_footprint": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_int64,
                                              ctypes.POINTER(ctypes.c_int64)]),
    "tsvd_server_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                          ctypes.POINTER(_vp)]),
    "tsvd_server_add_tenant": (ctypes.c_int, [_vp, ctypes.POINTER(Config), ctypes.c_int64,
                                              ctypes.POINTER(ctypes.c_int32)]),
    "tsvd_server_remove_tenant": (ctypes.c_int, [_vp, ctypes.c_int32]),
    "tsvd_server_submit_update": (ctypes.c_int, [_vp, ctypes.c_int32, _i32p, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_int64)]),
    "tsvd_server_submit_query": (ctypes.c_int, [_vp, ctypes.c_int32, _f64p,
                                                ctypes.POINTER(ctypes.c_int64)]),
    "tsvd_server_wait": (ctypes.c_int, [_vp, ctypes.c_int64, _f64p, _f64p]),
    "tsvd_server_drain": (ctypes.c_int, [_vp]),
    "tsvd_server_stats": (ctypes.c_int, [_vp, ctypes.c_void_p]),
    "tsvd_server_session": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(_vp)]),
    "tsvd_server_destroy": (ctypes.c_int, [_vp]),
    "tsvd_set_frpca_seed": (None, [ctypes.c_uint64]),
    "tsvd_frpca": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _i64p, _i32p,
                                  _f64p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_uint64, _f64p, _f64p, _f64p]),
    "tsvd_frpca_fp32": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _i64p,
                                       _i32p, _f64p, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_uint64, _f64p, _f64p, _f64p]),
    "tsvd_frpca_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _i64p,
                                          _i32p, _f64p, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_uint64, _f64p, _f64p, _f64p]),
    "tsvd_merge_svd": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _f64p, ctypes.c_int32,
                                      _f64p, _f64p]),
    "tsvd_config_default": (None, [ctypes.POINTER(Config)]),
    "tsvd_session_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_vp)]),
    "tsvd_session_destroy": (ctypes.c_int, [_vp]),
    "tsvd_session_step": (ctypes.c_int, [_vp, _i32p, ctypes.c_int64]),
    "tsvd_session_step_device": (ctypes.c_int, [_vp, _vp, ctypes.c_int64]),
    "tsvd_session_run": (ctypes.c_int, [_vp, _i32p, _i64p, ctypes.c_int32, _f64p,
                                        ctypes.POINTER(StepStats)]),
    "tsvd_session_run_device": (ctypes.c_int, [_vp, _vp, _i64p, ctypes.c_int32, _f64p,
                                               ctypes.POINTER(StepStats)]),
    "tsvd_session_embedding": (ctypes.c_int, [_vp, _f64p]),
    "tsvd_session_embedding_device": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "tsvd_session_last_stats": (ctypes.c_int, [_vp, ctypes.POINTER(StepStats)]),
    "tsvd_graph_insert": (ctypes.c_int, [_vp, _i32p, ctypes.c_int64]),
    "tsvd_ppr_refresh": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32]),
    "tsvd_ppr_push": (ctypes.c_int, [_vp, ctypes.c_int32]),
    "tsvd_blocks_materialize": (ctypes.c_int, [_vp, ctypes.c_int32, _u8p]),
    "tsvd_blocks_factorize": (ctypes.c_int, [_vp, ctypes.c_int32]),
    "tsvd_tree_merge": (ctypes.c_int, [_vp]),
    "tsvd_graph_degrees": (ctypes.c_int, [_vp, ctypes.c_int32, _i32p, _i32p]),
    "tsvd_graph_adjacency": (ctypes.c_int, [_vp, ctypes.c_int32, _i64p, _i32p, ctypes.c_int64]),
    "tsvd_ppr_state": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, _f32p]),
    "tsvd_ppr_state_rows": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32, _i32p,
                                           ctypes.c_int32, _f32p]),
    "tsvd_block_info": (ctypes.c_int, [_vp, _f64p, _f64p, _f64p, _i64p, _u8p]),
    "tsvd_tree_factor": (ctypes.c_int, [_vp, ctypes.c_int32, _f64p, _f64p]),
    "tsvd_block_dense": (ctypes.c_int, [_vp, ctypes.c_int32, _f32p]),
    "tsvd_rmat_edges": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                       ctypes.c_uint64, _i32p]),
    "tsvd_snapshot_sizes": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _i64p]),
    "tsvd_sample_sources": (ctypes.c_int, [ctypes.c_int32, _i32p, ctypes.c_int64, ctypes.c_int32,
                                           ctypes.c_uint64, _i32p]),
    "tsvd_read_edge_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32,
                                           ctypes.POINTER(_i32p), _i64p]),
    "tsvd_free": (None, [_vp]),
    "tsvd_write_edge_file_binary": (ctypes.c_int, [ctypes.c_char_p, _i32p, ctypes.c_int64]),
    "tsvd_gaussian": (ctypes.c_float, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32]),
    "frPCA": (None, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int]),
    "tsvd_lp_right_factor": (ctypes.c_int, [_vp, _f32p]),
    "tsvd_lp_scores": (ctypes.c_int, [_vp, _i32p, ctypes.c_int64, ctypes.c_int32, _f64p]),
    "tsvd_lp_precision": (ctypes.c_int, [_f64p, _u8p, ctypes.c_int64, ctypes.c_int64, _f64p]),
}

EXPORTS = sorted(_SIGS)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtsvd_gb300.so is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st):
    if st != 0:
        raise TsvdError(st, lib().tsvd_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(t)


# ----------------------------------------------------------------- synthetic inputs
def rmat_edges(n, m, a=0.57, b=0.19, c=0.19, directed=False, seed=20231):
    out = np.empty((int(m), 2), np.int32)
    _check(lib().tsvd_rmat_edges(int(n), int(m), a, b, c, int(directed), seed, _p(out, _i32p)))
    return out


def snapshot_sizes(m, n_snapshots, first_frac):
    out = np.zeros(int(n_snapshots), np.int64)
    _check(lib().tsvd_snapshot_sizes(int(m), int(n_snapshots), float(first_frac), _p(out, _i64p)))
    return out


def sample_sources(n, edges, k, seed=20231):
    e = np.ascontiguousarray(edges, dtype=np.int32)
    out = np.empty(int(k), np.int32)
    _check(lib().tsvd_sample_sources(int(n), _p(e, _i32p), e.shape[0], int(k), seed, _p(out, _i32p)))
    return out


def read_edge_file(path, compat_dup_last=False):
    ptr = _i32p()
    m = ctypes.c_int64()
    _check(lib().tsvd_read_edge_file(path.encode(), int(compat_dup_last), ctypes.byref(ptr),
                                     ctypes.byref(m)))
    try:
        arr = np.ctypeslib.as_array(ptr, shape=(m.value * 2,)).copy() if m.value else \
            np.zeros(0, np.int32)
    finally:
        lib().tsvd_free(ptr)
    return arr.reshape(-1, 2)


def write_edge_file_binary(path, edges):
    e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    _check(lib().tsvd_write_edge_file_binary(os.fsencode(path), _p(e, _i32p), e.shape[0]))


def gaussian(seed, stream, row, col):
    return lib().tsvd_gaussian(seed, stream, row, col)


def lp_precision(scores, positive, k):
    sc = np.ascontiguousarray(scores, dtype=np.float64)
    pos = np.ascontiguousarray(positive, dtype=np.uint8)
    out = ctypes.c_double()
    _check(lib().tsvd_lp_precision(_p(sc, _f64p), _p(pos, _u8p), len(sc), int(k),
                                   ctypes.byref(out)))
    return out.value


def launch_count():
    """Kernels launched by the library so far in this process."""
    return lib().tsvd_launch_count()


def frpca(csr_indptr, csr_indices, csr_data, shape, k, q, seed=20231, index_base=0,
          noalloc=False, fp32=False):
    """Randomized SVD of a CSR matrix; returns U (m x k), S (k, descending), V (n x k).
    noalloc=True calls tsvd_frpca_noalloc (no allocation, bounded sizes);
    fp32=True calls tsvd_frpca_fp32 (FP32 SpMM products)."""
    m, n = shape
    rp = np.ascontiguousarray(csr_indptr, dtype=np.int64)
    ci = np.ascontiguousarray(csr_indices, dtype=np.int32)
    va = np.ascontiguousarray(csr_data, dtype=np.float64)
    U = np.zeros((k, m), np.float64)
    S = np.zeros(k, np.float64)
    V = np.zeros((k, n), np.float64)
    fn = (lib().tsvd_frpca_noalloc if noalloc else
          lib().tsvd_frpca_fp32 if fp32 else lib().tsvd_frpca)
    _check(fn(m, n, len(va), _p(rp, _i64p), _p(ci, _i32p), _p(va, _f64p), index_base, k, q,
              seed, _p(U, _f64p), _p(S, _f64p), _p(V, _f64p)))
    return U.T.copy(), S, V.T.copy()


def merge_svd(M, d):
    """tsvd_merge_svd: (U_d diag(s_d) (rows x d), s_d) of a dense matrix."""
    M = np.asfortranarray(M, dtype=np.float64)
    rows, cols = M.shape
    US = np.zeros((rows, d), np.float64, order="F")
    sig = np.zeros(d, np.float64)
    _check(lib().tsvd_merge_svd(rows, cols, M.ctypes.data_as(_f64p), d, US.ctypes.data_as(_f64p),
                                _p(sig, _f64p)))
    return US, sig


# ----------------------------------------------------------------- session
def make_config(n_vertices, sources, directed=False, alpha=0.5, rmax=1e-7, n_parts=64,
                hierarchy_n=2, rank_d=128, oversample=5, passes_q=12, dynamic_ppr_start_iter=100,
                lazy_update_start_iter=100, delta=0.3, transform=TRANSFORM_LOG10_NC,
                dirty_rule=DIRTY_REFERENCE, dirty_frac=0.01, root_scaling=ROOT_SQRT_SIGMA,
                refresh_mode=REFRESH_EXACT, seed=20231, device=0, max_push_rounds=0,
                push_levels=1, push_ratio=8.0, push_cofrac=0.85, lp_right_factor=False,
                ppr_host_reserve=False, form=FORM_MIXED, block_path=BLOCKS_DENSE,
                plain_frontier_cap=0, push_hub_degree=0):
    """A tsvd_config; `sources` (int32, contiguous) must outlive it."""
    c = Config()
    lib().tsvd_config_default(ctypes.byref(c))
    c.n_vertices, c.directed = int(n_vertices), int(directed)
    c.n_sources = len(sources)
    c.sources = _p(sources, _i32p)
    c.alpha, c.rmax = float(alpha), float(rmax)
    c.n_parts, c.hierarchy_n = int(n_parts), int(hierarchy_n)
    c.rank_d, c.oversample, c.passes_q = int(rank_d), int(oversample), int(passes_q)
    c.dynamic_ppr_start_iter = int(dynamic_ppr_start_iter)
    c.lazy_update_start_iter = int(lazy_update_start_iter)
    c.delta = float(delta)
    c.transform, c.dirty_rule, c.dirty_frac = int(transform), int(dirty_rule), float(dirty_frac)
    c.root_scaling, c.refresh_mode = int(root_scaling), int(refresh_mode)
    c.seed, c.device, c.max_push_rounds = int(seed), int(device), int(max_push_rounds)
    c.push_levels, c.push_ratio = int(push_levels), float(push_ratio)
    c.push_cofrac = float(push_cofrac)
    c.lp_right_factor = int(bool(lp_right_factor))
    c.ppr_host_reserve = int(bool(ppr_host_reserve))
    c.form = int(form)
    c.block_path = int(block_path)
    c.plain_frontier_cap = int(plain_frontier_cap)
    c.push_hub_degree = int(push_hub_degree)
    return c


def footprint(n_vertices, sources, expected_edges, **kw):
    """tsvd_session_footprint: estimated device bytes of such a session."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    c = make_config(n_vertices, src, **kw)
    out = ctypes.c_int64()
    _check(lib().tsvd_session_footprint(ctypes.byref(c), int(expected_edges), ctypes.byref(out)))
    return out.value


class Session:
    """A device-resident Tree-SVD state: graph store, PPR store, block factors, tree."""

    def __init__(self, n_vertices, sources, directed=False, alpha=0.5, rmax=1e-7, n_parts=64,
                 hierarchy_n=2, rank_d=128, oversample=5, passes_q=12,
                 dynamic_ppr_start_iter=100, lazy_update_start_iter=100, delta=0.3,
                 transform=TRANSFORM_LOG10_NC, dirty_rule=DIRTY_REFERENCE, dirty_frac=0.01,
                 root_scaling=ROOT_SQRT_SIGMA, refresh_mode=REFRESH_EXACT, seed=20231, device=0,
                 max_push_rounds=0, push_levels=1, push_ratio=8.0, push_cofrac=0.85,
                 lp_right_factor=False, ppr_host_reserve=False, form=FORM_MIXED,
                 block_path=BLOCKS_DENSE, plain_frontier_cap=0, push_hub_degree=0):
        self.sources = np.ascontiguousarray(sources, dtype=np.int32)
        c = make_config(n_vertices, self.sources, directed, alpha, rmax, n_parts, hierarchy_n,
                        rank_d, oversample, passes_q, dynamic_ppr_start_iter,
                        lazy_update_start_iter, delta, transform, dirty_rule, dirty_frac,
                        root_scaling, refresh_mode, seed, device, max_push_rounds, push_levels,
                        push_ratio, push_cofrac, lp_right_factor, ppr_host_reserve, form,
                        block_path, plain_frontier_cap, push_hub_degree)
        self.cfg = c
        self.n, self.S, self.d = c.n_vertices, c.n_sources, c.rank_d
        self.n_parts, self.h, self.directed = c.n_parts, c.hierarchy_n, bool(directed)
        self._h = _vp()
        _check(lib().tsvd_session_create(ctypes.byref(c), ctypes.byref(self._h)))

    @classmethod
    def _view(cls, handle, cfg, sources):
        """A non-owning Session around a handle (a server tenant's session)."""
        self = cls.__new__(cls)
        self.sources = sources
        self.cfg = cfg
        self.n, self.S, self.d = cfg.n_vertices, cfg.n_sources, cfg.rank_d
        self.n_parts, self.h, self.directed = cfg.n_parts, cfg.hierarchy_n, bool(cfg.directed)
        self._h = handle
        self._owned = False
        return self


    _owned = True

    def close(self):
        if getattr(self, "_h", None) and self._owned:
            lib().tsvd_session_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # whole snapshot
    def step(self, edges):
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        _check(lib().tsvd_session_step(self._h, _p(e, _i32p), e.shape[0]))
        return self.stats()

    def step_device(self, ptr, m):
        _check(lib().tsvd_session_step_device(self._h, _vp(ptr), int(m)))

    def run(self, snapshots, embeddings=True):
        """Several snapshots in one call, the factor stage of each overlapped
        with the next one's push (tsvd_session_run). `snapshots` is a list of
        (m, 2) edge arrays. Returns (list of stats dicts, embeddings array of
        shape (len(snapshots), |S|, d) or None)."""
        snaps = [np.ascontiguousarray(e, dtype=np.int32).reshape(-1, 2) for e in snapshots]
        off = np.zeros(len(snaps) + 1, np.int64)
        off[1:] = np.cumsum([len(e) for e in snaps])
        edges = np.ascontiguousarray(np.concatenate(snaps) if snaps else np.zeros((0, 2), np.int32))
        return self._run(lambda *a: lib().tsvd_session_run(self._h, _p(edges, _i32p), *a),
                         off, embeddings)

    def run_device(self, ptr, offsets, embeddings=True):
        """tsvd_session_run_device: snapshot k is the device pairs
        [offsets[k], offsets[k+1]) at `ptr`."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        return self._run(lambda *a: lib().tsvd_session_run_device(self._h, _vp(ptr), *a),
                         off, embeddings)

    def _run(self, call, off, embeddings):
        count = len(off) - 1
        stats = (StepStats * max(count, 1))()
        emb = np.zeros((count, self.S, self.d), np.float64) if embeddings else None
        _check(call(_p(off, _i64p), count, _p(emb, _f64p) if embeddings else None, stats))
        return [stats[k].as_dict() for k in range(count)], emb

    def embedding(self):
        out = np.zeros((self.S, self.d), np.float64)
        _check(lib().tsvd_session_embedding(self._h, _p(out, _f64p)))
        return out

    def embedding_device_ptr(self):
        p = _vp()
        _check(lib().tsvd_session_embedding_device(self._h, ctypes.byref(p)))
        return p.value

    def set_form(self, form):
        """FORM_MIXED or FORM_PLAIN for the following snapshots."""
        _check(lib().tsvd_session_set_form(self._h, int(form)))

    def stream(self):
        p = _vp()
        _check(lib().tsvd_session_stream(self._h, ctypes.byref(p)))
        return p.value

    def stats(self):
        st = StepStats()
        _check(lib().tsvd_session_last_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    # granular stages
    def graph_insert(self, edges):
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        _check(lib().tsvd_graph_insert(self._h, _p(e, _i32p), e.shape[0]))

    def ppr_refresh(self, iter, transpose=False):
        _check(lib().tsvd_ppr_refresh(self._h, int(iter), int(transpose)))

    def ppr_push(self, transpose=False):
        _check(lib().tsvd_ppr_push(self._h, int(transpose)))

    def blocks_materialize(self, iter):
        d = np.zeros(self.n_parts, np.uint8)
        _check(lib().tsvd_blocks_materialize(self._h, int(iter), _p(d, _u8p)))
        return d

    def blocks_factorize(self, iter):
        _check(lib().tsvd_blocks_factorize(self._h, int(iter)))

    def tree_merge(self):
        _check(lib().tsvd_tree_merge(self._h))

    # inspection
    def degrees(self, dir=0):
        d = np.zeros(self.n, np.int32)
        f = np.zeros(self.n, np.int32)
        _check(lib().tsvd_graph_degrees(self._h, dir, _p(d, _i32p), _p(f, _i32p)))
        return d, f

    def adjacency(self, dir=0):
        d, _ = self.degrees(dir)
        tot = int(d.astype(np.int64).sum())
        off = np.zeros(self.n + 1, np.int64)
        nb = np.zeros(max(tot, 1), np.int32)
        _check(lib().tsvd_graph_adjacency(self._h, dir, _p(off, _i64p), _p(nb, _i32p), len(nb)))
        return off, nb[:tot]

    def ppr_state(self, transpose=False, which=1):
        out = np.zeros((self.S, self.n), np.float32)
        _check(lib().tsvd_ppr_state(self._h, int(transpose), int(which), _p(out, _f32p)))
        return out

    def ppr_state_rows(self, rows, transpose=False, which=1):
        """State of the listed source rows only (len(rows) x N float32)."""
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        out = np.zeros((len(rows), self.n), np.float32)
        _check(lib().tsvd_ppr_state_rows(self._h, int(transpose), int(which), _p(rows, _i32p),
                                         len(rows), _p(out, _f32p)))
        return out

    def block_info(self):
        P = self.n_parts
        a, dd, r = (np.zeros(P) for _ in range(3))
        nnz = np.zeros(P, np.int64)
        dirty = np.zeros(P, np.uint8)
        _check(lib().tsvd_block_info(self._h, _p(a, _f64p), _p(dd, _f64p), _p(r, _f64p),
                                     _p(nnz, _i64p), _p(dirty, _u8p)))
        return {"norm": a, "norm_diff": dd, "resid": r, "nnz": nnz, "dirty": dirty}

    def tree_factor(self, node):
        out = np.zeros((self.S, self.d), np.float64)
        sig = np.zeros(self.d, np.float64)
        _check(lib().tsvd_tree_factor(self._h, int(node), _p(out, _f64p), _p(sig, _f64p)))
        return out, sig

    # link prediction
    def lp_right_factor(self):
        out = np.zeros((self.n, self.d), np.float32)
        _check(lib().tsvd_lp_right_factor(self._h, _p(out, _f32p)))
        return out

    def lp_scores(self, pairs, degree_scaled=False):
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        out = np.zeros(pr.shape[0], np.float64)
        _check(lib().tsvd_lp_scores(self._h, _p(pr, _i32p), pr.shape[0], int(degree_scaled),
                                    _p(out, _f64p)))
        return out

    def block_dense(self, b):
        cd = self.n // self.n_parts
        nb = self.n - (self.n_parts - 1) * cd if b == self.n_parts - 1 else cd
        out = np.zeros((self.S, nb), np.float32)
        _check(lib().tsvd_block_dense(self._h, int(b), _p(out, _f32p)))
        return out

    @property
    def leaf_start(self):
        tot, pw = 0, 1
        levels = 1
        t = self.n_parts
        while t > 1:
            t //= self.h
            levels += 1
        for _ in range(levels):
            tot += pw
            pw *= self.h
        return tot - self.n_parts


# ----------------------------------------------------------------- serving
class ServerStats(ctypes.Structure):
    _fields_ = [("updates", ctypes.c_int64), ("edges", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("edges_per_s", ctypes.c_double), ("hbm_budget", ctypes.c_int64),
                ("hbm_charged", ctypes.c_int64), ("tenants", ctypes.c_int32)]


class Server:
    """tsvd_server: tenants resident on one GPU, requests taken as they arrive."""

    def __init__(self, device=0, hbm_budget_bytes=0, slots=4):
        self._h = _vp()
        _check(lib().tsvd_server_create(int(device), int(hbm_budget_bytes), int(slots),
                                        ctypes.byref(self._h)))
        self._tenants = {}
        self._pending = {}  # request id -> (kind, buffer kept alive)

    def add_tenant(self, n_vertices, sources, expected_edges, **kw):
        src = np.ascontiguousarray(sources, dtype=np.int32)
        c = make_config(n_vertices, src, **kw)
        t = ctypes.c_int32()
        _check(lib().tsvd_server_add_tenant(self._h, ctypes.byref(c), int(expected_edges),
                                            ctypes.byref(t)))
        self._tenants[t.value] = (c, src)
        return t.value

    def remove_tenant(self, tenant):
        _check(lib().tsvd_server_remove_tenant(self._h, int(tenant)))
        self._tenants.pop(tenant, None)

    def submit_update(self, tenant, edges):
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        r = ctypes.c_int64()
        _check(lib().tsvd_server_submit_update(self._h, int(tenant), _p(e, _i32p), e.shape[0],
                                               ctypes.byref(r)))
        self._pending[r.value] = ("update", None)
        return r.value

    def submit_query(self, tenant):
        c, src = self._tenants[tenant]
        out = np.zeros((c.n_sources, c.rank_d), np.float64)
        r = ctypes.c_int64()
        _check(lib().tsvd_server_submit_query(self._h, int(tenant), _p(out, _f64p),
                                              ctypes.byref(r)))
        self._pending[r.value] = ("query", out)
        return r.value

    def wait(self, request):
        """(latency ms, service ms, embedding for queries or None)."""
        lat, svc = ctypes.c_double(), ctypes.c_double()
        kind, buf = self._pending.pop(request, (None, None))
        _check(lib().tsvd_server_wait(self._h, int(request), ctypes.byref(lat), ctypes.byref(svc)))
        return lat.value, svc.value, buf

    def drain(self):
        _check(lib().tsvd_server_drain(self._h))

    def stats(self):
        st = ServerStats()
        _check(lib().tsvd_server_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def session(self, tenant):
        """A non-owning Session view of the tenant (inspection between requests)."""
        h = _vp()
        _check(lib().tsvd_server_session(self._h, int(tenant), ctypes.byref(h)))
        c, src = self._tenants[tenant]
        return Session._view(h, c, src)

    def close(self):
        if getattr(self, "_h", None):
            lib().tsvd_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
