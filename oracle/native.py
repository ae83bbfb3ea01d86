"""ctypes bindings for the CPU oracle (oracle/liboracle_ppr.so) and for the
reference-compiled pin library (oracle/_ref/libtsvd_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker, never by the product path.
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(HERE, "liboracle_ppr.so")
_REF_SO = os.path.join(HERE, "_ref", "libtsvd_ref.so")

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)


def build():
    subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")])


def build_ref():
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])


def _ptr(a, t):
    return a.ctypes.data_as(t)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_ORACLE_SO):
            build()
        L = ctypes.CDLL(_ORACLE_SO)
        L.or_graph_new.restype = ctypes.c_void_p
        L.or_graph_new.argtypes = [ctypes.c_int32, ctypes.c_int32]
        L.or_graph_free.argtypes = [ctypes.c_void_p]
        L.or_graph_insert.restype = ctypes.c_int
        L.or_graph_insert.argtypes = [ctypes.c_void_p, _i32p, ctypes.c_int64]
        L.or_graph_degrees.restype = ctypes.c_int
        L.or_graph_degrees.argtypes = [ctypes.c_void_p, ctypes.c_int32, _i32p, _i32p]
        L.or_graph_adjacency.restype = ctypes.c_int64
        L.or_graph_adjacency.argtypes = [ctypes.c_void_p, ctypes.c_int32, _i64p, _i32p]
        L.or_ppr_new.restype = ctypes.c_void_p
        L.or_ppr_new.argtypes = [ctypes.c_int32, ctypes.c_int32, _i32p]
        L.or_ppr_free.argtypes = [ctypes.c_void_p]
        L.or_ppr_residue.restype = _f32p
        L.or_ppr_residue.argtypes = [ctypes.c_void_p]
        L.or_ppr_reserve.restype = _f32p
        L.or_ppr_reserve.argtypes = [ctypes.c_void_p]
        L.or_ppr_pushes.restype = ctypes.c_int64
        L.or_ppr_pushes.argtypes = [ctypes.c_void_p]
        L.or_ppr_edge_updates.restype = ctypes.c_int64
        L.or_ppr_edge_updates.argtypes = [ctypes.c_void_p]
        L.or_ppr_refresh.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int32, ctypes.c_int32]
        L.or_ppr_push.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_int32]
        L.or_rmat_edges.restype = ctypes.c_int
        L.or_rmat_edges.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                    ctypes.c_uint64, ctypes.c_int32, _i32p]
        L.or_sample_sources.restype = ctypes.c_int
        L.or_sample_sources.argtypes = [ctypes.c_int32, _i32p, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_uint64, _i32p]
        L.or_write_edges_text.restype = ctypes.c_int
        L.or_write_edges_text.argtypes = [ctypes.c_char_p, _i32p, ctypes.c_int64]
        _lib = L
    return _lib


def rmat_edges(n, m, a=0.57, b=0.19, c=0.19, directed=True, seed=20231, threads=None):
    """The seeded R-MAT edge list (m x 2 int32, timestamp order) drawn by the
    oracle's own generator (oracle_synth.c); identical to the product's."""
    out = np.zeros((int(m), 2), np.int32)
    rc = lib().or_rmat_edges(int(n), int(m), a, b, c, int(bool(directed)), int(seed),
                             int(threads or os.cpu_count() or 1), _ptr(out, _i32p))
    if rc != 0:
        raise RuntimeError("or_rmat_edges failed (%d)" % rc)
    return out


def snapshot_sizes(m, count, first_frac):
    """First snapshot round(first_frac * m) edges, the rest split evenly (the
    earlier deltas take the remainder)."""
    first = m if count == 1 else int(np.floor(first_frac * m + 0.5))
    rest = m - first
    k = count - 1
    return [first] + [rest // k + (1 if i < rest % k else 0) for i in range(k)]


def sample_sources(n, edges, k, seed=20231):
    e = np.ascontiguousarray(edges, np.int32)
    out = np.zeros(int(k), np.int32)
    if lib().or_sample_sources(int(n), _ptr(e, _i32p), len(e), int(k), int(seed),
                               _ptr(out, _i32p)) != 0:
        raise RuntimeError("or_sample_sources failed")
    return out


def write_edges_text(path, edges):
    e = np.ascontiguousarray(edges, np.int32)
    if lib().or_write_edges_text(path.encode(), _ptr(e, _i32p), len(e)) != 0:
        raise OSError("cannot write %s" % path)


class OracleGraph:
    """Reference graph store semantics (Graph_dynamic.h): insertion-ordered lists."""

    def __init__(self, n, directed):
        self.n, self.directed = int(n), int(directed)
        self.h = lib().or_graph_new(self.n, self.directed)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_graph_free(self.h)
            self.h = None

    def insert(self, edges):
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        rc = lib().or_graph_insert(self.h, _ptr(e, _i32p), e.shape[0])
        if rc != 0:
            raise ValueError("oracle graph insert failed (%d)" % rc)

    def degrees(self, dir=0):
        d = np.zeros(self.n, np.int32)
        f = np.zeros(self.n, np.int32)
        lib().or_graph_degrees(self.h, dir, _ptr(d, _i32p), _ptr(f, _i32p))
        return d, f

    def adjacency(self, dir=0):
        tot = lib().or_graph_adjacency(self.h, dir, None, None)
        off = np.zeros(self.n + 1, np.int64)
        nb = np.zeros(max(tot, 1), np.int32)
        lib().or_graph_adjacency(self.h, dir, _ptr(off, _i64p), _ptr(nb, _i32p))
        return off, nb[:tot]


class OraclePPR:
    """Per-source FIFO push state (float residue/reserve, |S| x N)."""

    def __init__(self, n, sources):
        self.n = int(n)
        self.sources = np.ascontiguousarray(sources, dtype=np.int32)
        self.s = len(self.sources)
        self.h = lib().or_ppr_new(self.n, self.s, _ptr(self.sources, _i32p))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_ppr_free(self.h)
            self.h = None

    def refresh(self, g, dir, iter, dyn_start, alpha, rmax, intdiv=False, threads=1):
        lib().or_ppr_refresh(self.h, g.h, dir, iter, dyn_start, alpha, rmax, int(intdiv), threads)

    def push(self, g, dir, alpha, rmax, threads=1):
        lib().or_ppr_push(self.h, g.h, dir, alpha, rmax, threads)
        return lib().or_ppr_pushes(self.h), lib().or_ppr_edge_updates(self.h)

    def residue(self):
        p = lib().or_ppr_residue(self.h)
        return np.ctypeslib.as_array(p, shape=(self.s, self.n)).copy()

    def reserve(self):
        p = lib().or_ppr_reserve(self.h)
        return np.ctypeslib.as_array(p, shape=(self.s, self.n)).copy()


# ---------------------------------------------------------------- reference pin
_ref = None


def ref_available():
    return os.path.exists(_REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(_REF_SO)
        L.ref_graph_new.restype = ctypes.c_void_p
        L.ref_graph_new.argtypes = [ctypes.c_int, ctypes.c_int]
        L.ref_graph_insert_file.restype = ctypes.c_longlong
        L.ref_graph_insert_file.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.ref_graph_degrees.argtypes = [ctypes.c_void_p, ctypes.c_int, _i32p, _i32p]
        L.ref_graph_adjacency.restype = ctypes.c_longlong
        L.ref_graph_adjacency.argtypes = [ctypes.c_void_p, ctypes.c_int, _i64p, _i32p]
        L.ref_ppr_new.restype = ctypes.c_void_p
        L.ref_ppr_new.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_double]
        L.ref_ppr_free.argtypes = [ctypes.c_void_p]
        L.ref_ppr_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int]
        L.ref_ppr_state.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
        L.ref_ppr_dense.argtypes = [ctypes.c_void_p, _f64p]
        L.ref_log_blocks.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, _f64p, _f64p, _i32p, _i64p]
        L.ref_ppr_step_mt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ref_block_csr.restype = ctypes.c_longlong
        L.ref_block_csr.argtypes = [ctypes.c_void_p, ctypes.c_int, _i32p, _i32p, _f64p]
        _ref = L
    return _ref


def write_edge_file(path, edges, trailing_newline=True):
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    body = "\n".join("%d %d" % (a, b) for a, b in e)
    with open(path, "w") as f:
        f.write(body + ("\n" if trailing_newline and len(e) else ""))


class RefGraph:
    """The reference's UGraph/Graph, fed through its own file reader."""

    def __init__(self, n, directed):
        self.n, self.directed = int(n), int(directed)
        self.h = ref_lib().ref_graph_new(self.n, self.directed)

    def insert_file(self, path):
        return ref_lib().ref_graph_insert_file(self.h, path.encode())

    def insert(self, edges, trailing_newline=True):
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            name = f.name
        try:
            write_edge_file(name, edges, trailing_newline)
            return self.insert_file(name)
        finally:
            os.unlink(name)

    def degrees(self, dir=0):
        d = np.zeros(self.n, np.int32)
        f = np.zeros(self.n, np.int32)
        ref_lib().ref_graph_degrees(self.h, dir, _ptr(d, _i32p), _ptr(f, _i32p))
        return d, f

    def adjacency(self, dir=0):
        tot = ref_lib().ref_graph_adjacency(self.h, dir, None, None)
        off = np.zeros(self.n + 1, np.int64)
        nb = np.zeros(max(tot, 1), np.int32)
        ref_lib().ref_graph_adjacency(self.h, dir, _ptr(off, _i64p), _ptr(nb, _i32p))
        return off, nb[:tot]


class RefPPR:
    def __init__(self, n, sources, nparts, alpha, rmax):
        self.n = int(n)
        self.sources = np.ascontiguousarray(sources, dtype=np.int32)
        self.s = len(self.sources)
        self.h = ref_lib().ref_ppr_new(self.n, self.s, _ptr(self.sources, _i32p),
                                       nparts, alpha, rmax)

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_ppr_free(self.h)
            self.h = None

    def step(self, g, transpose, iter, dyn_start, threads=1):
        """Refresh + push of every source; threads > 1 splits the sources into
        contiguous ranges, one std::thread each, as the reference's drivers do."""
        if threads > 1:
            ref_lib().ref_ppr_step_mt(self.h, g.h, int(transpose), iter, dyn_start, int(threads))
        else:
            ref_lib().ref_ppr_step(self.h, g.h, int(transpose), iter, dyn_start)

    def log_only(self, iter, delta, resid, lp=False):
        """The reference's log transform + lazy test of every block, without
        copying anything out (for timing)."""
        r = np.ascontiguousarray(resid, np.float64)
        ref_lib().ref_log_blocks(self.h, int(lp), 1, int(iter), float(delta), _ptr(r, _f64p),
                                 None, None, None)

    def block_csr(self, b):
        """Block b's accepted log matrix (|S| x cols) as (indptr, indices, data)."""
        L = ref_lib()
        nnz = L.ref_block_csr(self.h, int(b), None, None, None)
        rp = np.zeros(self.s + 1, np.int32)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        L.ref_block_csr(self.h, int(b), _ptr(rp, _i32p), _ptr(ci, _i32p), _ptr(va, _f64p))
        return rp, ci[:nnz], va[:nnz]

    def state(self, which):
        out = np.zeros((self.s, self.n), np.float32)
        ref_lib().ref_ppr_state(self.h, which, _ptr(out, _f32p))
        return out

    def dense(self):
        out = np.zeros((self.s, self.n), np.float64)
        ref_lib().ref_ppr_dense(self.h, _ptr(out, _f64p))
        return out

    def log_blocks(self, lp, with_norm, iter, delta, resid):
        """The reference's log transform + lazy test of every block of the
        accumulated dense matrix (Code/ppr_computation_store_dynamic.h
        :2527-2826). Returns (accepted log blocks |S| x N, update record per
        block: -1 kept / iter refreshed, nnz record)."""
        nparts = len(resid)
        acc = np.zeros((self.s, self.n), np.float64)
        rec = np.zeros(nparts, np.int32)
        nnz = np.zeros(nparts, np.int64)
        r = np.ascontiguousarray(resid, np.float64)
        ref_lib().ref_log_blocks(self.h, int(lp), int(with_norm), int(iter), float(delta),
                                 _ptr(r, _f64p), _ptr(acc, _f64p), _ptr(rec, _i32p),
                                 _ptr(nnz, _i64p))
        return acc, rec, nnz


# ---------------------------------------------------- reference frPCA / merge
_REF_FRPCA_SO = os.path.join(HERE, "_ref", "libtsvd_ref_frpca.so")
_ref_frpca_lib = None


def ref_frpca_available():
    return os.path.exists(_REF_FRPCA_SO)


def ref_frpca_lib():
    """The reference's frpca.c and matrix_vector_functions_intel_mkl{,_ext}.c
    compiled against oracle/mkl_shim (oracle/build_ref.sh)."""
    global _ref_frpca_lib
    if _ref_frpca_lib is None:
        L = ctypes.CDLL(_REF_FRPCA_SO)
        L.tsvd_ref_set_seed.argtypes = [ctypes.c_uint64]
        L.tsvd_ref_last_gaussian.restype = ctypes.c_int
        L.tsvd_ref_last_gaussian.argtypes = [_f32p, ctypes.c_int]
        L.tsvd_ref_frpca.restype = ctypes.c_int
        L.tsvd_ref_frpca.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f64p,
                                     ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p]
        L.tsvd_ref_merge_svd.restype = ctypes.c_int
        L.tsvd_ref_merge_svd.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, _f64p,
                                         _f64p]
        _ref_frpca_lib = L
    return _ref_frpca_lib


def ref_frpca(A, k, q, seed=7):
    """frPCA(A, k, q) of the reference (Code/frpca.c:239-326) on a scipy CSR
    matrix. Returns U (m x k), S (k, in the reference's order), V (n x k) and
    the Gaussian test matrix it drew (n x (k+5) for even q, m x (k+5) for odd
    q), so the oracle can be run on the same one."""
    L = ref_frpca_lib()
    m, n = A.shape
    rp = np.ascontiguousarray(A.indptr, np.int32)
    ci = np.ascontiguousarray(A.indices, np.int32)
    va = np.ascontiguousarray(A.data, np.float64)
    U = np.zeros(m * k)
    S = np.zeros(k)
    V = np.zeros(n * k)
    L.tsvd_ref_set_seed(seed)
    L.tsvd_ref_frpca(m, n, _ptr(rp, _i32p), _ptr(ci, _i32p), _ptr(va, _f64p), k, q,
                     _ptr(U, _f64p), _ptr(S, _f64p), _ptr(V, _f64p))
    rows, l = (n if q % 2 == 0 else m), k + 5
    g = np.zeros(rows * l, np.float32)
    got = L.tsvd_ref_last_gaussian(_ptr(g, _f32p), rows * l)
    assert got == rows * l, (got, rows * l)
    omega = g.astype(np.float64).reshape(l, rows).T  # column-major, as the reference's mat
    return U.reshape(k, m).T, S, V.reshape(k, n).T, omega


def ref_merge_svd(M, d):
    """dense_sub_svd_function's factor U_d S_d of M (Code/Tree_u_NC.cpp:238-262
    via truncated_singular_value_decomposition, matrix_vector_functions_intel_mkl.c
    :1259-1300). Returns (U S (m x d), sigma (d,))."""
    L = ref_frpca_lib()
    m, n = M.shape
    Mc = np.asfortranarray(M, np.float64).ravel(order="F")
    US = np.zeros(m * d)
    sig = np.zeros(d)
    L.tsvd_ref_merge_svd(m, n, _ptr(Mc, _f64p), d, _ptr(US, _f64p), _ptr(sig, _f64p))
    return US.reshape(d, m).T, sig
