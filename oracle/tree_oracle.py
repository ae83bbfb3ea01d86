"""FP64 CPU oracle of the Tree-SVD per-snapshot refresh — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker. It restates the reference's algorithm literally:

  snapshot loop ........ Code/Tree_u_NC.cpp:507-866, Code/Tree_d_NC.cpp:566-1140
  graph / refresh / push  oracle/oracle_ppr.c (bit-exact with the reference code)
  log + lazy test ...... Code/ppr_computation_store_dynamic.h:2527-2561 (NC),
                         :2598-2638 (LP), :2649-2732 / :2742-2826 (with norms)
  frPCA ................ Code/frpca.c:239-326 with LUfraction (:4-41) and
                         eigSVD (:99-136), in float64 (numpy/scipy LAPACK)
  block factor/residual  Code/Tree_u_NC.cpp:139-204 (dense residual, as there)
  merge ................ Code/Tree_u_NC.cpp:723-850 (LAPACK gesvd via numpy)
  LP right factor ...... Code/Tree_u_LP.cpp:291-407 (V_b = A_b^T U per updated
                         block), U cache per block :1002-1038, scores and
                         precision :1046-1122, degree-scaled scores
                         Code/ppr_computation_store_dynamic.h:7704-7755

The reference seeds its Gaussian test matrix from time(NULL)
(Code/matrix_vector_functions_intel_mkl.c:495); the oracle and the GPU both
draw it from the shared counter-based generator instead, so the two consume
identical test matrices. The reference has no tests or golden vectors for
these steps; this module is pinned against the reference compiled from its
own sources (oracle/build_ref.sh): the push/refresh/insert half bit-exactly
(oracle/_ref/libtsvd_ref.so), the log transform and lazy test to the last bit
of log10 (same library, with a sparse-matrix stand-in for Eigen), frPCA and
the merge SVD to float64 rounding
(oracle/_ref/libtsvd_ref_frpca.so: frpca.c and the MKL helper files built
against the OpenBLAS-backed MKL stand-in in oracle/mkl_shim/, run on the same
Gaussian draw), with golden fixtures of both in tests/golden/.
"""
import ctypes

import numpy as np
import scipy.linalg

from . import native

TRANSFORM_LOG10_NC, TRANSFORM_LOG10_LP, TRANSFORM_LN_N = 0, 1, 2
DIRTY_REFERENCE, DIRTY_FROBENIUS, DIRTY_ALL = 0, 1, 2


def gaussian_matrix(seed, stream, nrows, ncols):
    L = native.lib()
    f = L.or_gaussian_matrix
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int64, ctypes.c_int32,
                  ctypes.POINTER(ctypes.c_double)]
    out = np.zeros((int(nrows), int(ncols)), np.float64)
    f(seed, stream, nrows, ncols, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def log_transform(x, rmin, transform, n):
    """Code/ppr_computation_store_dynamic.h:2549-2556 (NC), :2621-2632 (LP)."""
    out = np.zeros_like(x, dtype=np.float64)
    if transform == TRANSFORM_LOG10_NC:
        m = x > rmin
        out[m] = np.log10(x[m] / rmin)
    elif transform == TRANSFORM_LOG10_LP:
        m = x != 0
        out[m] = np.log10(1.0 + x[m] / rmin)
    else:
        m = x > 0
        out[m] = np.maximum(0.0, np.log(x[m] * n))
    return out


def lu_fraction(Q):
    """[L, ~] = lu(Q): the row-permuted unit lower factor (frpca.c:4-41)."""
    P, L, _ = scipy.linalg.lu(Q)
    return P @ L


def eig_svd(A):
    """frpca.c:99-136: G = A^T A, ascending eigenpairs, S = sqrt(max(lam, 0)),
    columns with S <= 1e-4 zeroed, U = A V / S."""
    G = A.T @ A
    w, V = np.linalg.eigh(G)
    S = np.sqrt(np.maximum(w, 0.0))
    V1 = V.copy()
    small = S <= 1e-4
    S[small] = 0.0
    V1[:, small] = 0.0
    V1[:, ~small] /= S[~small]
    return A @ V1, S, V


def frpca(A, k, q, omega=None, qrand=None, s=5):
    """frpca.c:239-326. Returns U (m x k), S (k, ascending), V (n x k), Q."""
    l = k + s
    if q % 2 == 0:
        Qt = omega
        Q = A @ Qt
        Q = eig_svd(Q)[0] if q == 2 else lu_fraction(Q)
    else:
        Q = qrand
    niter = (q - 1) // 2
    for i in range(1, niter + 1):
        Qt = A.T @ Q
        Q = A @ Qt
        Q = eig_svd(Q)[0] if i == niter else lu_fraction(Q)
    Qt = A.T @ Q
    UU, SS, VV = eig_svd(Qt)
    V = UU[:, s:l]
    S = SS[s:l]
    U = Q @ VV[:, s:l]
    return U, S, V


class OracleTreeSVD:
    """Snapshot-by-snapshot CPU restatement of the reference pipeline (float64)."""

    def __init__(self, n, sources, directed=False, alpha=0.5, rmax=1e-7, n_parts=64,
                 hierarchy_n=2, rank_d=128, oversample=5, passes_q=12,
                 dynamic_ppr_start_iter=100, lazy_update_start_iter=100, delta=0.3,
                 transform=TRANSFORM_LOG10_NC, dirty_rule=DIRTY_REFERENCE, dirty_frac=0.01,
                 root_scaling=0, refresh_mode=0, seed=20231, threads=1, lp_right_factor=False,
                 block_path=0, push_levels=1, push_ratio=8.0, push_hub_degree=0):
        # block_path (the GPU's product path for a block's frPCA) and the push's
        # threshold schedule (the order in which the GPU pushes; its last level is
        # the rmax test the FIFO applies) do not change what the oracle computes:
        # accepted and unused
        self.n, self.directed = int(n), bool(directed)
        self.sources = np.ascontiguousarray(sources, dtype=np.int32)
        self.S = len(self.sources)
        self.alpha, self.rmax = float(alpha), float(rmax)
        self.P, self.h, self.d, self.s, self.q = n_parts, hierarchy_n, rank_d, oversample, passes_q
        self.dyn, self.lazy, self.delta = dynamic_ppr_start_iter, lazy_update_start_iter, delta
        self.transform, self.rule, self.frac = transform, dirty_rule, dirty_frac
        self.root_scaling, self.intdiv, self.seed = root_scaling, refresh_mode == 1, seed
        self.threads = threads
        self.g = native.OracleGraph(n, directed)
        self.ppr = [native.OraclePPR(n, self.sources)]
        if directed:
            self.ppr.append(native.OraclePPR(n, self.sources))
        self.col_dim = n // n_parts
        self.accepted = [None] * n_parts   # mat_mapping: accepted log blocks
        self.resid = np.zeros(n_parts)
        self.norm = np.zeros(n_parts)
        self.norm_diff = np.zeros(n_parts)
        self.nnz = np.zeros(n_parts, np.int64)
        self.dirty = np.zeros(n_parts, np.uint8)
        levels, t = 1, n_parts
        while t > 1:
            t //= hierarchy_n
            levels += 1
        self.total = sum(hierarchy_n ** i for i in range(levels))
        self.leaf_start = self.total - n_parts
        self.factor = [np.zeros((self.S, rank_d)) for _ in range(self.total)]
        self.sigma = [np.zeros(rank_d) for _ in range(self.total)]
        self.embedding = None
        self.iter = 0
        self.push_counts = (0, 0)
        self.last_factorized = []
        self.lp = bool(lp_right_factor)
        self.lp_V = np.zeros((n, rank_d))       # V_matrix (zero where never computed)
        self.lp_U = [None] * n_parts            # left_matrix_U_cache per block

    def block_cols(self, b):
        c0 = b * self.col_dim
        c1 = self.n if b == self.P - 1 else c0 + self.col_dim
        return c0, c1

    def reserve(self):
        p = self.ppr[0].reserve().astype(np.float64)
        if self.directed:
            p += self.ppr[1].reserve().astype(np.float64)
        return p

    def ppr_stage(self, iter):
        pushes = upd = 0
        for dirn, st in enumerate(self.ppr):
            st.refresh(self.g, dirn, iter, self.dyn, self.alpha, self.rmax, self.intdiv, self.threads)
            a, b = st.push(self.g, dirn, self.alpha, self.rmax, self.threads)
            pushes += a
            upd += b
        self.push_counts = (pushes, upd)

    def blocks_stage(self, iter, p=None):
        p = self.reserve() if p is None else np.asarray(p, dtype=np.float64)
        with_norm = iter >= self.lazy
        todo = []
        for b in range(self.P):
            c0, c1 = self.block_cols(b)
            x = p[:, c0:c1]
            A = log_transform(x, self.rmax, self.transform, self.n)
            stored = int(np.count_nonzero(x))
            self.nnz[b] = int(np.count_nonzero(A))
            self.norm[b] = np.linalg.norm(A)
            old = self.accepted[b]
            self.norm_diff[b] = np.linalg.norm(A - old) if old is not None else self.norm[b]
            dirty = True
            if with_norm:
                if self.rule == DIRTY_REFERENCE:
                    dirty = not (self.resid[b] + self.norm_diff[b] <
                                 self.delta * np.sqrt(2.0) * self.norm[b])
                elif self.rule == DIRTY_FROBENIUS:
                    dirty = self.norm_diff[b] > self.frac * self.norm[b]
            self.dirty[b] = dirty
            if dirty:
                self.accepted[b] = A
                if stored > 0:
                    todo.append(b)
        return todo

    def factor_block(self, b, iter):
        A = self.accepted[b]
        c0, c1 = self.block_cols(b)
        l = self.d + self.s
        omega = gaussian_matrix(self.seed, b, c1 - c0, l) if self.q % 2 == 0 else None
        qrand = gaussian_matrix(self.seed, 0x80000000 | b, self.S, l) if self.q % 2 else None
        U, S, V = frpca(A, self.d, self.q, omega, qrand, self.s)
        B = U * S[None, :]
        self.factor[self.leaf_start + b] = B
        self.sigma[self.leaf_start + b] = S[::-1].copy()
        if iter >= self.lazy - 1:
            self.resid[b] = np.linalg.norm(B @ V.T - A)
        return U, S, V

    def merge_stage(self, done):
        h = self.h
        level = sorted({(self.leaf_start + b - 1) // h for b in done})
        while level:
            if level == [0]:
                M = np.hstack([self.factor[1 + c] for c in range(h)])
                U, S, _ = np.linalg.svd(M, full_matrices=False)
                U, S = U[:, :self.d], S[:self.d]
                self.sigma[0] = S
                self.embedding = U * np.sqrt(np.abs(S))[None, :] if self.root_scaling == 0 else U
                self.factor[0] = self.embedding
                return
            for p in level:
                M = np.hstack([self.factor[p * h + 1 + c] for c in range(h)])
                U, S, _ = np.linalg.svd(M, full_matrices=False)
                self.factor[p] = U[:, :self.d] * S[None, :self.d]
                self.sigma[p] = S[:self.d]
            level = sorted({(p - 1) // h for p in level})

    def step(self, edges, reserve=None):
        """One snapshot. With `reserve` (|S| x N, forward + reverse summed) the
        PPR stage is skipped and the block stages run on the given reserve."""
        self.iter += 1
        it = self.iter
        self.g.insert(edges)
        if self.lazy != 100 and it < self.lazy - 1:
            return None
        if reserve is None:
            self.ppr_stage(it)
        todo = self.blocks_stage(it, reserve)
        for b in todo:
            self.factor_block(b, it)
        self.last_factorized = todo
        if todo:
            self.merge_stage(todo)
        if self.lp and todo and self.embedding is not None:
            self.lp_stage()
        return self.embedding

    def lp_stage(self):
        """Right factor of every block updated in this snapshot with this
        snapshot's root U (Tree_u_LP.cpp:1040-1044 -> :291-407)."""
        for b in range(self.P):
            if not self.dirty[b]:
                continue
            c0, c1 = self.block_cols(b)
            self.lp_V[c0:c1] = self.accepted[b].T @ self.embedding
            self.lp_U[b] = self.embedding.copy()


def lp_scores(lp_U, lp_V, sources, col_dim, n_parts, pairs, degree_scaled=False,
              deg_i=None, deg_j=None):
    """score(i, j) = U_b[row(i)] . V[j] with U_b the root factor block b(j)'s
    V rows were computed with (Tree_u_LP.cpp:1051-1070); times
    outdeg(i) * indeg(j) when degree_scaled (ppr:7725, 7749)."""
    row = {int(v): k for k, v in enumerate(sources)}
    out = np.zeros(len(pairs))
    for k, (i, j) in enumerate(np.asarray(pairs).reshape(-1, 2)):
        b = min(int(j) // col_dim, n_parts - 1)
        U = lp_U[b]
        sc = 0.0 if U is None else float(np.dot(U[row[int(i)]], lp_V[int(j)]))
        if degree_scaled:
            sc *= float(deg_i[i]) * float(deg_j[j])
        out[k] = sc
    return out


def lp_precision(scores, positive, k):
    """Positives among the k highest scores over k (Tree_u_LP.cpp:1104-1122);
    ties go to the lower index."""
    scores = np.asarray(scores, dtype=np.float64)
    order = np.lexsort((np.arange(len(scores)), -scores))
    return float(np.count_nonzero(np.asarray(positive)[order[:k]])) / k
