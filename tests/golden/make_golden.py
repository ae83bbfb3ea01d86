"""Generates tests/golden/ref_ppr_*.npz, ref_frpca_*.npz and ref_merge.npz
from the reference's own code.

Runs the reference's graph store (Code/Graph_dynamic.h, fed through its own
file reader) and its dense-path refresh + push functions
(Code/ppr_computation_store_dynamic.h, compiled from the reference sources by
oracle/build_ref.sh into oracle/_ref/libtsvd_ref.so) on small seeded graphs,
and stores the inputs and the reference's outputs (adjacency, degrees,
residue, reserve, accumulated dense matrix) after every snapshot.

The frPCA and merge fixtures come from the reference's frpca.c and
matrix_vector_functions_intel_mkl{,_ext}.c compiled against the MKL stand-in
(oracle/_ref/libtsvd_ref_frpca.so): a seeded sparse matrix, the Gaussian test
matrix the reference drew, and its U, S, V; a seeded two-child merge matrix
and dense_sub_svd_function's U S and singular values. ref_log.npz: the
reference's log transform + lazy test (Log_sparse_matrix_entries*, both
transforms) on its own accumulated matrix over a few snapshots.

    sh oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import scipy.sparse as sp
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import native  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (directed, n, S, snapshot sizes, alpha, rmax, dynamic_start, nparts, seed)
    "undirected": (0, 240, 8, [600, 80, 80], 0.2, 1e-4, 2, 4, 101),
    "directed": (1, 240, 8, [700, 90, 90], 0.2, 1e-4, 2, 4, 202),
    "undirected_scratch": (0, 180, 6, [400, 60], 0.5, 1e-3, 100, 3, 303),
}


def make(name, directed, n, S, sizes, alpha, rmax, dyn, nparts, seed):
    rng = np.random.default_rng(seed)
    snaps = []
    for k in sizes:
        e = rng.integers(0, n, size=(k, 2)).astype(np.int32)
        e = e[e[:, 0] != e[:, 1]]
        snaps.append(e)
    deg0 = np.bincount(snaps[0].ravel(), minlength=n)
    sources = np.sort(rng.choice(np.nonzero(deg0)[0], S, replace=False)).astype(np.int32)
    g = native.RefGraph(n, directed)
    fwd = native.RefPPR(n, sources, nparts, alpha, rmax)
    tr = native.RefPPR(n, sources, nparts, alpha, rmax) if directed else None
    out = dict(directed=directed, n=n, sources=sources, alpha=alpha, rmax=rmax,
               dynamic_start=dyn, nparts=nparts, nsnap=len(snaps))
    with tempfile.TemporaryDirectory() as d:
        for it, e in enumerate(snaps, start=1):
            path = os.path.join(d, "s%d.txt" % it)
            native.write_edge_file(path, e, trailing_newline=True)
            g.insert_file(path)
            out["edges_%d" % it] = e
            for dirn in range(2 if directed else 1):
                off, nb = g.adjacency(dirn)
                deg, former = g.degrees(dirn)
                out["off_%d_%d" % (it, dirn)] = off
                out["nbr_%d_%d" % (it, dirn)] = nb
                out["former_%d_%d" % (it, dirn)] = former
                st = fwd if dirn == 0 else tr
                st.step(g, dirn, it, dyn)
                out["r_%d_%d" % (it, dirn)] = st.state(0)
                out["p_%d_%d" % (it, dirn)] = st.state(1)
            out["dense_%d" % it] = fwd.dense() + (tr.dense() if tr is not None else 0.0)
    np.savez_compressed(os.path.join(HERE, "ref_ppr_%s.npz" % name), **out)


FRPCA_CASES = {
    # name: (m, n, rank, support fraction, k, q, seed)
    "q6": (120, 500, 20, 0.12, 16, 6, 404),
    "q3": (96, 400, 16, 0.15, 12, 3, 505),
}


def make_frpca(name, m, n, rank, frac, k, q, seed):
    """A sum of `rank` sparse non-negative rank-one terms with weights 0.8^i
    (rank <= k + 5, so frPCA recovers it up to rounding whatever the
    Gaussian draw)."""
    rng = np.random.default_rng(seed)
    D = np.zeros((m, n))
    for i in range(rank):
        u = np.where(rng.random(m) < frac, rng.random(m) + 0.5, 0.0)
        v = np.where(rng.random(n) < frac, rng.random(n) + 0.5, 0.0)
        D += 5.0 * 0.8 ** i * np.outer(u, v)
    A = sp.csr_matrix(D)
    U, S, V, omega = native.ref_frpca(A, k, q, seed=seed)
    np.savez_compressed(os.path.join(HERE, "ref_frpca_%s.npz" % name), indptr=A.indptr,
                        indices=A.indices, data=A.data, shape=np.array(A.shape), k=k, q=q,
                        omega=omega.astype(np.float32), U=U, S=S, V=V)


def make_log(seed=707, n=200, S=6, P=4, alpha=0.2, rmax=1e-4, delta=0.3, snaps=4):
    """The reference's log transform + lazy test (both transforms) on the
    dense matrix its own push accumulated, snapshot by snapshot, with
    residuals drawn on the scale of the block norms."""
    rng = np.random.default_rng(seed)
    out = dict(n=n, S=S, P=P, alpha=alpha, rmax=rmax, delta=delta, nsnap=snaps)
    for lp in (0, 1):
        g = native.RefGraph(n, 0)
        src = np.sort(rng.choice(n, S, replace=False)).astype(np.int32)
        st = native.RefPPR(n, src, P, alpha, rmax)
        out["sources_%d" % lp] = src
        cd = n // P
        prev = np.ones(P)
        with tempfile.TemporaryDirectory() as d:
            for it in range(1, snaps + 1):
                e = rng.integers(0, n, (1200 if it == 1 else 50, 2)).astype(np.int32)
                e = e[e[:, 0] != e[:, 1]]
                path = os.path.join(d, "s%d.txt" % it)
                native.write_edge_file(path, e, trailing_newline=True)
                g.insert_file(path)
                st.step(g, 0, it, 2)
                dense = st.dense()
                # residuals on the scale of the accepted blocks: both decisions occur
                resid = rng.uniform(0.2, 0.6, P) * prev
                acc, rec, nnz = st.log_blocks(lp, it >= 2, it, delta, resid)
                prev = np.array([np.linalg.norm(acc[:, b * cd:(n if b == P - 1 else (b + 1) * cd)])
                                 for b in range(P)])
                for k, v in dict(dense=dense, resid=resid, accepted=acc, record=rec,
                                 nnz=nnz).items():
                    out["%s_%d_%d" % (k, lp, it)] = v
    np.savez_compressed(os.path.join(HERE, "ref_log.npz"), **out)


def make_merge(seed=606, rows=150, d=32, h=2):
    rng = np.random.default_rng(seed)
    kids = []
    for c in range(h):
        Q = np.linalg.qr(rng.standard_normal((rows, d)))[0]
        kids.append(Q * np.geomspace(50.0 / (c + 1), 0.5, d)[None, :])
    M = np.hstack(kids)
    US, sigma = native.ref_merge_svd(M, d)
    np.savez_compressed(os.path.join(HERE, "ref_merge.npz"), M=M, d=d, US=US, sigma=sigma)


if __name__ == "__main__":
    if not native.ref_available() or not native.ref_frpca_available():
        native.build_ref()
    for name, args in CASES.items():
        make(name, *args)
        print("wrote", name)
    for name, args in FRPCA_CASES.items():
        make_frpca(name, *args)
        print("wrote frpca", name)
    make_merge()
    print("wrote merge")
    make_log()
    print("wrote log")
