"""Pins the CPU oracle to the reference.

1. Golden fixtures (tests/golden/ref_ppr_*.npz, produced by the reference's
   own graph store / refresh / push compiled from its sources, see
   tests/golden/make_golden.py) must be reproduced bit for bit.
2. Where oracle/_ref/libtsvd_ref.so exists (built here from the reference
   sources), random cases are compared live as well.
"""
import glob
import os
import tempfile

import numpy as np
import pytest

import tsvd_gb300 as T
from oracle import native

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_ppr_*.npz")))


def _read_like_reference(edges):
    """The reference reads each delta with a trailing newline: last pair twice."""
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "e.txt")
        native.write_edge_file(p, edges, trailing_newline=True)
        return T.read_edge_file(p, compat_dup_last=True)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_reproduces_reference_golden(path):
    z = np.load(path)
    directed, n = int(z["directed"]), int(z["n"])
    src = z["sources"]
    alpha, rmax, dyn = float(z["alpha"]), float(z["rmax"]), int(z["dynamic_start"])
    g = native.OracleGraph(n, directed)
    st = [native.OraclePPR(n, src) for _ in range(2 if directed else 1)]
    for it in range(1, int(z["nsnap"]) + 1):
        g.insert(_read_like_reference(z["edges_%d" % it]))
        for d in range(len(st)):
            off, nb = g.adjacency(d)
            assert np.array_equal(off, z["off_%d_%d" % (it, d)])
            assert np.array_equal(nb, z["nbr_%d_%d" % (it, d)])
            assert np.array_equal(g.degrees(d)[1], z["former_%d_%d" % (it, d)])
            # the reference's dense path divides (j+1)/j in integers (ppr:2102)
            st[d].refresh(g, d, it, dyn, alpha, rmax, intdiv=True)
            st[d].push(g, d, alpha, rmax)
            assert np.array_equal(st[d].residue(), z["r_%d_%d" % (it, d)])
            assert np.array_equal(st[d].reserve(), z["p_%d_%d" % (it, d)])


def test_reference_dense_matrix_is_the_reserve_when_pushing_from_scratch():
    """With every snapshot pushed from scratch, the reference's accumulated
    dense matrix after the first snapshot is the reserve (up to float vs double
    accumulation) except on isolated sources; this build derives the block
    matrix from the reserve."""
    z = np.load([p for p in GOLDEN if "scratch" in p][0])
    p = z["p_1_0"].astype(np.float64)
    dense = z["dense_1"]
    assert np.allclose(p, dense, rtol=1e-5, atol=1e-7)


@pytest.mark.skipif(not native.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("directed,intdiv", [(0, True), (1, True)])
def test_oracle_matches_reference_live(directed, intdiv):
    rng = np.random.default_rng(7 + directed)
    n, S = 400, 12
    g, rg = native.OracleGraph(n, directed), native.RefGraph(n, directed)
    src = np.sort(rng.choice(n, S, replace=False)).astype(np.int32)
    ors = [native.OraclePPR(n, src) for _ in range(2)]
    rps = [native.RefPPR(n, src, 4, 0.15, 5e-5) for _ in range(2)]
    for it in range(1, 5):
        e = rng.integers(0, n, (900 if it == 1 else 120, 2)).astype(np.int32)
        rg.insert(e, trailing_newline=True)
        g.insert(np.concatenate([e, e[-1:]]))
        for d in range(2 if directed else 1):
            assert np.array_equal(g.adjacency(d)[1], rg.adjacency(d)[1])
            ors[d].refresh(g, d, it, 2, 0.15, 5e-5, intdiv=intdiv, threads=3)
            ors[d].push(g, d, 0.15, 5e-5, threads=3)
            rps[d].step(rg, d, it, 2)
            assert np.array_equal(ors[d].residue(), rps[d].state(0))
            assert np.array_equal(ors[d].reserve(), rps[d].state(1))


def test_oracle_push_identity_and_threshold():
    """Exact-division refresh keeps p (I - (1-a) P) = a (e_s - r) after every snapshot."""
    from helpers import push_identity_residual, transition
    rng = np.random.default_rng(3)
    n, S, alpha, rmax = 500, 10, 0.2, 1e-5
    g = native.OracleGraph(n, False)
    src = np.sort(rng.choice(n, S, replace=False)).astype(np.int32)
    o = native.OraclePPR(n, src)
    first = rng.integers(0, n, (2500, 2)).astype(np.int32)
    first = first[first[:, 0] != first[:, 1]]
    # make every source non-isolated
    first = np.concatenate([first, np.stack([src, (src + 1) % n], 1)]).astype(np.int32)
    for it, e in enumerate([first] + [rng.integers(0, n, (200, 2)).astype(np.int32) for _ in range(3)], 1):
        e = e[e[:, 0] != e[:, 1]]
        g.insert(e)
        o.refresh(g, 0, it, 2, alpha, rmax)
        o.push(g, 0, alpha, rmax)
        off, nb = g.adjacency(0)
        P, deg = transition(n, off, nb)
        r, p = o.residue(), o.reserve()
        assert push_identity_residual(p, r, src, P, alpha) < 1e-5
        assert (r[:, deg > 0] <= rmax).all()


# ------------------------------------------------- frPCA and merge (MKL path)
FRPCA_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden",
                                             "ref_frpca_*.npz")))
MERGE_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_merge.npz")


def _csr(z):
    import scipy.sparse as sp
    return sp.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))


def _check_frpca_against(A, k, q, omega, U, S, V, tol):
    """Oracle frPCA on the reference's own Gaussian draw vs the reference's
    U, S, V: same values, columns equal up to sign."""
    from oracle.tree_oracle import frpca
    if q % 2 == 0:
        Uo, So, Vo = frpca(A.toarray(), k, q, omega=omega)
    else:
        Uo, So, Vo = frpca(A.toarray(), k, q, qrand=omega)
    assert np.allclose(So, S, rtol=tol, atol=tol * np.abs(S).max())
    for X, Xo in ((U, Uo), (V, Vo)):
        cos = np.abs(np.sum(X * Xo, 0)) / (np.linalg.norm(X, axis=0) * np.linalg.norm(Xo, axis=0))
        assert np.abs(cos - 1).max() < tol, np.abs(cos - 1).max()


@pytest.mark.parametrize("path", FRPCA_GOLDEN, ids=[os.path.basename(p) for p in FRPCA_GOLDEN])
def test_oracle_frpca_reproduces_reference_golden(path):
    """tests/golden/ref_frpca_*.npz: the reference's frpca.c (compiled against
    the MKL stand-in) on a seeded sparse matrix, with the Gaussian matrix it
    drew. The oracle restates frpca.c:239-326 (LUfraction :4-41, eigSVD
    :99-136) and must reproduce U, S, V to float64 rounding."""
    z = np.load(path)
    _check_frpca_against(_csr(z), int(z["k"]), int(z["q"]), z["omega"].astype(np.float64),
                         z["U"], z["S"], z["V"], 1e-9)


def test_oracle_merge_reproduces_reference_golden():
    """tests/golden/ref_merge.npz: dense_sub_svd_function's U_d S_d and
    singular values (LAPACK gesvd through the reference's own
    truncated_singular_value_decomposition) of a two-child merge matrix,
    against the oracle's merge step (numpy SVD)."""
    z = np.load(MERGE_GOLDEN)
    M, d = z["M"], int(z["d"])
    U, S, _ = np.linalg.svd(M, full_matrices=False)
    US = U[:, :d] * S[None, :d]
    assert np.allclose(S[:d], z["sigma"], rtol=1e-12)
    cos = np.abs(np.sum(US * z["US"], 0)) / (np.linalg.norm(US, axis=0) * np.linalg.norm(z["US"], axis=0))
    assert np.abs(cos - 1).max() < 1e-10


@pytest.mark.skipif(not native.ref_frpca_available(), reason="reference frpca.c not compiled here")
@pytest.mark.parametrize("q", [2, 5, 6])
def test_oracle_frpca_matches_reference_live(q):
    import scipy.sparse as sp
    rng = np.random.default_rng(40 + q)
    m, n, k = 90, 420, 10
    base = (rng.standard_normal((m, 16)) * np.geomspace(3.0, 0.1, 16)) @ rng.standard_normal((16, n))
    A = sp.csr_matrix(np.where(rng.random((m, n)) < 0.15, np.abs(base) + 0.5, 0.0))
    U, S, V, omega = native.ref_frpca(A, k, q, seed=q)
    _check_frpca_against(A, k, q, omega, U, S, V, 1e-9)


@pytest.mark.skipif(not native.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("transform", [0, 1])
def test_oracle_log_and_lazy_test_match_reference_live(transform):
    """The reference's own Log_sparse_matrix_entries[_LP] and
    ..._with_norm_computation[_LP] (compiled from its header by line range,
    with a minimal sparse-matrix stand-in for Eigen) on the dense matrix its
    own push accumulated, against the oracle's log transform and reference
    lazy rule on the same matrix and residuals: the same accepted blocks (up
    to the last bit of log10, where numpy's and the C library's differ by one
    ulp on a few percent of inputs), identical keep / refresh decisions (cases
    within 1e-9 of the threshold excluded), identical nnz counts."""
    from oracle.tree_oracle import OracleTreeSVD, TRANSFORM_LOG10_LP, TRANSFORM_LOG10_NC
    rng = np.random.default_rng(11 + transform)
    n, S, P, alpha, rmax, delta = 360, 10, 4, 0.2, 1e-4, 0.3
    rg = native.RefGraph(n, 0)
    src = np.sort(rng.choice(n, S, replace=False)).astype(np.int32)
    rp = native.RefPPR(n, src, P, alpha, rmax)
    tf = TRANSFORM_LOG10_LP if transform else TRANSFORM_LOG10_NC
    o = OracleTreeSVD(n, src, alpha=alpha, rmax=rmax, n_parts=P, lazy_update_start_iter=2,
                      delta=delta, transform=tf)
    kept = refreshed = 0
    for it in range(1, 6):
        e = rng.integers(0, n, (1500 if it == 1 else 60, 2)).astype(np.int32)
        e = e[e[:, 0] != e[:, 1]]
        rg.insert(e, trailing_newline=True)
        rp.step(rg, 0, it, 2)
        dense = rp.dense()
        # residuals on the scale of the block norms, so both decisions occur
        norms = np.array([np.linalg.norm(o.accepted[b]) if o.accepted[b] is not None else 1.0
                          for b in range(P)])
        resid = rng.uniform(0.0, 0.5, P) * norms
        with_norm = it >= 2
        acc, rec, nnz = rp.log_blocks(transform, with_norm, it, delta, resid)
        o.resid[:] = resid
        o.blocks_stage(it, p=dense)
        for b in range(P):
            c0, c1 = o.block_cols(b)
            margin = o.resid[b] + o.norm_diff[b] - delta * np.sqrt(2.0) * o.norm[b]
            if with_norm and abs(margin) <= 1e-9 * o.norm[b]:
                continue
            assert (rec[b] != -1) == bool(o.dirty[b]), (it, b, rec[b], o.dirty[b])
            kept += rec[b] == -1
            refreshed += rec[b] != -1
            assert np.allclose(acc[:, c0:c1], o.accepted[b], rtol=1e-15, atol=0), (it, b)
            assert np.array_equal(acc[:, c0:c1] != 0, o.accepted[b] != 0)
            if rec[b] != -1:
                assert nnz[b] == (np.count_nonzero(o.accepted[b]) if transform else
                                  np.count_nonzero(dense[:, c0:c1] > rmax))
    assert kept > 0 and refreshed > 0


def test_oracle_log_and_lazy_test_reproduce_reference_golden():
    """tests/golden/ref_log.npz: the reference's log transform + lazy test on
    its own accumulated matrix (both transforms, four snapshots), replayed
    through the oracle's block stage with the same matrix and residuals."""
    from oracle.tree_oracle import OracleTreeSVD, TRANSFORM_LOG10_LP, TRANSFORM_LOG10_NC
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_log.npz"))
    n, P, rmax, delta = int(z["n"]), int(z["P"]), float(z["rmax"]), float(z["delta"])
    for lp in (0, 1):
        o = OracleTreeSVD(n, z["sources_%d" % lp], alpha=float(z["alpha"]), rmax=rmax, n_parts=P,
                          lazy_update_start_iter=2, delta=delta,
                          transform=TRANSFORM_LOG10_LP if lp else TRANSFORM_LOG10_NC)
        for it in range(1, int(z["nsnap"]) + 1):
            o.resid[:] = z["resid_%d_%d" % (lp, it)]
            o.blocks_stage(it, p=z["dense_%d_%d" % (lp, it)])
            acc, rec = z["accepted_%d_%d" % (lp, it)], z["record_%d_%d" % (lp, it)]
            for b in range(P):
                c0, c1 = o.block_cols(b)
                margin = o.resid[b] + o.norm_diff[b] - delta * np.sqrt(2.0) * o.norm[b]
                if it >= 2 and abs(margin) <= 1e-9 * o.norm[b]:
                    continue
                assert (rec[b] != -1) == bool(o.dirty[b]), (lp, it, b)
                assert np.allclose(acc[:, c0:c1], o.accepted[b], rtol=1e-15, atol=0)
