"""The plain GPU form (TSVD_FORM_PLAIN) against the oracle, and the FP32 frPCA
entry point. The plain form pushes one (vertex, source) cell per frontier
entry with fp64 push arithmetic, factorizes every dirty block on its own with
FP32 CSR SpMM products and merges one tree node at a time; it is the baseline
the mixed form is measured against, so it gets the same parity checks:

* its PPR state satisfies the push identity, leaves no eligible residue above
  rmax, and lies within the residual bounds of the oracle's FIFO push;
* its block stages agree with the oracle run on its own reserve (singular
  values within 1e-3, embedding Gram within 5e-3);
* a session may switch forms between snapshots (mixed -> plain -> mixed)
  and stays consistent.
"""
import numpy as np
import pytest

import tsvd_gb300 as T
import workloads as W
from helpers import (gap_index, gram_rel_err, max_principal_sine, push_identity_residual,
                     residual_error_bound, transition)
from oracle import native
from oracle.tree_oracle import OracleTreeSVD, frpca as oracle_frpca, gaussian_matrix

pytestmark = pytest.mark.gpu


def small_cfg(directed=False, n=6000, m=40000, sources=64, n_parts=4, rank_d=32, snapshots=4):
    base = "rmat-d-2.7m" if directed else "rmat-u-100k"
    c = W.scaled(base, n=n, m=m, sources=sources, n_parts=n_parts, rank_d=rank_d,
                 snapshots=snapshots)
    c["rmax"] = 1e-5
    return c


def _ppr_against_oracle(s, g, src, cfg, oracle_states):
    for t, o in enumerate(oracle_states):
        off, nb = g.adjacency(t)
        P, deg = transition(cfg["n"], off, nb)
        p = s.ppr_state(bool(t), 1)
        r = s.ppr_state(bool(t), 0)
        assert push_identity_residual(p, r, src, P, cfg["alpha"]) < 2e-5
        assert (r[:, deg > 0] <= np.float32(cfg["rmax"])).all()
        assert (p >= 0).all()
        po, ro = o.reserve().astype(np.float64), o.residue()
        bound = (residual_error_bound(r, P, cfg["alpha"]) +
                 residual_error_bound(ro, P, cfg["alpha"]))
        assert (np.abs(p.astype(np.float64) - po) <= bound * (1 + 1e-3) + 1e-6).all()


@pytest.mark.parametrize("directed,cap", [(False, 0), (True, 0), (True, 700)])
def test_plain_form_snapshots_match_the_oracle(directed, cap):
    """cap = 700: the frontier list holds far fewer cells than a round
    touches, so most cells wait in the bitset for later rounds (the path a
    large graph takes with the default 2^26 entries)."""
    cfg = small_cfg(directed, n=7003, m=50000, sources=96)
    _, snaps, src = W.build(cfg, seed=41)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    okw = dict(kw)
    okw.pop("seed")
    iso = OracleTreeSVD(cfg["n"], src, seed=kw["seed"], **okw)
    g = native.OracleGraph(cfg["n"], directed)
    ors = [native.OraclePPR(cfg["n"], src) for _ in range(2 if directed else 1)]
    with T.Session(cfg["n"], src, form=T.FORM_PLAIN, plain_frontier_cap=cap, **kw) as s:
        for it, e in enumerate(snaps, start=1):
            st = s.step(e)
            g.insert(e)
            for t, o in enumerate(ors):
                o.refresh(g, t, it, 2, cfg["alpha"], cfg["rmax"])
                o.push(g, t, cfg["alpha"], cfg["rmax"])
            _ppr_against_oracle(s, g, src, cfg, ors)
            assert st["pushes"] > 0 and st["pushes"] == st["push_items"]
            p = s.ppr_state(False, 1).astype(np.float64)
            if directed:
                p += s.ppr_state(True, 1)
            emb_o = iso.step(e, reserve=p)
            info = s.block_info()
            assert np.allclose(info["norm"], iso.norm, rtol=1e-5)
            frac = kw["dirty_frac"]
            if kw["dirty_rule"] == T.DIRTY_FROBENIUS:
                tie = np.abs(iso.norm_diff - frac * iso.norm) <= 1e-3 * iso.norm
            else:
                tie = np.abs(iso.resid + iso.norm_diff - kw["delta"] * np.sqrt(2) * iso.norm) \
                    <= 1e-3 * iso.norm
            assert np.array_equal(info["dirty"][~tie], iso.dirty[~tie])
            if tie.any() and not np.array_equal(info["dirty"][tie], iso.dirty[tie]):
                break
            for b in iso.last_factorized:
                _, sg = s.tree_factor(s.leaf_start + b)
                so = iso.sigma[s.leaf_start + b]
                j = gap_index(so, cfg["rank_d"])
                assert np.allclose(sg[:j], so[:j], rtol=1e-3), (b, np.abs(sg[:j] / so[:j] - 1).max())
            emb = s.embedding()
            _, sig = s.tree_factor(0)
            assert np.allclose(sig[:16], iso.sigma[0][:16], rtol=1e-3)
            assert gram_rel_err(emb, emb_o) < 5e-3


def test_forms_can_alternate_within_a_session():
    """mixed, plain, mixed, plain: every snapshot leaves a valid push state
    and block stages that agree with the oracle on the session's reserve."""
    cfg = small_cfg(True, n=6000, m=45000, sources=80, snapshots=5)
    _, snaps, src = W.build(cfg, seed=43)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    okw = dict(kw)
    okw.pop("seed")
    iso = OracleTreeSVD(cfg["n"], src, seed=kw["seed"], **okw)
    g = native.OracleGraph(cfg["n"], True)
    ors = [native.OraclePPR(cfg["n"], src) for _ in range(2)]
    with T.Session(cfg["n"], src, **kw) as s:
        for it, e in enumerate(snaps, start=1):
            s.set_form(T.FORM_PLAIN if it % 2 == 0 else T.FORM_MIXED)
            s.step(e)
            g.insert(e)
            for t, o in enumerate(ors):
                o.refresh(g, t, it, 2, cfg["alpha"], cfg["rmax"])
                o.push(g, t, cfg["alpha"], cfg["rmax"])
            _ppr_against_oracle(s, g, src, cfg, ors)
            p = s.ppr_state(False, 1).astype(np.float64) + s.ppr_state(True, 1)
            emb_o = iso.step(e, reserve=p)
            if not np.array_equal(s.block_info()["dirty"], iso.dirty):
                break  # a near-tie decision parted the histories
            _, sig = s.tree_factor(0)
            assert np.allclose(sig[:16], iso.sigma[0][:16], rtol=1e-3)
            assert gram_rel_err(s.embedding(), emb_o) < 5e-3
        # the pipelined driver loop refuses the plain form
        s.set_form(T.FORM_PLAIN)
        with pytest.raises(T.TsvdError):
            s.run([snaps[-1][:10]])


def test_frpca_fp32_against_the_oracle():
    """FP32 SpMM products: the matrix is not rounded to half precision, so
    the leading singular values agree with the float64 oracle on the same
    Gaussian matrix far inside the 1e-3 tolerance of the tensor-core path."""
    rng = np.random.default_rng(6)
    m, n, k, q = 600, 5000, 48, 6
    D = (rng.standard_normal((m, 120)) * 0.95 ** np.arange(120)) @ rng.standard_normal((120, n))
    D = np.where(rng.random((m, n)) < 0.2, np.abs(D), 0.0)
    D[:, rng.choice(n, n // 7, replace=False)] = 0.0
    import scipy.sparse as sp
    A = sp.csr_matrix(D)
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=17, fp32=True)
    omega = gaussian_matrix(17, 0, n, k + 5)
    Uo, So, Vo = oracle_frpca(A.toarray(), k, q, omega=omega)
    So, Uo, Vo = So[::-1], Uo[:, ::-1], Vo[:, ::-1]
    j = gap_index(So, k)
    assert j > 0
    rel = np.abs(S[:j] / So[:j] - 1).max()
    assert rel < 1e-4, rel
    assert max_principal_sine(U[:, :j], Uo[:, :j]) < 1e-3
    assert max_principal_sine(V[:, :j], Vo[:, :j]) < 1e-3
    # and the half-precision path, on the same input, within its own tolerance
    U2, S2, _ = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=17)
    assert np.abs(S2[:j] / So[:j] - 1).max() < 1e-3
