"""GPU parity tests: every stage of the per-snapshot refresh, through the C-ABI,
against the CPU oracle on the same seeded inputs."""
import numpy as np
import pytest
import scipy.sparse as sp

import tsvd_gb300 as T
import workloads as W
from oracle import native
from oracle.tree_oracle import (OracleTreeSVD, frpca as oracle_frpca, gaussian_matrix,
                                log_transform, lp_scores)

from helpers import (gap_index, gram_rel_err, max_principal_sine, push_identity_residual,
                     residual_error_bound, transition)

pytestmark = pytest.mark.gpu


def small_cfg(directed=False, n=6000, m=40000, sources=64, n_parts=4, rank_d=32, snapshots=4):
    base = "rmat-d-2.7m" if directed else "rmat-u-100k"
    c = W.scaled(base, n=n, m=m, sources=sources, n_parts=n_parts, rank_d=rank_d,
                 snapshots=snapshots)
    c["rmax"] = 1e-5
    return c


@pytest.mark.parametrize("directed", [False, True])
def test_graph_insert_bit_exact(directed):
    cfg = small_cfg(directed)
    _, snaps, src = W.build(cfg, seed=11)
    g = native.OracleGraph(cfg["n"], directed)
    with T.Session(cfg["n"], src, **W.session_kwargs(cfg)) as s:
        for k, e in enumerate(snaps):
            if k == 2:  # a batch with repeated pairs and a self loop: stored as given
                e = np.concatenate([e, e[:5], [[7, 7]]]).astype(np.int32)
            s.graph_insert(e)
            g.insert(e)
            for d in range(2 if directed else 1):
                off_g, nb_g = s.adjacency(d)
                off_o, nb_o = g.adjacency(d)
                assert np.array_equal(off_g, off_o)
                assert np.array_equal(nb_g, nb_o)
                deg_g, fo_g = s.degrees(d)
                deg_o, fo_o = g.degrees(d)
                assert np.array_equal(deg_g, deg_o) and np.array_equal(fo_g, fo_o)


def test_graph_insert_empty_and_invalid():
    cfg = small_cfg()
    _, snaps, src = W.build(cfg, seed=3)
    with T.Session(cfg["n"], src, **W.session_kwargs(cfg)) as s:
        s.graph_insert(snaps[0])
        before = s.adjacency(0)
        s.graph_insert(np.zeros((0, 2), np.int32))
        with pytest.raises(T.TsvdError) as ei:
            s.graph_insert(np.array([[0, cfg["n"]]], np.int32))
        assert ei.value.status == 1
        after = s.adjacency(0)
        assert np.array_equal(before[1], after[1])


def _ppr_checks(s, g, src, cfg, transpose, oracle=None):
    d = 1 if transpose else 0
    off, nb = g.adjacency(d)
    P, deg = transition(cfg["n"], off, nb)
    p = s.ppr_state(transpose, 1)
    r = s.ppr_state(transpose, 0)
    alpha, rmax = cfg["alpha"], cfg["rmax"]
    # exact forward-push identity p (I - (1-a) P) = a (e_s - r), any push order
    assert push_identity_residual(p, r, src, P, alpha) < 2e-5
    # every residual of a vertex that can push is at most rmax
    elig = deg > 0
    assert (r[:, elig] <= np.float32(rmax)).all()
    assert (p >= 0).all()
    if oracle is not None:
        # both states are within alpha |r| (I-(1-a)P)^-1 of the exact PPR
        po, ro = oracle.reserve().astype(np.float64), oracle.residue()
        bound = residual_error_bound(r, P, alpha) + residual_error_bound(ro, P, alpha)
        assert (np.abs(p.astype(np.float64) - po) <= bound * (1 + 1e-3) + 1e-6).all()


@pytest.mark.parametrize("directed", [False, True])
def test_ppr_from_scratch_and_dynamic(directed):
    cfg = small_cfg(directed)
    _, snaps, src = W.build(cfg, seed=5)
    g = native.OracleGraph(cfg["n"], directed)
    ors = [native.OraclePPR(cfg["n"], src) for _ in range(2 if directed else 1)]
    kw = W.session_kwargs(cfg, dynamic_start=2)
    with T.Session(cfg["n"], src, **kw) as s:
        for it, e in enumerate(snaps[:3], start=1):
            s.graph_insert(e)
            g.insert(e)
            for t in range(2 if directed else 1):
                s.ppr_refresh(it, bool(t))
                s.ppr_push(bool(t))
                ors[t].refresh(g, t, it, 2, cfg["alpha"], cfg["rmax"])
                ors[t].push(g, t, cfg["alpha"], cfg["rmax"])
                _ppr_checks(s, g, src, cfg, bool(t), ors[t])


SCHEDULES = {
    "rmax": {},
    # threshold schedule rmax * 8^k, k = 2, 1, 0, for every vertex
    "levels": dict(push_levels=3, push_ratio=8.0),
    # the same schedule for hubs only (deg >= 1024); the rest push at rmax
    "hub-levels": dict(push_levels=3, push_ratio=8.0, push_hub_degree=1024),
}


@pytest.mark.parametrize("schedule", sorted(SCHEDULES))
@pytest.mark.parametrize("directed", [False, True])
def test_ppr_hub_vertices(directed, schedule):
    """Vertices with thousands of neighbours take the hub path: their pushes
    are split into 1024-neighbour units (push_heavy_kernel). Three hubs of
    2500-3000 neighbours on top of a small R-MAT graph, sources among the
    hubs and their neighbours; same checks against the FIFO oracle, under
    each threshold schedule (the last level of every schedule is the plain
    rmax test, so each leaves the same invariant)."""
    cfg = small_cfg(directed, n=5000, m=20000)
    _, snaps, _ = W.build(cfg, seed=9)
    rng = np.random.default_rng(9)
    hubs = np.array([17, 1234, 4321], np.int32)
    star = []
    for h, k in zip(hubs, (2500, 2800, 3000)):
        nb = rng.choice(np.setdiff1d(np.arange(cfg["n"]), hubs), k, replace=False).astype(np.int32)
        star.append(np.stack([np.full(k, h, np.int32), nb], 1))
        star.append(np.stack([nb[:k // 2], np.full(k // 2, h, np.int32)], 1))
    first = np.concatenate([snaps[0]] + star).astype(np.int32)
    src = np.unique(np.concatenate([hubs, star[0][:20, 1], rng.choice(cfg["n"], 20, replace=False)]))
    src = src.astype(np.int32)
    g = native.OracleGraph(cfg["n"], directed)
    ors = [native.OraclePPR(cfg["n"], src) for _ in range(2 if directed else 1)]
    kw = W.session_kwargs(cfg, dynamic_start=2)
    kw.update(SCHEDULES[schedule])
    with T.Session(cfg["n"], src, **kw) as s:
        for it, e in enumerate([first, snaps[1], snaps[2]], start=1):
            s.graph_insert(e)
            g.insert(e)
            deg, _ = g.degrees(0)
            assert deg[hubs].min() > 2 * 1024
            for t in range(2 if directed else 1):
                s.ppr_refresh(it, bool(t))
                s.ppr_push(bool(t))
                ors[t].refresh(g, t, it, 2, cfg["alpha"], cfg["rmax"])
                ors[t].push(g, t, cfg["alpha"], cfg["rmax"])
                _ppr_checks(s, g, src, cfg, bool(t), ors[t])


def test_ppr_intdiv_refresh_tracks_oracle():
    cfg = small_cfg()
    _, snaps, src = W.build(cfg, seed=9)
    g = native.OracleGraph(cfg["n"], False)
    o = native.OraclePPR(cfg["n"], src)
    kw = W.session_kwargs(cfg, dynamic_start=2)
    kw["refresh_mode"] = T.REFRESH_INTDIV
    with T.Session(cfg["n"], src, **kw) as s:
        for it, e in enumerate(snaps[:3], start=1):
            s.graph_insert(e)
            g.insert(e)
            s.ppr_refresh(it)
            s.ppr_push()
            o.refresh(g, 0, it, 2, cfg["alpha"], cfg["rmax"], intdiv=True)
            o.push(g, 0, cfg["alpha"], cfg["rmax"])
        off, nb = g.adjacency(0)
        P, deg = transition(cfg["n"], off, nb)
        p = s.ppr_state(False, 1).astype(np.float64)
        r = s.ppr_state(False, 0)
        # the integer-division refresh breaks the push identity (in the
        # reference as here), so compare the states directly
        assert (r[:, deg > 0] <= np.float32(cfg["rmax"])).all()
        po = o.reserve().astype(np.float64)
        assert np.linalg.norm(p - po) <= 1e-2 * np.linalg.norm(po)


def test_block_materialize_matches_transform():
    cfg = small_cfg()
    _, snaps, src = W.build(cfg, seed=13)
    kw = W.session_kwargs(cfg)
    with T.Session(cfg["n"], src, **kw) as s:
        s.graph_insert(snaps[0])
        s.ppr_refresh(1)
        s.ppr_push()
        dirty = s.blocks_materialize(1)
        assert dirty.all()
        p = s.ppr_state(False, 1).astype(np.float64)
        info = s.block_info()
        cd = cfg["n"] // cfg["n_parts"]
        for b in range(cfg["n_parts"]):
            c0 = b * cd
            c1 = cfg["n"] if b == cfg["n_parts"] - 1 else c0 + cd
            ref = log_transform(p[:, c0:c1], cfg["rmax"], cfg["transform"], cfg["n"])
            got = s.block_dense(b).astype(np.float64)
            # half precision storage: |err| <= 2^-11 |a| (+ subnormal floor)
            assert (np.abs(got - ref) <= 2.0 ** -11 * np.abs(ref) + 1e-7).all()
            assert info["norm"][b] == pytest.approx(np.linalg.norm(ref), rel=1e-5)
            assert info["nnz"][b] == np.count_nonzero(ref)


def _random_lowrank_csr(m, n, rank, density, seed):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    U = rng.standard_normal((m, rank))
    V = rng.standard_normal((rank, n))
    s = 0.97 ** np.arange(rank)
    D = (U * s) @ V
    mask = rng.random((m, n)) < density
    D = np.where(mask, np.abs(D), 0.0)
    return sp.csr_matrix(D)


def test_frpca_abi_block_sized():
    """A 3000 x 12000 block at 10 % density, rank 128, q = 6: the products
    run over several 384-row tiles and hundreds of 32-deep K stages of the
    tensor-core GEMM in both directions. Against the oracle's frPCA on the
    same Omega."""
    m, n, k, q = 3000, 12000, 128, 6
    A = _random_lowrank_csr(m, n, 400, 0.1, seed=4)
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=91)
    omega = gaussian_matrix(91, 0, n, k + 5)
    Uo, So, _ = oracle_frpca(A.toarray(), k, q, omega=omega)
    So = So[::-1]
    Uo = Uo[:, ::-1]
    assert np.allclose(S, So, rtol=1e-3, atol=1e-6 * So[0]), np.abs(S / So - 1).max()
    j = gap_index(So, k)
    assert j > 0
    assert max_principal_sine(U[:, :j], Uo[:, :j]) < 1e-2
    assert np.abs(U.T @ U - np.eye(k)).max() < 1e-3


def test_frpca_abi_matches_oracle():
    m, n, k, q = 300, 2000, 32, 6
    A = _random_lowrank_csr(m, n, 80, 0.3, seed=1)
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=77)
    l = k + 5
    omega = gaussian_matrix(77, 0, n, l)
    Uo, So, Vo = oracle_frpca(A.toarray(), k, q, omega=omega)
    So = So[::-1]
    Uo = Uo[:, ::-1]
    assert np.allclose(S, So, rtol=1e-3, atol=1e-6 * So[0])
    j = gap_index(So, k)
    assert j > 0
    assert max_principal_sine(U[:, :j], Uo[:, :j]) < 1e-2
    assert np.abs(U.T @ U - np.eye(k)).max() < 1e-3
    # the reconstruction U S V^T agrees with the oracle's
    R = (U * S) @ V.T
    Ro = (Uo * So) @ Vo[:, ::-1].T
    assert np.linalg.norm(R - Ro) / np.linalg.norm(Ro) < 1e-3


@pytest.mark.parametrize("name", ["q6", "q3"])
def test_frpca_abi_matches_reference_golden(name):
    """The GPU frPCA against the reference's own frpca.c output on the same
    matrix (tests/golden/ref_frpca_*.npz, made by the reference compiled
    against the MKL stand-in). The two draw different Gaussian matrices, so
    the comparison is on what the randomization leaves fixed: the leading
    singular values and the gap-separated leading subspace."""
    import os
    import scipy.sparse as sp
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_frpca_%s.npz" % name))
    A = sp.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
    k, q = int(z["k"]), int(z["q"])
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=5)
    Sr, Ur, Vr = z["S"][::-1], z["U"][:, ::-1], z["V"][:, ::-1]  # reference order: ascending
    j = gap_index(Sr, k)
    assert j > 0
    assert np.allclose(S[:j], Sr[:j], rtol=1e-3)
    assert max_principal_sine(U[:, :j], Ur[:, :j]) < 1e-2
    assert max_principal_sine(V[:, :j], Vr[:, :j]) < 1e-2


def _lowrank_exact(m, n, s, seed):
    rng = np.random.default_rng(seed)
    U0, _ = np.linalg.qr(rng.standard_normal((m, len(s))))
    V0, _ = np.linalg.qr(rng.standard_normal((n, len(s))))
    return sp.csr_matrix((U0 * s) @ V0.T), U0


def test_frpca_abi_repeated_singular_values():
    """A triple and a double singular value at the top of a full-rank
    spectrum: equal eigenvalues of the Gram form a cluster, whose vectors
    must still come out orthonormal and span the right subspaces."""
    m, n, k, q = 300, 400, 10, 4
    s = np.concatenate([[5.0, 5.0, 5.0, 2.0, 1.0, 1.0], 0.5 * 0.9 ** np.arange(40)])
    A, U0 = _lowrank_exact(m, n, s, seed=5)
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=11)
    assert np.allclose(S[:6], s[:6], rtol=2e-3)
    assert np.abs(U.T @ U - np.eye(k)).max() < 1e-3
    assert max_principal_sine(U[:, :3], U0[:, :3]) < 1e-2
    assert max_principal_sine(U[:, :6], U0[:, :6]) < 1e-2


def test_frpca_abi_rank_deficient():
    """Rank 6 < k: the leading 6 singular triplets are exact and orthonormal,
    the rest are (numerically) zero; nothing is NaN. The directions of the
    zero singular values are arbitrary (the reference's eigSVD divides by
    them), so only their singular values are checked."""
    m, n, k, q = 300, 400, 10, 4
    s = np.array([5.0, 5.0, 5.0, 2.0, 1.0, 1.0])
    A, U0 = _lowrank_exact(m, n, s, seed=6)
    U, S, V = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=11)
    assert np.isfinite(U).all() and np.isfinite(S).all() and np.isfinite(V).all()
    assert np.allclose(S[:6], s, rtol=2e-3)
    assert np.all(S[6:] < 1e-2)
    assert np.abs(U[:, :6].T @ U[:, :6] - np.eye(6)).max() < 1e-3
    assert max_principal_sine(U[:, :6], U0) < 1e-2


@pytest.mark.parametrize("directed,n,sources,parts,h,d", [
    (False, 8000, 96, 4, 2, 32), (True, 8000, 96, 4, 2, 32), (False, 7003, 40, 4, 2, 32),
    (False, 8000, 96, 8, 8, 40), (True, 8000, 300, 8, 8, 64), (False, 8000, 120, 64, 8, 40)])
def test_session_matches_oracle_pipeline(directed, n, sources, parts, h, d):
    """Whole snapshots through tsvd_session_step. The block stages (log
    transform, lazy test, frPCA, merge) are checked against the oracle run on
    the GPU's own reserve, so the comparison isolates their arithmetic; the
    PPR stage is covered by test_ppr_from_scratch_and_dynamic. The third case
    has a wider last block (7003 = 3 x 1750 + 1753) and fewer sources than
    one 64-source chunk. The last three merge 8 children at a time (the
    reference's run.sh arity): 320, 512 and 320 columns per merge, wider than
    one Jacobi matrix, through the subspace-iteration merge; the last with two
    merge levels (64 -> 8 -> 1)."""
    cfg = small_cfg(directed, n=n, m=60000, sources=sources, n_parts=parts, rank_d=d,
                    snapshots=4)
    cfg["hierarchy_n"] = h
    _, snaps, src = W.build(cfg, seed=21)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    okw = dict(kw)
    okw.pop("seed")
    o = OracleTreeSVD(cfg["n"], src, seed=kw["seed"], **okw)
    frac = kw["dirty_frac"]
    with T.Session(cfg["n"], src, **kw) as s:
        for e in snaps:
            st = s.step(e)
            p = s.ppr_state(False, 1).astype(np.float64)
            if directed:
                p += s.ppr_state(True, 1)
            emb_o = o.step(e, reserve=p)
            info = s.block_info()
            assert np.allclose(info["norm"], o.norm, rtol=1e-5)
            if kw["dirty_rule"] == T.DIRTY_FROBENIUS:
                tie = np.abs(o.norm_diff - frac * o.norm) <= 1e-3 * o.norm
            else:
                lhs = o.resid + o.norm_diff
                tie = np.abs(lhs - kw["delta"] * np.sqrt(2) * o.norm) <= 1e-3 * o.norm
            assert np.array_equal(info["dirty"][~tie], o.dirty[~tie])
            if tie.any():
                # a near-tie decision may legitimately differ; when one does,
                # the two sides accept different block matrices from here on
                # (norm_diff is taken against the last accepted one), so
                # later snapshots are no longer comparable
                if not np.array_equal(info["dirty"][tie], o.dirty[tie]):
                    break
                continue
            assert st["factorized_blocks"] == len(o.last_factorized)
            for b in o.last_factorized:
                _, sg = s.tree_factor(s.leaf_start + b)
                so = o.sigma[s.leaf_start + b]
                j = gap_index(so, cfg["rank_d"])
                assert np.allclose(sg[:j], so[:j], rtol=1e-3), (b, np.abs(sg[:j] / so[:j] - 1).max())
            emb = s.embedding()
            assert np.isfinite(emb).all()
            _, sig = s.tree_factor(0)
            assert np.allclose(sig[:16], o.sigma[0][:16], rtol=1e-3)
            assert gram_rel_err(emb, emb_o) < 5e-3


@pytest.mark.parametrize("directed", [False, True])
def test_lp_right_factor_and_scores(directed):
    """LP drivers: V_b = A_b^T U for the blocks refreshed in a snapshot (U that
    snapshot's root factor, kept beside V_b), untouched for the others; pair
    scores U_b[row(i)] . V[j], plain and degree-scaled, against the oracle's
    restatement on the GPU's own blocks and factors."""
    cfg = small_cfg(directed, n=6000, m=40000, sources=64, n_parts=4, rank_d=32, snapshots=4)
    _, snaps, src = W.build(cfg, seed=31)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw.update(transform=T.TRANSFORM_LOG10_LP, root_scaling=T.ROOT_U,
              dirty_rule=T.DIRTY_FROBENIUS, dirty_frac=0.3 if directed else 0.15,
              lp_right_factor=True)
    P, cd = cfg["n_parts"], cfg["n"] // cfg["n_parts"]
    rng = np.random.default_rng(7)
    lp_U = [None] * P
    V_prev = None
    clean_seen = False
    with T.Session(cfg["n"], src, **kw) as s:
        for e in snaps:
            s.step(e)
            U = s.embedding()
            assert np.abs(U.T @ U - np.eye(cfg["rank_d"])).max() < 5e-3  # root U (fp32 M V S^-1)
            V = s.lp_right_factor().astype(np.float64)
            dirty = s.block_info()["dirty"]
            for b in range(P):
                c0 = b * cd
                c1 = cfg["n"] if b == P - 1 else c0 + cd
                if dirty[b]:
                    ref = s.block_dense(b).astype(np.float64).T @ U
                    assert np.abs(V[c0:c1] - ref).max() <= 1e-4 * max(np.abs(ref).max(), 1e-30)
                    lp_U[b] = U.copy()
                else:
                    clean_seen = True
                    assert np.array_equal(V[c0:c1], V_prev[c0:c1])
            V_prev = V
            pairs = np.stack([rng.choice(src, 500), rng.integers(0, cfg["n"], 500)], 1)
            deg_i, _ = s.degrees(0)
            deg_j, _ = s.degrees(1 if directed else 0)
            for scaled in (False, True):
                got = s.lp_scores(pairs, degree_scaled=scaled)
                ref = lp_scores(lp_U, V, src, cd, P, pairs, scaled, deg_i, deg_j)
                assert np.allclose(got, ref, rtol=1e-9, atol=1e-12 * max(np.abs(ref).max(), 1.0))
        not_a_source = int(np.setdiff1d(np.arange(cfg["n"]), src)[0])
        with pytest.raises(T.TsvdError):
            s.lp_scores(np.array([[not_a_source, 0]]))
    assert clean_seen  # the lazy rule kept some block's V and U across a snapshot


@pytest.mark.parametrize("directed,rule", [(False, T.DIRTY_REFERENCE), (True, T.DIRTY_FROBENIUS)])
def test_pipelined_run_matches_steps(directed, rule):
    """tsvd_session_run overlaps the factor stage of snapshot k with the push
    of snapshot k+1. Its per-snapshot embeddings and refactorized block
    counts agree with one-at-a-time steps up to the push-order differences of
    two PPR runs (the reference dirty rule reads the previous snapshot's
    residuals, so a stale read would change which blocks are refactorized).
    Push order can flip a lazy decision that is within a few percent of its
    threshold; the comparison stops at the first such near-tie of the stepped
    run. The first snapshot only grows the graph (lazy_update_start_iter 3,
    the second is pushed from scratch): its embedding is zeros."""
    cfg = small_cfg(directed, n=8000, m=60000, sources=96, n_parts=4, rank_d=32, snapshots=6)
    _, snaps, src = W.build(cfg, seed=41)
    kw = W.session_kwargs(cfg, dynamic_start=3, lazy_start=3)
    kw["dirty_rule"] = rule
    ref_emb, ref_stats = [], []
    tie_from = len(snaps)
    with T.Session(cfg["n"], src, **kw) as a:
        prev_resid = None
        for k, e in enumerate(snaps):
            st = a.step(e)
            ref_stats.append(st)
            ref_emb.append(a.embedding() if not st["skipped"] else None)
            info = a.block_info()
            if st["iter"] >= kw["lazy_update_start_iter"]:
                if rule == T.DIRTY_REFERENCE:
                    lhs = prev_resid + info["norm_diff"]
                    thr = kw["delta"] * np.sqrt(2) * info["norm"]
                else:
                    lhs, thr = info["norm_diff"], kw["dirty_frac"] * info["norm"]
                if (np.abs(lhs - thr) <= 0.05 * info["norm"]).any():
                    tie_from = min(tie_from, k)
            prev_resid = info["resid"]
        _, sig_ref = a.tree_factor(0)
    assert tie_from >= 2  # the from-scratch snapshot and the first lazy decision compare
    import torch
    dev = torch.from_numpy(np.concatenate(snaps)).cuda()
    off = np.concatenate([[0], np.cumsum([len(e) for e in snaps])])
    for use_device in (False, True):
        with T.Session(cfg["n"], src, **kw) as s:
            if use_device:
                stats, emb = s.run_device(dev.data_ptr(), off)
            else:
                stats, emb = s.run(snaps)
            _, sig = s.tree_factor(0)
            assert s.stats()["iter"] == len(snaps)
            assert np.allclose(s.embedding(), emb[-1])
        assert [x["iter"] for x in stats] == [x["iter"] for x in ref_stats]
        assert [x["skipped"] for x in stats] == [x["skipped"] for x in ref_stats]
        assert stats[0]["skipped"] == 1 and not emb[0].any()
        for k in range(1, len(snaps)):
            st = stats[k]
            assert np.isfinite(emb[k]).all()
            assert st["edges_inserted"] == len(snaps[k])
            assert st["ms_total"] >= st["ms_push"] > 0 and st["ms_frpca"] > 0
            if k < tie_from:
                assert st["factorized_blocks"] == ref_stats[k]["factorized_blocks"], k
                err = gram_rel_err(emb[k], ref_emb[k])
                assert err < 3e-2, (k, err)
        if tie_from == len(snaps):
            assert np.allclose(sig[:16], sig_ref[:16], rtol=5e-3)


def test_pipelined_run_lp_and_errors():
    """The LP right factor on the pipelined path: after the run, the blocks
    refreshed in the last snapshot hold V_b = A_b^T U with that snapshot's U.
    A snapshot with an invalid endpoint fails the run with TSVD_ERR_INVALID,
    after the snapshot before it has completed; the session stays usable."""
    cfg = small_cfg(True, n=6000, m=40000, sources=64, n_parts=4, rank_d=32, snapshots=4)
    _, snaps, src = W.build(cfg, seed=43)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw.update(transform=T.TRANSFORM_LOG10_LP, root_scaling=T.ROOT_U, lp_right_factor=True)
    P, cd = cfg["n_parts"], cfg["n"] // cfg["n_parts"]
    with T.Session(cfg["n"], src, **kw) as s:
        stats, emb = s.run(snaps)
        U = emb[-1]
        assert np.abs(U.T @ U - np.eye(cfg["rank_d"])).max() < 5e-3
        V = s.lp_right_factor().astype(np.float64)
        dirty = s.block_info()["dirty"]
        assert dirty.any()
        for b in np.flatnonzero(dirty):
            c0 = b * cd
            c1 = cfg["n"] if b == P - 1 else c0 + cd
            ref = s.block_dense(b).astype(np.float64).T @ U
            assert np.abs(V[c0:c1] - ref).max() <= 1e-4 * max(np.abs(ref).max(), 1e-30)
    bad = [snaps[0], snaps[1], np.array([[0, cfg["n"]]], np.int32), snaps[2]]
    with T.Session(cfg["n"], src, **kw) as s:
        with pytest.raises(T.TsvdError) as ei:
            s.run(bad)
        assert ei.value.status == 1
        assert s.stats()["iter"] == 2  # the last completed snapshot
        s.step(snaps[2])
        assert np.isfinite(s.embedding()).all()


def test_host_reserve_matches_device_reserve():
    """ppr_host_reserve: the reserve p in mapped pinned host memory (reached
    over NVLink-C2C), the residues in HBM. Refresh and push keep the push
    identity and the rmax bound and stay within the error bound of the
    oracle, and whole snapshots give the embedding of the all-device layout
    up to push order."""
    cfg = small_cfg(True)
    _, snaps, src = W.build(cfg, seed=47)
    g = native.OracleGraph(cfg["n"], True)
    ors = [native.OraclePPR(cfg["n"], src) for _ in range(2)]
    kw = W.session_kwargs(cfg, dynamic_start=2)
    with T.Session(cfg["n"], src, ppr_host_reserve=True, **kw) as s:
        for it, e in enumerate(snaps[:3], start=1):
            s.graph_insert(e)
            g.insert(e)
            for t in range(2):
                s.ppr_refresh(it, bool(t))
                s.ppr_push(bool(t))
                ors[t].refresh(g, t, it, 2, cfg["alpha"], cfg["rmax"])
                ors[t].push(g, t, cfg["alpha"], cfg["rmax"])
                _ppr_checks(s, g, src, cfg, bool(t), ors[t])
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    emb = {}
    for host in (False, True):
        with T.Session(cfg["n"], src, ppr_host_reserve=host, **kw) as s:
            for e in snaps:
                s.step(e)
            emb[host] = s.embedding()
    assert gram_rel_err(emb[True], emb[False]) < 3e-2


def _cos_cols(X, Y):
    return np.abs(np.sum(X * Y, 0)) / (np.linalg.norm(X, axis=0) * np.linalg.norm(Y, axis=0))


def test_merge_svd_matches_reference_golden():
    """tsvd_merge_svd (the tree merge on one matrix) against the reference's
    own dense_sub_svd_function output (tests/golden/ref_merge.npz, LAPACK
    gesvd through its truncated_singular_value_decomposition)."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_merge.npz"))
    US, sig = T.merge_svd(z["M"], int(z["d"]))
    assert np.allclose(sig, z["sigma"], rtol=1e-5)
    assert (1 - _cos_cols(US, z["US"])).max() < 1e-5


@pytest.mark.parametrize("cols", [2, 3, 17, 64, 133, 255])
def test_merge_svd_sizes_and_cluster_splits(cols):
    """One eigenproblem spread over the CTAs of a cluster, at the sizes where
    the split changes: 2 columns (one pair, one CTA, nobody moves), 3 (a
    dummy player, two CTAs of one slot), 17 (two CTAs of 5 and 4 slots), 64
    (eight CTAs of 4 slots), 133 (eight CTAs of 9 slots, the last with 4; a
    dummy player), 255 (eight CTAs of 16 slots, a dummy player). Singular
    values and vectors against an exact SVD."""
    rng = np.random.default_rng(cols)
    rows = 300
    Q = np.linalg.qr(rng.standard_normal((rows, cols)))[0]
    Vt = np.linalg.qr(rng.standard_normal((cols, cols)))[0].T
    M = (Q * np.geomspace(1e2, 1e-1, cols)) @ Vt
    d = min(cols, 16)
    US, sig = T.merge_svd(M, d)
    U0, S0, _ = np.linalg.svd(M.astype(np.float32).astype(np.float64), full_matrices=False)
    assert np.allclose(sig, S0[:d], rtol=1e-4), np.abs(sig / S0[:d] - 1).max()
    assert (1 - _cos_cols(US, U0[:, :d] * S0[:d])).max() < 1e-4


@pytest.mark.parametrize("rows,cols,d,top,bottom", [(600, 256, 128, 1e3, 1e-1), (400, 512, 64, 1e2, 1.0)])
def test_merge_svd_wide_spread(rows, cols, d, top, bottom):
    """Singular values spread over four orders of magnitude (the Gram squares
    that to eight): the eigen-solve's fp64 refinement keeps every kept value
    within 1e-4 of an exact SVD. 512 columns go through the wide merge's
    subspace iteration."""
    rng = np.random.default_rng(rows + cols)
    Q = np.linalg.qr(rng.standard_normal((rows, min(rows, cols))))[0]
    Vt = np.linalg.qr(rng.standard_normal((cols, min(rows, cols))))[0].T
    s = np.geomspace(top, bottom, min(rows, cols))
    M = (Q * s) @ Vt
    US, sig = T.merge_svd(M, d)
    U0, S0, _ = np.linalg.svd(M.astype(np.float32).astype(np.float64), full_matrices=False)
    assert np.allclose(sig, S0[:d], rtol=1e-4), np.abs(sig / S0[:d] - 1).max()
    assert (1 - _cos_cols(US, U0[:, :d] * S0[:d])).max() < 1e-4
