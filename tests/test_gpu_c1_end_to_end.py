"""End-to-end parity at the CPU-runnable configuration, exactly as configured:
undirected R-MAT (0.57, 0.19, 0.19, 0.05), N = 100,000, M = 1,000,000, ten
snapshots (the first with half the edges), |S| = 500, alpha = 0.2,
rmax = 1e-6, ln(x N) transform, 16 column blocks, d = 128, q = 6, binary
merge tree, the reference's lazy rule (delta = 0.3) from the second snapshot.

Every snapshot runs through tsvd_session_step on the GPU and, independently,
through the FP64 oracle with its own FIFO push (Code/Tree_u_NC.cpp:507-866
restated in oracle/). A second oracle runs the block stages on the GPU's own
reserve, which isolates the log transform, lazy test, frPCA and merges from
the push-order difference. Checked on every snapshot:

* PPR: every entry of both the GPU's and the oracle's reserve lies within
  the forward-push bound of the exact FP64 PPR (power iteration to 1e-13);
  the bound is alpha |r| (I - (1-alpha) P)^-1 of each state's own residues,
  which is rmax d(v) wherever every residue lies in [0, rmax] (undirected
  graph) and stays exact where the dynamic refresh left negative residues,
  plus 64 roundings of relative 2^-24 per entry for the fp32 storage both
  sides share with the reference's dense path.
  No positive residue above rmax remains on either side.
* dirty blocks: identical to the oracle run on the GPU's reserve; identical to
  the independent oracle outside near-ties (decision margin below 2 %, where
  the two pushes' matrices may legitimately fall on either side).
* root singular values within 1e-3 relative against the oracle run on the
  GPU's reserve (the factorization arithmetic alone), plus the error the
  mixed form's half-precision block storage allows by Weyl's inequality:
  each stored entry is within 2^-12 of itself, so every singular value moves
  by at most 2^-12 ||A||_F (this term matters only in the tail of the 128
  kept values, which sit far below the first); within 1e-2 against the
  independent oracle (the two pushes stop at different valid states; with
  the ln(x N) transform at rmax = 1e-6 that moves the root singular values
  by up to 5.3e-3, measured on a GB300); the largest principal-angle sine of
  the gap-separated leading subspace within 1e-2 against both (against the
  independent one while its dirty decisions have agreed). The leading
  subspace ends at a relative gap of 5 %. Against the independent oracle the
  two inputs differ (the push-order freedom above), and no algorithm can do
  better than the rotation that difference itself causes: there the bound is
  1e-2 or twice the sin-theta bound ||A_gpu - A_oracle||_2 / (sigma_j -
  sigma_j+1) of the two log matrices, whichever is larger (the first
  snapshot's 5 %-gap subspace turned by 1.1e-2, measured on a GB300).

The tree's embedding is not the exact SVD of the current matrix: blocks the
lazy rule keeps are a snapshot old, and every block is truncated to rank d
before the merge. That gap belongs to the algorithm (the FP64 oracle shows
it too) and is printed, not asserted.
"""
import time

import numpy as np
import pytest
import scipy.sparse as sp

import tsvd_gb300 as T
import workloads as W
from helpers import gap_index, max_principal_sine, spectral_norm
from oracle.tree_oracle import OracleTreeSVD, log_transform

pytestmark = pytest.mark.gpu


def _torch_cuda():
    try:
        import torch
        return torch if torch.cuda.is_available() else None
    except Exception:
        return None


class _Propagator:
    """x -> x P for row-stochastic P (dangling rows zero), |S| rows at a time,
    in fp64 (cuSPARSE through torch when a GPU is present, scipy otherwise)."""

    def __init__(self, n, off, nbr):
        deg = np.diff(off)
        rows = np.repeat(np.arange(n), deg)
        P = sp.csr_matrix((np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)[rows], (rows, nbr)),
                          shape=(n, n))
        self.PT = P.T.tocsr()
        self.torch = _torch_cuda()
        if self.torch is not None:
            t = self.torch
            self.PTd = t.sparse_csr_tensor(t.from_numpy(self.PT.indptr.astype(np.int64)),
                                           t.from_numpy(self.PT.indices.astype(np.int64)),
                                           t.from_numpy(self.PT.data), size=(n, n),
                                           dtype=t.float64, device="cuda")
        self.deg = deg

    def to(self, x):
        return self.torch.from_numpy(np.ascontiguousarray(x.T)).cuda() if self.torch else x.T.copy()

    def back(self, y):
        return (y.cpu().numpy() if self.torch else y).T

    def step(self, yT):  # yT: N x |S| (columns are sources)
        return self.PTd @ yT if self.torch else self.PT @ yT


def exact_ppr(prop, sources, alpha, iters=130):
    """pi_s = alpha sum_t (1-alpha)^t e_s P^t; the omitted tail is below
    (1-alpha)^iters = 2.5e-13 entrywise."""
    y0 = np.zeros((len(sources), prop.PT.shape[0]))
    y0[np.arange(len(sources)), sources] = 1.0
    y = prop.to(y0)
    acc = alpha * y
    for _ in range(iters):
        y = (1 - alpha) * prop.step(y)
        acc = acc + alpha * y
    return prop.back(acc)


def push_bound(prop, r, alpha, iters=100):
    """alpha |r| (I - (1-alpha) P)^-1, truncated after `iters` terms plus the
    tail's entrywise bound ||r_s||_1 (1-alpha)^iters, so it stays an upper bound."""
    a = np.abs(r.astype(np.float64))
    y = prop.to(a)
    acc = alpha * y
    for _ in range(iters):
        y = (1 - alpha) * prop.step(y)
        acc = acc + alpha * y
    return prop.back(acc) + (a.sum(axis=1) * (1 - alpha) ** iters)[:, None]


def test_c1_end_to_end_against_the_fp64_oracle():
    cfg = W.scaled("rmat-u-100k")
    assert (cfg["n"], cfg["m"], cfg["snapshots"], cfg["sources"], cfg["n_parts"],
            cfg["rank_d"], cfg["passes_q"], cfg["hierarchy_n"]) == \
        (100_000, 1_000_000, 10, 500, 16, 128, 6, 2)
    _, snaps, src = W.build(cfg, seed=20231)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    okw = dict(kw)
    okw.pop("seed")
    indep = OracleTreeSVD(cfg["n"], src, seed=kw["seed"], threads=16, **okw)  # its own push
    iso = OracleTreeSVD(cfg["n"], src, seed=kw["seed"], **okw)                # on the GPU's reserve
    n, alpha, rmax, d = cfg["n"], cfg["alpha"], cfg["rmax"], cfg["rank_d"]
    agreed = {"iso": True, "indep": True}  # each oracle's dirty decisions matched so far
    report = []

    def ties(o, resid_before, tol):
        lhs = resid_before + o.norm_diff
        return np.abs(lhs / (kw["delta"] * np.sqrt(2) * o.norm) - 1) < tol

    with T.Session(n, src, **kw) as s:
        for it, e in enumerate(snaps):
            t0 = time.perf_counter()
            before = {"iso": iso.resid.copy(), "indep": indep.resid.copy()}
            st = s.step(e)
            emb_o = indep.step(e)
            p = s.ppr_state(False, 1).astype(np.float64)
            r = s.ppr_state(False, 0).astype(np.float64)
            emb_i = iso.step(e, reserve=p)
            # ---- PPR against the exact FP64 PPR, both sides
            off, nbr = indep.g.adjacency(0)
            prop = _Propagator(n, off, nbr)
            pi = exact_ppr(prop, src, alpha)
            po = indep.reserve()
            ro = indep.ppr[0].residue().astype(np.float64)
            for name, pp, rr in (("gpu", p, r), ("oracle", po, ro)):
                assert rr.max() <= rmax * (1 + 1e-6), (it, name, rr.max())
                # both states are stored in fp32 (the reference's dense path):
                # an entry carries up to 64 roundings of relative 2^-24
                fp32_slack = 64 * 2.0 ** -24 * np.abs(pp) + 1e-12
                bnd = push_bound(prop, rr, alpha)
                excess = np.abs(pp - pi) - bnd * (1 + 1e-6) - fp32_slack
                assert excess.max() <= 0, (it, name, excess.max())
                if rr.min() >= 0:  # every residue in [0, rmax]: the bound is rmax d(v)
                    simple = (np.abs(pp - pi) - rmax * np.maximum(prop.deg, 1)[None, :] *
                              (1 + 1e-6) - fp32_slack)
                    assert simple.max() <= 0, (it, name, simple.max())
            # ---- dirty blocks (the lazy rule applies from the second snapshot)
            dirty = s.block_info()["dirty"].astype(bool)
            ntie = {}
            for name, o, tol in (("iso", iso, 1e-3), ("indep", indep, 2e-2)):
                tie = ties(o, before[name], tol) if it >= 1 else np.zeros(len(dirty), bool)
                ntie[name] = int(tie.sum())
                if not agreed[name]:
                    continue
                same = dirty == o.dirty.astype(bool)
                assert same[~tie].all(), (it, name, np.flatnonzero(~same))
                if not same.all():
                    agreed[name] = False  # a near-tie fell the other way: histories part here
            # ---- root factor
            emb = s.embedding()
            _, sig = s.tree_factor(0)
            assert np.isfinite(emb).all()
            A_g = log_transform(p, rmax, cfg["transform"], n)
            dA = spectral_norm(A_g - log_transform(po, rmax, cfg["transform"], n))
            fp16_storage = 2.0 ** -12 * float(np.linalg.norm(A_g))
            del A_g
            for name, ref_emb, ref_sig, tol in (("iso", emb_i, iso.sigma[0], 1e-3),
                                                ("indep", emb_o, indep.sigma[0], 1e-2)):
                if not agreed[name]:
                    continue
                err = np.abs(sig - ref_sig)
                allowed = tol * ref_sig + (fp16_storage if name == "iso" else 0.0)
                assert (err <= allowed).all(), (it, name, (err / ref_sig).max(),
                                                int((err - allowed).argmax()))
                j = gap_index(ref_sig, d)
                assert j > 0
                sine = max_principal_sine(emb[:, :j], ref_emb[:, :j])
                bound = 1e-2
                if name == "indep":
                    bound = max(bound, 2 * dA / (ref_sig[j - 1] - ref_sig[j]))
                assert sine <= bound, (it, name, j, sine, bound)
            # ---- the algorithm's own distance to the exact SVD (reported)
            exact_sine = None
            if it in (0, len(snaps) // 2, len(snaps) - 1):
                A = log_transform(po, rmax, cfg["transform"], n)
                Ux, Sx, _ = np.linalg.svd(A, full_matrices=False)
                jx = gap_index(Sx, 16)
                exact_sine = max_principal_sine(emb_o[:, :jx], Ux[:, :jx]) if jx else None
            report.append((it, int(dirty.sum()), ntie["indep"], agreed["indep"],
                           float(np.abs(p - pi).max()), exact_sine, st["ms_total"],
                           time.perf_counter() - t0))
    for row in report:
        print("snapshot %d: dirty %d (near-ties %d, histories agree %s), max |p - pi| %.2e, "
              "oracle tree vs exact SVD leading-subspace sine %s, GPU step %.1f ms, check %.1f s"
              % row)
