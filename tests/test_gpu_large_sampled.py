"""Sampled parity at two bench-sized directed configurations, |S| = 3000,
d = 128, q = 6, alpha = 0.2, rmax = 1e-7:

* Patent-sized: N = 2,738,013, M = 13,960,811, 64 blocks; second snapshot
  1/38 of the edges;
* Wikipedia-sized, the latency workload: N = 6,216,199, M = 177,862,656,
  128 blocks, a 70 % first snapshot then a 1 % (1,778,627-edge) delta; the
  reserve in pinned host memory, as the bench runs it.

One session each, its first (from-scratch) and second (dynamic) snapshots,
checked on samples the CPU oracle can afford:

* 64 of the 3000 sources: their PPR rows in both directions, against the
  oracle's FIFO push of the same sources on the same graph (each state within
  alpha |r| (I - (1-alpha) P)^-1 of the exact PPR, so the two within the sum
  of their bounds, plus fp32 storage slack); no positive residue above rmax
  on a vertex that can push;
* two blocks of the first snapshot (every block is factorized there): the
  block's singular values and leading subspace against the oracle's float64
  frPCA of the same block with the same Gaussian matrix.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import tsvd_gb300 as T
import workloads as W
from helpers import gap_index, max_principal_sine
from oracle import native
from oracle.tree_oracle import frpca as oracle_frpca, gaussian_matrix

pytestmark = pytest.mark.gpu


def _bound(PT, r, alpha, torch, iters=100):
    """alpha |r| (I - (1-alpha) P)^-1 for the rows of r (fp64, on the GPU)."""
    a = np.abs(r.astype(np.float64))
    if torch is not None:
        M = torch.sparse_csr_tensor(torch.from_numpy(PT.indptr.astype(np.int64)),
                                    torch.from_numpy(PT.indices.astype(np.int64)),
                                    torch.from_numpy(PT.data), size=PT.shape,
                                    dtype=torch.float64, device="cuda")
        y = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
        acc = alpha * y
        for _ in range(iters):
            y = (1 - alpha) * (M @ y)
            acc = acc + alpha * y
        out = acc.cpu().numpy().T
    else:
        y = a.T.copy()
        acc = alpha * y
        for _ in range(iters):
            y = (1 - alpha) * (PT @ y)
            acc = acc + alpha * y
        out = acc.T
    return out + (a.sum(axis=1) * (1 - alpha) ** iters)[:, None]


def _transition_T(n, off, nbr):
    deg = np.diff(off)
    rows = np.repeat(np.arange(n), deg)
    P = sp.csr_matrix((np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)[rows], (rows, nbr)),
                      shape=(n, n))
    return P.T.tocsr(), deg


@pytest.mark.parametrize("name,blocks", [("rmat-d-2.7m", (0, 40)),
                                         ("rmat-d-6.2m-1pct", (0, 90))])
def test_bench_sized_session_sampled_against_the_oracle(name, blocks):
    try:
        import torch
        torch = torch if torch.cuda.is_available() else None
    except Exception:
        torch = None
    cfg = W.scaled(name)
    _, snaps, src = W.build(cfg, seed=20231)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw["ppr_host_reserve"] = bool(cfg.get("host_reserve"))
    n, alpha, rmax, d = cfg["n"], cfg["alpha"], cfg["rmax"], cfg["rank_d"]
    rng = np.random.default_rng(64)
    rows = np.sort(rng.choice(len(src), 64, replace=False)).astype(np.int32)
    g = native.OracleGraph(n, True)
    ors = [native.OraclePPR(n, src[rows]) for _ in range(2)]
    with T.Session(n, src, **kw) as s:
        for it, e in enumerate(snaps[:2], start=1):
            s.step(e)
            g.insert(e)
            for t in range(2):
                ors[t].refresh(g, t, it, 2, alpha, rmax, threads=16)
                ors[t].push(g, t, alpha, rmax, threads=16)
                off, nbr = g.adjacency(t)
                PT, deg = _transition_T(n, off, nbr)
                p = s.ppr_state_rows(rows, bool(t), 1).astype(np.float64)
                r = s.ppr_state_rows(rows, bool(t), 0).astype(np.float64)
                po = ors[t].reserve().astype(np.float64)
                ro = ors[t].residue().astype(np.float64)
                assert (r[:, deg > 0] <= np.float32(rmax)).all(), (it, t)
                assert (ro[:, deg > 0] <= np.float32(rmax)).all(), (it, t)
                bound = _bound(PT, r, alpha, torch) + _bound(PT, ro, alpha, torch)
                slack = 64 * 2.0 ** -24 * (np.abs(p) + np.abs(po)) + 1e-12
                excess = np.abs(p - po) - bound * (1 + 1e-6) - slack
                assert excess.max() <= 0, (it, t, excess.max())
            if it == 1:
                # every block was factorized in the first snapshot
                for b in blocks:
                    A = s.block_dense(b).astype(np.float64)
                    Bg, sg = s.tree_factor(s.leaf_start + b)
                    omega = gaussian_matrix(kw["seed"], b, A.shape[1], d + 5)
                    Uo, So, _ = oracle_frpca(A, d, cfg["passes_q"], omega=omega)
                    So, Uo = So[::-1], Uo[:, ::-1]
                    # the subspace whose gap is also 1e-3 of sigma_1: the
                    # tensor-core products carry errors near 1e-5 of sigma_1,
                    # which a smaller gap turns into a larger rotation
                    # (sin-theta theorem)
                    j = gap_index(So, d, min_abs=1e-3)
                    assert j > 0
                    rel = np.abs(sg[:j] / So[:j] - 1).max()
                    assert rel < 1e-3, (b, rel)
                    assert max_principal_sine(Bg[:, :j], Uo[:, :j]) < 1e-2, b
