"""The node-classification evaluation (labelclassification_dynamic.py
restated): CPU checks of the metric and of the scipy fallback, and a GPU
check that the embedding of a planted-partition graph classifies its
communities."""
import builtins

import numpy as np
import pytest

import eval_nc as E


def _clusters(n=400, k=4, d=16, seed=0):
    rng = np.random.default_rng(seed)
    lab = rng.integers(0, k, n)
    centers = rng.standard_normal((k, d)) * 3
    X = centers[lab] + rng.standard_normal((n, d))
    return X, [[str(l)] for l in lab]


def test_f1_scores_known_values():
    yt = np.array([[1, 0], [0, 1], [1, 1]], bool)
    yp = np.array([[1, 0], [1, 0], [1, 1]], bool)
    r = E.f1_scores(yt, yp)
    # tp = (2, 1), fp = (1, 0), fn = (0, 1)
    assert r["micro"] == pytest.approx(2 * 3 / (2 * 3 + 1 + 1))
    assert r["macro"] == pytest.approx((4 / 5 + 2 / 3) / 2)


def test_separable_clusters_score_high_with_and_without_sklearn(monkeypatch):
    X, Y = _clusters()
    with_sk = E.split_train_evaluate(X, Y, 0.5)
    real_import = builtins.__import__

    def no_sklearn(name, *a, **k):
        if name.startswith("sklearn"):
            raise ImportError(name)
        return real_import(name, *a, **k)

    monkeypatch.setattr(builtins, "__import__", no_sklearn)
    fallback = E.split_train_evaluate(X, Y, 0.5)
    assert fallback["micro"] > 0.95
    assert abs(fallback["micro"] - with_sk["micro"]) < 0.03


@pytest.mark.gpu
def test_planted_partition_embedding_classifies_communities():
    import tsvd_gb300 as T
    rng = np.random.default_rng(11)
    n, k = 4000, 4
    comm = rng.integers(0, k, n)
    # planted partition: p_in = 0.01, p_out = 0.0005
    m = 60000
    u = rng.integers(0, n, m)
    same = rng.random(m) < 0.8
    v = np.where(same, -1, rng.integers(0, n, m))
    pools = [np.flatnonzero(comm == c) for c in range(k)]
    for i in np.flatnonzero(same):
        v[i] = rng.choice(pools[comm[u[i]]])
    e = np.stack([u, v], 1)
    e = e[e[:, 0] != e[:, 1]].astype(np.int32)
    rng.shuffle(e)
    snaps = [e[: len(e) // 2], e[len(e) // 2:]]
    deg = np.bincount(snaps[0].ravel(), minlength=n)
    src = np.sort(rng.choice(np.flatnonzero(deg > 0), 400, replace=False)).astype(np.int32)
    with T.Session(n, src, alpha=0.2, rmax=1e-5, n_parts=4, hierarchy_n=2, rank_d=64,
                   passes_q=6, dynamic_ppr_start_iter=2, lazy_update_start_iter=2) as s:
        for sn in snaps:
            s.step(sn)
        emb = s.embedding()
    Y = [[str(comm[v])] for v in src]
    res = E.split_train_evaluate(emb, Y, 0.5)
    assert res["micro"] > 0.8, res
