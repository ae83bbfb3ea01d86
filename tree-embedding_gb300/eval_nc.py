"""Node-classification quality of the embeddings: micro / macro F1 of a
one-vs-rest logistic regression that predicts, for every test node, its k
highest-scored labels (k = the node's number of true labels).

Restates Code/labelclassification_dynamic.py:1-131: per snapshot block of
|S| rows of the embedding file, for every train ratio, shuffle the labelled
nodes with seed 0, train on the first ratio * |S|, evaluate on the rest.
scikit-learn's OneVsRestClassifier(LogisticRegression()) is used when it is
installed; otherwise an equivalent L2-regularised (C = 1) binary logistic
regression per label is fitted with scipy's L-BFGS.

    python eval_nc.py EMBEDDINGS(.csv|.npy) LABELS [--ratios 0.1,0.3,...]

LABELS has one line per embedding row: "vertex label [label ...]".
"""
import argparse
import sys

import numpy as np


def load_embeddings(path):
    if path.endswith(".npy"):
        return np.load(path)
    return np.loadtxt(path, delimiter=",")


def read_node_label(path):
    X, Y = [], []
    with open(path) as f:
        for line in f:
            v = line.strip().split()
            if not v:
                continue
            X.append(int(v[0]))
            Y.append(v[1:])
    return X, Y


def _fit_binary(Xtr, y, C=1.0):
    """min  0.5 ||w||^2 + C sum log(1 + exp(-s_i (x_i w + b)))  (bias not
    penalised), the objective of LogisticRegression(penalty='l2', C=1)."""
    from scipy.optimize import minimize
    s = np.where(y > 0, 1.0, -1.0)
    Xb = np.hstack([Xtr, np.ones((Xtr.shape[0], 1))])

    def f(wb):
        z = s * (Xb @ wb)
        loss = C * np.sum(np.logaddexp(0.0, -z)) + 0.5 * wb[:-1] @ wb[:-1]
        g = -C * (Xb.T @ (s / (1.0 + np.exp(z))))
        g[:-1] += wb[:-1]
        return loss, g

    res = minimize(f, np.zeros(Xb.shape[1]), jac=True, method="L-BFGS-B",
                   options={"maxiter": 100})
    return res.x


class _OneVsRest:
    def fit(self, X, Y):
        try:
            from sklearn.linear_model import LogisticRegression
            from sklearn.multiclass import OneVsRestClassifier
            self.sk = OneVsRestClassifier(LogisticRegression()).fit(X, Y)
        except ImportError:
            self.sk = None
            self.W = np.stack([_fit_binary(X, Y[:, j]) for j in range(Y.shape[1])], 1)
        return self

    def scores(self, X):
        if self.sk is not None:
            return np.asarray(self.sk.predict_proba(X))
        return np.hstack([X, np.ones((X.shape[0], 1))]) @ self.W


def f1_scores(Ytrue, Ypred):
    tp = (Ytrue & Ypred).sum(0).astype(np.float64)
    fp = (~Ytrue & Ypred).sum(0).astype(np.float64)
    fn = (Ytrue & ~Ypred).sum(0).astype(np.float64)
    micro = 2 * tp.sum() / max(2 * tp.sum() + fp.sum() + fn.sum(), 1e-300)
    denom = 2 * tp + fp + fn
    per = np.where(denom > 0, 2 * tp / np.where(denom > 0, denom, 1), 0.0)
    return {"micro": float(micro), "macro": float(per.mean())}


def split_train_evaluate(emb, Y, train_percent, seed=0):
    classes = sorted({l for ls in Y for l in ls})
    idx = {c: i for i, c in enumerate(classes)}
    B = np.zeros((len(Y), len(classes)), bool)
    for r, ls in enumerate(Y):
        for l in ls:
            B[r, idx[l]] = True
    state = np.random.get_state()
    np.random.seed(seed)
    perm = np.random.permutation(np.arange(len(Y)))
    np.random.set_state(state)
    ntr = int(train_percent * len(Y))
    tr, te = perm[:ntr], perm[ntr:]
    clf = _OneVsRest().fit(emb[tr], B[tr].astype(int))
    sc = clf.scores(emb[te])
    pred = np.zeros_like(B[te])
    for i, r in enumerate(te):
        k = int(B[r].sum())
        pred[i, np.argsort(sc[i])[len(classes) - k:]] = True
    return f1_scores(B[te], pred)


def evaluate(emb_all, Y, ratios=(0.1, 0.3, 0.5, 0.7, 0.9)):
    base = len(Y)
    out = []
    for i in range(emb_all.shape[0] // base):
        blk = emb_all[i * base:(i + 1) * base]
        out.append({r: split_train_evaluate(blk, Y, r) for r in ratios})
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("embeddings")
    ap.add_argument("labels")
    ap.add_argument("--ratios", default="0.1,0.3,0.5,0.7,0.9")
    a = ap.parse_args(argv)
    emb = load_embeddings(a.embeddings)
    _, Y = read_node_label(a.labels)
    ratios = [float(x) for x in a.ratios.split(",")]
    for i, res in enumerate(evaluate(emb, Y, ratios)):
        print("In the", i, "Round:")
        for r in ratios:
            print("Training classifier using {:.2f}% nodes... {}".format(r * 100, res[r]))


if __name__ == "__main__":
    sys.exit(main())
