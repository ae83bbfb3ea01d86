"""Shared checks for the parity tests (CPU-side arithmetic only)."""
import numpy as np
import scipy.linalg
import scipy.sparse as sp


def transition(n, off, nbr):
    """Row-stochastic P = D^-1 A from insertion-ordered adjacency (dangling rows 0)."""
    deg = np.diff(off)
    rows = np.repeat(np.arange(n), deg)
    A = sp.csr_matrix((np.ones(len(nbr)), (rows, nbr)), shape=(n, n))
    dinv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    return sp.diags(dinv) @ A, deg


def push_identity_residual(p, r, sources, P, alpha):
    """max |p (I - (1-alpha) P) - alpha (e_s - r)| over all entries: zero for any
    exact forward-push state, whatever the push order."""
    p = p.astype(np.float64)
    r = r.astype(np.float64)
    lhs = p - (1 - alpha) * (P.T @ p.T).T
    rhs = -alpha * r
    rhs[np.arange(len(sources)), sources] += alpha
    return np.abs(lhs - rhs).max()


def reach_weight(P, alpha, iters=400):
    """c(t) = sum_v pi_v(t) = alpha (1^T (I - (1-alpha) P)^-1)(t): solves
    y = 1 + (1-alpha) P^T y and returns alpha y. A forward-push state with every
    eligible residue <= rmax has |p_s(t) - pi_s(t)| <= rmax c(t)."""
    n = P.shape[0]
    PT = P.T.tocsr()
    y = np.ones(n)
    for _ in range(iters):
        y = 1.0 + (1 - alpha) * (PT @ y)
    return alpha * y


def residual_error_bound(r, P, alpha, iters=400):
    """|p_s - pi_s| <= (alpha |r_s| (I - (1-alpha) P)^-1) entrywise, for any
    state satisfying the push identity (the dynamic refresh can leave negative
    residues, so rmax alone does not bound the error). Solved by the fixed
    point x = alpha |r| + (1-alpha) x P, one row per source."""
    a = np.abs(r.astype(np.float64))
    x = alpha * a
    PT = P.T.tocsr()
    for _ in range(iters):
        x = alpha * a + (1 - alpha) * (PT @ x.T).T
    return x


def max_principal_sine(A, B):
    """Largest principal-angle sine between the column spaces of A and B."""
    qa = scipy.linalg.orth(A)
    qb = scipy.linalg.orth(B)
    s = scipy.linalg.svdvals(qa.T @ qb)
    s = np.clip(s, 0, 1)
    return float(np.sqrt(max(0.0, 1 - s.min() ** 2))) if len(s) else 0.0


def gap_index(sig, k, min_gap=1.05, min_abs=0.0):
    """Largest j <= k whose singular value is separated from the next by the
    ratio min_gap and by at least min_abs * sig[0]."""
    for j in range(k, 0, -1):
        if (j < len(sig) and sig[j] > 0 and sig[j - 1] / sig[j] >= min_gap and
                sig[j - 1] - sig[j] >= min_abs * sig[0]):
            return j
    return 0


def spectral_norm(D):
    """||D||_2 of a wide matrix through its small Gram D D^T."""
    G = D @ D.T
    return float(np.sqrt(max(np.linalg.eigvalsh(G).max(), 0.0)))


def gram_rel_err(B, B_ref):
    """||B B^T - R R^T||_F / ||R R^T||_F: rotation- and sign-invariant."""
    G = B @ B.T
    Gr = B_ref @ B_ref.T
    return float(np.linalg.norm(G - Gr) / max(np.linalg.norm(Gr), 1e-300))
