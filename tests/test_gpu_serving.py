"""The serving layer (tsvd_server_*): tenants admitted by HBM footprint,
update and query requests taken as they arrive by several worker slots, so
different tenants' snapshots overlap on the device.

The check that matters for a server: every result is the same whether its
tenant ran alone or in the mix. Four tenants of different sizes and shapes
(directed and undirected, |S| and d different) are run once alone (one slot,
one tenant at a time) and once together (four slots, all requests submitted
up front, interleaved); after every update a query returns the embedding.
The two runs execute the same arithmetic except for the order of the push's
floating-point atomics: residues that land within rounding of rmax can be
pushed in one run and not in the other, so the two runs stop at two valid
push states, like any two runs of the same session. The results must then
agree within the tolerance every parity test states: root singular values
(the squared column norms of the U sqrt(S) embedding) within 1e-3 relative
plus 1e-4 of the largest (the Weyl floor of the two runs' push-order
difference) and the largest principal-angle sine of the gap-separated leading subspace
within 1e-2 (the subspace ends where the gap is at least 5 % of the next
singular value and 1e-2 of the largest: a difference of 1e-4 of the largest,
the floor of the singular-value check, can then turn it by at most 1e-2 by
the sin-theta theorem). Every block is refreshed every snapshot, so no lazy
decision can part the two runs.
"""
import numpy as np
import pytest

import tsvd_gb300 as T
import workloads as W
from helpers import gap_index, max_principal_sine

pytestmark = pytest.mark.gpu

TENANTS = [
    dict(base="rmat-u-100k", n=12000, m=80000, sources=96, n_parts=8, rank_d=32, seed=61),
    dict(base="rmat-d-2.7m", n=20000, m=120000, sources=160, n_parts=8, rank_d=64, seed=62),
    dict(base="rmat-u-100k", n=30000, m=150000, sources=200, n_parts=16, rank_d=32, seed=63),
    dict(base="rmat-d-2.7m", n=9000, m=50000, sources=64, n_parts=4, rank_d=32, seed=64),
]


def _tenant(spec):
    cfg = W.scaled(spec["base"], n=spec["n"], m=spec["m"], sources=spec["sources"],
                   n_parts=spec["n_parts"], rank_d=spec["rank_d"], snapshots=4)
    # the runs' push-order difference scales with rmax: at 1e-8 it stays far
    # below the tolerance, so any dependence on the mix would show
    cfg["rmax"] = 1e-8
    _, snaps, src = W.build(cfg, seed=spec["seed"])
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    kw["dirty_rule"] = T.DIRTY_ALL
    return cfg, snaps, src, kw


def _sigma_agree(sig, ref):
    """Every singular value within 1e-3 of itself plus 1e-4 of the largest:
    two runs' matrices differ by the order of the push's float reductions,
    and by Weyl's inequality that moves every singular value by the same
    absolute amount (measured near 4e-5 of the largest at rmax 1e-7), which
    is a large relative change only in the tail."""
    return bool((np.abs(sig - ref) <= 1e-3 * np.abs(ref) + 1e-4 * np.abs(ref).max()).all())


def _run(server, tenants, interleave):
    ids, reqs = [], []
    for cfg, snaps, src, kw in tenants:
        ids.append(server.add_tenant(cfg["n"], src, cfg["m"], **kw))
    nsnap = len(tenants[0][1])
    if interleave:
        order = [(k, t) for k in range(nsnap) for t in range(len(tenants))]
    else:
        order = [(k, t) for t in range(len(tenants)) for k in range(nsnap)]
    for k, t in order:
        u = server.submit_update(ids[t], tenants[t][1][k])
        q = server.submit_query(ids[t])
        reqs.append((t, k, u, q))
        if not interleave:
            server.wait(u)
    out = {}
    for t, k, u, q in reqs:
        lat, svc, _ = server.wait(u) if interleave else (0.0, 0.0, None)
        _, _, emb = server.wait(q)
        out[(t, k)] = emb
    sig = {t: server.session(ids[t]).tree_factor(0)[1] for t in range(len(tenants))}
    return out, sig, ids


def test_each_result_is_the_same_alone_and_in_the_mix():
    tenants = [_tenant(s) for s in TENANTS]
    with T.Server(slots=1) as alone_srv:
        alone, sig_alone, _ = _run(alone_srv, tenants, interleave=False)
    with T.Server(slots=4) as mix_srv:
        mixed, sig_mix, ids = _run(mix_srv, tenants, interleave=True)
        st = mix_srv.stats()
    assert st["updates"] == len(tenants) * 4 and st["tenants"] == len(tenants)
    assert st["p99_ms"] >= st["p50_ms"] > 0 and st["edges_per_s"] > 0
    for key, emb in alone.items():
        mix = mixed[key]
        assert np.isfinite(emb).all() and np.isfinite(mix).all()
        sa = (emb ** 2).sum(axis=0)  # U sqrt(S): column norms squared are S
        sm = (mix ** 2).sum(axis=0)
        order = np.argsort(-sa)
        sa, sm = sa[order], sm[np.argsort(-sm)]
        assert _sigma_agree(sm, sa), (key, np.abs(sm / sa - 1).max())
        j = gap_index(sa, len(sa), min_abs=1e-2)
        assert j > 0, key
        ua = emb[:, order[:j]]
        um = mix[:, np.argsort(-(mix ** 2).sum(axis=0))[:j]]
        assert max_principal_sine(um, ua) <= 1e-2, key
    for t in sig_alone:
        assert _sigma_agree(sig_mix[t], sig_alone[t]), t


def test_admission_by_hbm_footprint():
    cfg, snaps, src, kw = _tenant(TENANTS[0])
    need = T.footprint(cfg["n"], src, cfg["m"], **kw)
    with T.Server(hbm_budget_bytes=int(need * 1.5), slots=2) as srv:
        a = srv.add_tenant(cfg["n"], src, cfg["m"], **kw)
        with pytest.raises(T.TsvdError) as ei:  # a second one does not fit
            srv.add_tenant(cfg["n"], src, cfg["m"], **kw)
        assert ei.value.status == 2
        r = srv.submit_update(a, snaps[0])
        srv.wait(r)
        srv.remove_tenant(a)  # frees the budget
        b = srv.add_tenant(cfg["n"], src, cfg["m"], **kw)
        srv.wait(srv.submit_update(b, snaps[0]))
        assert srv.stats()["tenants"] == 1
