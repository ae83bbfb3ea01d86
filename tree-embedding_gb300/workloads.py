"""Seeded synthetic workloads standing in for the reference's datasets.

Each config follows one of the five workload descriptions of the build
(R-MAT (0.57, 0.19, 0.19, 0.05), self-loops and duplicates dropped, uniform
random timestamps split into a first snapshot plus equal deltas). The graphs
take their vertex and edge counts from the reference README's dataset table
(Patent, Wikipedia, YouTube/Flickr, Twitter); no dataset content is used.
"""
import numpy as np

import tsvd_gb300 as T

CONFIGS = {
    # Plain method, CPU-runnable (undirected, N=1e5, M=1e6, 10 snapshots).
    "rmat-u-100k": dict(n=100_000, m=1_000_000, directed=False, snapshots=10, first=0.5,
                        sources=500, alpha=0.2, rmax=1e-6, transform=T.TRANSFORM_LN_N,
                        n_parts=16, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=T.DIRTY_REFERENCE, delta=0.3),
    # Plain GPU form (directed, Patent-sized, 20 snapshots).
    "rmat-d-2.7m": dict(n=2_738_013, m=13_960_811, directed=True, snapshots=20, first=0.5,
                        sources=3000, alpha=0.2, rmax=1e-7, transform=T.TRANSFORM_LOG10_NC,
                        n_parts=64, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=T.DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3),
    # Precision form (directed, Wikipedia-sized, 10 snapshots, first 70%).
    "rmat-d-6.2m": dict(n=6_216_199, m=177_862_656, directed=True, snapshots=10, first=0.7,
                        sources=3000, alpha=0.2, rmax=1e-7, transform=T.TRANSFORM_LOG10_NC,
                        n_parts=128, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=T.DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3),
}


def scaled(name, n=None, m=None, sources=None, n_parts=None, rank_d=None, snapshots=None):
    c = dict(CONFIGS[name])
    for k, v in dict(n=n, m=m, sources=sources, n_parts=n_parts, rank_d=rank_d,
                     snapshots=snapshots).items():
        if v is not None:
            c[k] = v
    return c


def build(cfg, seed=20231):
    """Edges (in timestamp order), the snapshot deltas and the source subset."""
    edges = T.rmat_edges(cfg["n"], cfg["m"], directed=cfg["directed"], seed=seed)
    sizes = T.snapshot_sizes(len(edges), cfg["snapshots"], cfg["first"])
    bounds = np.concatenate([[0], np.cumsum(sizes)])
    snaps = [edges[bounds[i]:bounds[i + 1]] for i in range(len(sizes))]
    sources = T.sample_sources(cfg["n"], snaps[0], cfg["sources"], seed=seed)
    return edges, snaps, sources


def session_kwargs(cfg, dynamic_start=2, lazy_start=2, seed=20231):
    return dict(directed=cfg["directed"], alpha=cfg["alpha"], rmax=cfg["rmax"],
                n_parts=cfg["n_parts"], hierarchy_n=cfg["hierarchy_n"], rank_d=cfg["rank_d"],
                passes_q=cfg["passes_q"], dynamic_ppr_start_iter=dynamic_start,
                lazy_update_start_iter=lazy_start, delta=cfg.get("delta", 0.3),
                transform=cfg["transform"], dirty_rule=cfg["dirty_rule"],
                dirty_frac=cfg.get("dirty_frac", 0.01), seed=seed)
