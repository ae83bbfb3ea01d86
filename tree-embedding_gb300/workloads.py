"""Seeded synthetic workloads standing in for the reference's datasets.

Each config follows one of the five workload descriptions of the build
(R-MAT (0.57, 0.19, 0.19, 0.05), self-loops and duplicates dropped, uniform
random timestamps split into a first snapshot plus equal deltas). The graphs
take their vertex and edge counts from the reference README's dataset table
(Patent, Wikipedia, YouTube/Flickr, Twitter); no dataset content is used.

This module does not load the library by itself: `build` draws the inputs
with the generator module it is given (the library's binding by default; the
CPU reference arm passes the oracle's own generator, which gives the same
bytes without the library).
"""
import numpy as np

# values of the TSVD_TRANSFORM_* and TSVD_DIRTY_* constants of include/tsvd.h
TRANSFORM_LOG10_NC, TRANSFORM_LOG10_LP, TRANSFORM_LN_N = 0, 1, 2
DIRTY_REFERENCE, DIRTY_FROBENIUS, DIRTY_ALL = 0, 1, 2
BLOCKS_DENSE, BLOCKS_SPARSE, BLOCKS_AUTO = 0, 1, 2

CONFIGS = {
    # Plain method, CPU-runnable (undirected, N=1e5, M=1e6, 10 snapshots).
    "rmat-u-100k": dict(n=100_000, m=1_000_000, directed=False, snapshots=10, first=0.5,
                        sources=500, alpha=0.2, rmax=1e-6, transform=TRANSFORM_LN_N,
                        n_parts=16, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=DIRTY_REFERENCE, delta=0.3),
    # Plain GPU form (directed, Patent-sized, 20 snapshots).
    "rmat-d-2.7m": dict(n=2_738_013, m=13_960_811, directed=True, snapshots=20, first=0.5,
                        sources=3000, alpha=0.2, rmax=1e-7, transform=TRANSFORM_LOG10_NC,
                        n_parts=64, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3),
    # Precision form (directed, Wikipedia-sized, 10 snapshots, first 70%).
    # Its PPR state (16 N Sp bytes = 305 GB) exceeds HBM: the reserve half
    # lives in pinned host memory.
    "rmat-d-6.2m": dict(n=6_216_199, m=177_862_656, directed=True, snapshots=10, first=0.7,
                        sources=3000, alpha=0.2, rmax=1e-7, transform=TRANSFORM_LOG10_NC,
                        n_parts=128, hierarchy_n=2, rank_d=128, passes_q=6,
                        dirty_rule=DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3,
                        host_reserve=True),
    # The same graph refreshed by 1%-insertion snapshots (1.78M edges each)
    # after a 70 % first snapshot: 30 deltas.
    # The push holds hubs (degree >= 1024) back until their residue reaches
    # 16 rmax, then 4 rmax, then finishes at rmax (measured on this graph:
    # snapshot p50 -3 % against two levels of ratio 8, which took -4.4 %
    # against none; the same levels for every vertex: +5.6 %).
    "rmat-d-6.2m-1pct": dict(n=6_216_199, m=177_862_656, directed=True, snapshots=31,
                             first=0.7, sources=3000, alpha=0.2, rmax=1e-7,
                             transform=TRANSFORM_LOG10_NC, n_parts=128, hierarchy_n=2,
                             rank_d=128, passes_q=6, dirty_rule=DIRTY_FROBENIUS,
                             dirty_frac=0.01, delta=0.3, host_reserve=True,
                             push_levels=3, push_ratio=4.0, push_hub_degree=1024),
    # Batched form: two undirected graphs (YouTube- and Flickr-sized), monthly
    # splits (24 snapshots, the first with 40 % of the edges), 256 column
    # blocks made deliberately uneven by numbering the vertices in descending
    # order of their final degree (block 0 holds the hubs); the block-path
    # autotuner picks tensor-core or SpMM products per block.
    "rmat-u-3.2m-deg": dict(n=3_223_589, m=9_375_374, directed=False, snapshots=24, first=0.4,
                            sources=3000, alpha=0.2, rmax=1e-7, transform=TRANSFORM_LOG10_NC,
                            n_parts=256, hierarchy_n=2, rank_d=128, passes_q=6,
                            dirty_rule=DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3,
                            degree_sort=True, block_path=BLOCKS_AUTO),
    "rmat-u-2.3m-deg": dict(n=2_302_925, m=33_140_017, directed=False, snapshots=24, first=0.4,
                            sources=3000, alpha=0.2, rmax=1e-7, transform=TRANSFORM_LOG10_NC,
                            n_parts=256, hierarchy_n=2, rank_d=128, passes_q=6,
                            dirty_rule=DIRTY_FROBENIUS, dirty_frac=0.01, delta=0.3,
                            degree_sort=True, block_path=BLOCKS_AUTO),
}


def degree_order(edges, n):
    """Vertex ids renumbered in descending order of final degree (both
    endpoints counted; ties keep the lower id first)."""
    deg = np.bincount(edges.ravel(), minlength=n)
    order = np.argsort(-deg, kind="stable")
    new_id = np.empty(n, np.int32)
    new_id[order] = np.arange(n, dtype=np.int32)
    return new_id[edges].astype(np.int32)


def scaled(name, n=None, m=None, sources=None, n_parts=None, rank_d=None, snapshots=None):
    c = dict(CONFIGS[name])
    c["name"] = name
    for k, v in dict(n=n, m=m, sources=sources, n_parts=n_parts, rank_d=rank_d,
                     snapshots=snapshots).items():
        if v is not None:
            c[k] = v
    return c


def build(cfg, seed=20231, generator=None):
    """Edges (in timestamp order), the snapshot deltas and the source subset.
    `generator` provides rmat_edges / snapshot_sizes / sample_sources (the
    library binding when None)."""
    if generator is None:
        import tsvd_gb300 as generator
    edges = generator.rmat_edges(cfg["n"], cfg["m"], directed=cfg["directed"], seed=seed)
    if cfg.get("degree_sort"):
        edges = degree_order(edges, cfg["n"])
    sizes = generator.snapshot_sizes(len(edges), cfg["snapshots"], cfg["first"])
    bounds = np.concatenate([[0], np.cumsum(sizes)])
    snaps = [edges[bounds[i]:bounds[i + 1]] for i in range(len(sizes))]
    sources = generator.sample_sources(cfg["n"], snaps[0], cfg["sources"], seed=seed)
    return edges, snaps, sources


def session_kwargs(cfg, dynamic_start=2, lazy_start=2, seed=20231):
    return dict(directed=cfg["directed"], alpha=cfg["alpha"], rmax=cfg["rmax"],
                n_parts=cfg["n_parts"], hierarchy_n=cfg["hierarchy_n"], rank_d=cfg["rank_d"],
                passes_q=cfg["passes_q"], dynamic_ppr_start_iter=dynamic_start,
                lazy_update_start_iter=lazy_start, delta=cfg.get("delta", 0.3),
                transform=cfg["transform"], dirty_rule=cfg["dirty_rule"],
                dirty_frac=cfg.get("dirty_frac", 0.01), block_path=cfg.get("block_path", 0),
                seed=seed, push_levels=cfg.get("push_levels", 1),
                push_ratio=cfg.get("push_ratio", 8.0),
                push_hub_degree=cfg.get("push_hub_degree", 0))
