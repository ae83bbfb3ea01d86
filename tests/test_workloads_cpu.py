"""Host-side checks of the workload definitions (no GPU): every configuration's
session keywords build a tsvd_config the library accepts, the oracle's tree
accepts the same keywords (the parity tests hand it the session's), and the
push schedule a configuration names reaches the config struct."""
import numpy as np
import pytest

import tsvd_gb300 as T
import workloads as W
from oracle.tree_oracle import OracleTreeSVD


@pytest.mark.parametrize("name", sorted(W.CONFIGS))
def test_session_keywords_build_a_config_and_an_oracle(name):
    cfg = W.scaled(name, n=2000, m=10000, sources=64, n_parts=4, rank_d=16)
    kw = W.session_kwargs(cfg, dynamic_start=2, lazy_start=2)
    src = np.arange(64, dtype=np.int32)
    c = T.make_config(cfg["n"], src, **kw)
    assert c.push_levels == cfg.get("push_levels", 1)
    assert c.push_hub_degree == cfg.get("push_hub_degree", 0)
    assert c.block_path == cfg.get("block_path", 0)
    assert T.footprint(cfg["n"], src, cfg["m"], **kw) > 0
    okw = dict(kw)
    okw.pop("seed")
    OracleTreeSVD(cfg["n"], src, seed=kw["seed"], **okw)  # must not reject a keyword


def test_latency_workload_runs_the_hub_schedule():
    cfg = W.scaled("rmat-d-6.2m-1pct")
    kw = W.session_kwargs(cfg)
    assert kw["push_levels"] > 1 and kw["push_hub_degree"] > 0
    assert cfg["snapshots"] == 31 and cfg["first"] == 0.7  # 30 deltas of 1 %
