"""The oracle's own workload generator (oracle/oracle_synth.c) against the
product's (tsvd_rmat_edges, tsvd_snapshot_sizes, tsvd_sample_sources): the
CPU reference arm of bench.py builds its inputs with the oracle's, so that it
never loads the product library; both must give the same bytes."""
import numpy as np
import pytest

import tsvd_gb300 as T
from oracle import native


@pytest.mark.parametrize("n,m,directed,seed", [
    (5000, 40000, True, 3),
    (3000, 20000, False, 11),
    (100_000, 1_000_000, False, 20231),   # the N = 1e5, M = 1e6 undirected configuration
])
def test_oracle_rmat_is_bit_identical_to_the_product(n, m, directed, seed):
    a = T.rmat_edges(n, m, directed=directed, seed=seed)
    b = native.rmat_edges(n, m, directed=directed, seed=seed, threads=4)
    assert a.dtype == b.dtype == np.int32
    assert np.array_equal(a, b)


def test_oracle_snapshot_split_and_sources_match_the_product():
    for m, count, first in [(1_000_000, 10, 0.5), (13_960_811, 20, 0.5), (177_862_656, 31, 0.7),
                            (17, 4, 0.3)]:
        assert list(T.snapshot_sizes(m, count, first)) == native.snapshot_sizes(m, count, first)
    e = T.rmat_edges(20000, 150000, directed=True, seed=5)
    assert np.array_equal(T.sample_sources(20000, e[:70000], 300, seed=9),
                          native.sample_sources(20000, e[:70000], 300, seed=9))
