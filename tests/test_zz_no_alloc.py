"""tsvd_frpca_noalloc — the frPCA entry point that allocates nothing.

Callers that cannot allocate device memory (plug-ins inside an application
that reserves the GPU's memory pool for its own allocator, host loops that
must stay off the allocator) use tsvd_frpca_noalloc instead of tsvd_frpca.
It keeps its scratch in one static device array and its host staging in
static arrays, so it has size limits. This file checks, through the C-ABI,
that two calls in a row (a larger matrix, then a smaller one, so the second
runs on the first one's leftovers in the shared array) agree with the
allocating entry point to the tolerance of the frPCA tests, at exactly the
documented limits and on an all-zero matrix too, that free device memory is
unchanged across repeated calls, and that inputs beyond the limits are
rejected.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import tsvd_gb300 as T

pytestmark = pytest.mark.gpu


def _lowrank_csr(m, n, rank, density, seed):
    rng = np.random.default_rng(seed)
    D = (rng.standard_normal((m, rank)) * 0.96 ** np.arange(rank)) @ rng.standard_normal((rank, n))
    D = np.where(rng.random((m, n)) < density, np.abs(D), 0.0)
    D[:, rng.choice(n, n // 5, replace=False)] = 0.0  # empty columns are compacted away
    return sp.csr_matrix(D)


def _check_same(a, b, k):
    U, S, V = a
    U2, S2, V2 = b
    assert np.allclose(S2, S, rtol=1e-3, atol=1e-6 * S[0])
    R = (U * S) @ V.T
    R2 = (U2 * S2) @ V2.T
    assert np.linalg.norm(R2 - R) <= 1e-3 * np.linalg.norm(R)
    G = U @ U.T
    G2 = U2 @ U2.T
    assert np.linalg.norm(G2 - G) <= 1e-2 * np.linalg.norm(G)


def test_noalloc_matches_allocating_entry_point_twice_in_a_row():
    cases = [(500, 2500, 48, 6, 11, 0.2), (160, 1200, 24, 4, 12, 0.3)]
    for m, n, k, q, seed, dens in cases:
        A = _lowrank_csr(m, n, 96, dens, seed)
        assert A.nnz <= 262144
        ref = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=seed)
        got = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=seed, noalloc=True)
        _check_same(ref, got, k)
    # 1-based input is accepted too
    A = _lowrank_csr(100, 900, 40, 0.3, 13)
    ref = T.frpca(A.indptr, A.indices, A.data, A.shape, 16, 4, seed=3)
    got = T.frpca(A.indptr + 1, A.indices + 1, A.data, A.shape, 16, 4, seed=3, index_base=1,
                  noalloc=True)
    _check_same(ref, got, 16)


def test_noalloc_rejects_inputs_beyond_its_limits():
    A = _lowrank_csr(600, 1000, 8, 0.05, 1)  # 600 rows > 512
    with pytest.raises(T.TsvdError) as ei:
        T.frpca(A.indptr, A.indices, A.data, A.shape, 16, 4, noalloc=True)
    assert ei.value.status == 1
    A = _lowrank_csr(100, 5000, 8, 0.2, 2)  # ~4000 non-empty columns > 2048
    with pytest.raises(T.TsvdError):
        T.frpca(A.indptr, A.indices, A.data, A.shape, 16, 4, noalloc=True)
    A = _lowrank_csr(100, 900, 40, 0.3, 3)
    with pytest.raises(T.TsvdError):
        T.frpca(A.indptr, A.indices, A.data, A.shape, 65, 4, noalloc=True)  # k > 64


def test_noalloc_at_the_limits_and_on_an_all_zero_matrix():
    # exactly nrows = 512, 2048 non-empty columns and k = 64
    rng = np.random.default_rng(21)
    m, n, k = 512, 3000, 64
    D = (rng.standard_normal((m, 96)) * 0.95 ** np.arange(96)) @ rng.standard_normal((96, 2048))
    D = np.where(rng.random(D.shape) < 0.2, np.abs(D), 0.0)
    D[0, :] = 1.0 + np.abs(D[0, :])  # every one of the 2048 columns non-empty
    full = np.zeros((m, n))
    full[:, np.sort(rng.choice(n, 2048, replace=False))] = D
    A = sp.csr_matrix(full)
    assert A.nnz <= 262144 and np.count_nonzero(A.getnnz(axis=0)) == 2048
    ref = T.frpca(A.indptr, A.indices, A.data, A.shape, k, 4, seed=5)
    got = T.frpca(A.indptr, A.indices, A.data, A.shape, k, 4, seed=5, noalloc=True)
    _check_same(ref, got, k)
    # no non-zero at all (explicit zeros only): the kernels are skipped and
    # both entry points return zero factors
    Z = sp.csr_matrix((np.zeros(40), np.arange(40) * 7 % 200, np.arange(0, 41, 4)[:11]),
                      shape=(10, 200))
    assert Z.nnz == 40 and not Z.data.any()
    for noalloc in (False, True):
        U, S, V = T.frpca(Z.indptr, Z.indices, Z.data, Z.shape, 8, 2, seed=1, noalloc=noalloc)
        assert not U.any() and not S.any() and not V.any()


def test_noalloc_leaves_free_device_memory_unchanged():
    torch = pytest.importorskip("torch")
    A = _lowrank_csr(300, 1500, 48, 0.25, 31)
    T.frpca(A.indptr, A.indices, A.data, A.shape, 32, 4, seed=2, noalloc=True)  # set-up call
    torch.cuda.mem_get_info()  # torch's own context set-up happens here, not below
    free0, _ = torch.cuda.mem_get_info()
    out = [T.frpca(A.indptr, A.indices, A.data, A.shape, 32, 4, seed=2, noalloc=True)
           for _ in range(2)]
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert np.array_equal(out[0][1], out[1][1])
