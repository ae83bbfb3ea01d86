"""The reference-compatible frPCA symbol, called from C the way the
reference's drivers call it (Code/Tree_u_NC.cpp:139-145 over
Code/frpca.c:239-326): 1-based mat_csr with pointerB/pointerE, caller-
preallocated U, S, V, ascending singular values. Checked against the
status-returning tsvd_frpca on the same seed and against the reference's own
frpca.c output (tests/golden/ref_frpca_q6.npz)."""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import tsvd_gb300 as T
from helpers import gap_index, max_principal_sine

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "tree-embedding_gb300")


@pytest.fixture(scope="module")
def legacy_exe(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("legacy") / "frpca_legacy_check")
    subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(HERE, "native", "frpca_legacy_check.c"), "-o", exe,
                           "-L" + PKG, "-ltsvd_gb300", "-Wl,-rpath," + PKG, "-lm"])
    return exe


def _run(exe, tmp, A, k, q, seed):
    m, n = A.shape
    A = sp.csr_matrix(A)
    inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    with open(inp, "wb") as f:
        np.array([m, n, A.nnz, k, q], np.int32).tofile(f)
        np.array([seed], np.uint64).tofile(f)
        (A.indptr[:-1] + 1).astype(np.int32).tofile(f)   # pointerB, 1-based
        (A.indptr[1:] + 1).astype(np.int32).tofile(f)    # pointerE, 1-based
        (A.indices + 1).astype(np.int32).tofile(f)
        A.data.astype(np.float64).tofile(f)
    subprocess.check_call([exe, inp, out])
    raw = np.fromfile(out, np.uint8)
    vals = raw[:-4].view(np.float64)
    unset = int(raw[-4:].view(np.int32)[0])
    U = vals[:m * k].reshape(k, m).T
    S = vals[m * k:m * k + k]
    V = vals[m * k + k:].reshape(k, n).T
    return U, S, V, unset


def test_legacy_frpca_symbol_from_c_matches_tsvd_frpca(legacy_exe, tmp_path):
    rng = np.random.default_rng(8)
    m, n, k, q = 400, 3000, 32, 6
    D = (rng.standard_normal((m, 80)) * 0.93 ** np.arange(80)) @ rng.standard_normal((80, n))
    D = np.where(rng.random((m, n)) < 0.25, np.abs(D), 0.0)
    A = sp.csr_matrix(D)
    U, S, V, unset = _run(legacy_exe, str(tmp_path), A, k, q, seed=19)
    assert unset == 0
    assert np.all(np.diff(S) >= 0), "frPCA hands singular values back ascending"
    Ud, Sd, Vd = T.frpca(A.indptr, A.indices, A.data, A.shape, k, q, seed=19)
    assert np.allclose(S[::-1], Sd, rtol=1e-3, atol=1e-6 * Sd[0])
    j = gap_index(Sd, k)
    assert j > 0
    assert max_principal_sine(U[:, ::-1][:, :j], Ud[:, :j]) < 1e-2
    assert max_principal_sine(V[:, ::-1][:, :j], Vd[:, :j]) < 1e-2
    assert np.abs(U.T @ U - np.eye(k)).max() < 1e-3


def test_legacy_frpca_symbol_from_c_matches_the_reference_golden(legacy_exe, tmp_path):
    z = np.load(os.path.join(HERE, "golden", "ref_frpca_q6.npz"))
    A = sp.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
    k, q = int(z["k"]), int(z["q"])
    U, S, V, unset = _run(legacy_exe, str(tmp_path), A, k, q, seed=5)
    assert unset == 0
    assert np.all(np.diff(S) >= 0)
    # both in the reference's ascending order
    Sr, Ur, Vr = z["S"], z["U"], z["V"]
    j = gap_index(Sr[::-1], k)
    assert j > 0
    assert np.allclose(S[::-1][:j], Sr[::-1][:j], rtol=1e-3)
    assert max_principal_sine(U[:, ::-1][:, :j], Ur[:, ::-1][:, :j]) < 1e-2
    assert max_principal_sine(V[:, ::-1][:, :j], Vr[:, ::-1][:, :j]) < 1e-2
