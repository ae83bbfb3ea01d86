"""CPU checks of the C-ABI library: it loads without a GPU and exports every
function include/tsvd.h declares; host-side generators behave as specified."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import tsvd_gb300 as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "tsvd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", src, flags=re.M):
        name = m.group(1)
        if name not in ("if", "defined"):
            names.add(name)
    return names


def test_library_exports_every_declared_symbol():
    decl = declared_functions()
    assert "tsvd_session_step" in decl and "frPCA" in decl
    out = subprocess.run(["nm", "-D", "--defined-only", T.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(decl - exported)
    assert not missing, missing
    # and the binding covers them all
    assert not (decl - set(T.EXPORTS)), sorted(decl - set(T.EXPORTS))


def test_status_strings_and_version():
    L = T.lib()
    assert L.tsvd_status_string(0) == b"ok"
    assert L.tsvd_status_string(4) == b"timeout"
    assert b"sm_103a" in L.tsvd_version()


@pytest.mark.parametrize("directed", [False, True])
def test_rmat_edges_properties(directed):
    n, m = 5000, 30000
    e = T.rmat_edges(n, m, directed=directed, seed=3)
    assert e.shape == (m, 2) and e.min() >= 0 and e.max() < n
    assert (e[:, 0] != e[:, 1]).all()
    key = np.sort(e, axis=1) if not directed else e
    assert len(np.unique(key, axis=0)) == m
    e2 = T.rmat_edges(n, m, directed=directed, seed=3)
    assert np.array_equal(e, e2)
    e3 = T.rmat_edges(n, m, directed=directed, seed=4)
    assert not np.array_equal(e, e3)
    # R-MAT skew: the top 1% of vertices carry a large share of the endpoints
    deg = np.bincount(e.ravel(), minlength=n)
    top = np.sort(deg)[::-1][: n // 100].sum()
    assert top > 0.1 * deg.sum()


def test_rmat_rejects_bad_arguments():
    with pytest.raises(T.TsvdError):
        T.rmat_edges(1, 10)
    with pytest.raises(T.TsvdError):
        T.rmat_edges(10, 1000)  # more than half of all pairs


def test_snapshot_sizes():
    s = T.snapshot_sizes(1_000_000, 10, 0.5)
    assert s.sum() == 1_000_000 and s[0] == 500_000
    assert s[1:].max() - s[1:].min() <= 1
    s = T.snapshot_sizes(13_960_811, 20, 0.5)
    assert s.sum() == 13_960_811 and len(s) == 20
    assert np.array_equal(T.snapshot_sizes(7, 1, 0.5), [7])


def test_sample_sources_sorted_distinct_from_first_snapshot():
    e = T.rmat_edges(3000, 12000, seed=1)
    src = T.sample_sources(3000, e[:6000], 200, seed=5)
    assert len(np.unique(src)) == 200 and np.all(np.diff(src) > 0)
    touched = np.unique(e[:6000])
    assert np.isin(src, touched).all()
    assert np.array_equal(src, T.sample_sources(3000, e[:6000], 200, seed=5))


def test_edge_file_reader_matches_reference_reader_semantics():
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "e.txt")
        with open(p, "w") as f:
            f.write("1 2\n3 4\n")
        assert T.read_edge_file(p).tolist() == [[1, 2], [3, 4]]
        # the reference loop repeats the last pair when whitespace follows it
        assert T.read_edge_file(p, compat_dup_last=True).tolist() == [[1, 2], [3, 4], [3, 4]]
        with open(p, "w") as f:
            f.write("1 2\n3 4")
        assert T.read_edge_file(p, compat_dup_last=True).tolist() == [[1, 2], [3, 4]]
        with open(p, "w") as f:
            f.write("1 2\n3\n")
        with pytest.raises(T.TsvdError):
            T.read_edge_file(p)
        with pytest.raises(T.TsvdError):
            T.read_edge_file(os.path.join(d, "missing.txt"))


def test_gaussian_is_standard_normal_and_matches_oracle():
    from oracle.tree_oracle import gaussian_matrix
    import scipy.stats as st
    g = gaussian_matrix(20231, 5, 2000, 133)
    assert abs(g.mean()) < 0.01 and abs(g.std() - 1) < 0.01
    assert st.kstest(g.ravel(), "norm").pvalue > 1e-3
    # half-precision values (the precision of the tensor-core operand)
    assert np.array_equal(g, g.astype(np.float16).astype(np.float64))
    for (r, c) in [(0, 0), (0, 1), (17, 132), (1999, 64)]:
        assert T.gaussian(20231, 5, r, c) == g[r, c]


def test_lp_precision_matches_oracle_including_ties():
    from oracle.tree_oracle import lp_precision
    rng = np.random.default_rng(3)
    for m, k in [(10, 3), (1000, 100), (257, 257)]:
        scores = np.round(rng.standard_normal(m), 1)  # many ties
        pos = (rng.random(m) < 0.3).astype(np.uint8)
        assert T.lp_precision(scores, pos, k) == pytest.approx(lp_precision(scores, pos, k))
    with pytest.raises(T.TsvdError):
        T.lp_precision(np.zeros(3), np.zeros(3, np.uint8), 4)
    with pytest.raises(T.TsvdError):
        T.lp_precision(np.zeros(3), np.zeros(3, np.uint8), 0)


def test_binary_edge_file_round_trip(tmp_path):
    e = np.random.default_rng(1).integers(0, 1 << 30, (1000, 2)).astype(np.int32)
    p = str(tmp_path / "delta.bin")
    T.write_edge_file_binary(p, e)
    assert np.array_equal(T.read_edge_file(p), e)
    (tmp_path / "bad.bin").write_bytes(b"\x00" * 12)  # not whole pairs
    with pytest.raises(T.TsvdError):
        T.read_edge_file(str(tmp_path / "bad.bin"))


def test_cli_split_matches_reference_batch_splitter(tmp_path):
    """tree_svd split: Code/split_edges_NC.cpp semantics (keep the first
    round_index config lines, re-cut the following edges into batches)."""
    cli = os.path.join(os.path.dirname(os.path.abspath(T.__file__)), "tree_svd")
    d = tmp_path / "DY_Dataset" / "q"
    d.mkdir(parents=True)
    rng = np.random.default_rng(2)
    files = [str(d / "subset.txt")]
    (d / "subset.txt").write_text("1\n2\n")
    snaps = [rng.integers(0, 500, (n, 2)) for n in (300, 170, 260)]
    for k, e in enumerate(snaps):
        files.append(str(d / ("s%d.txt" % k)))
        np.savetxt(files[-1], e, fmt="%d %d")
    (d / "config.txt").write_text("\n".join(files) + "\n")
    r = subprocess.run([cli, "split", "nc", "q", "2", "--batch", "100", "--count", "3"],
                       cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "DY_Dataset" / "q_batch" / "config.txt").read_text().split()
    assert lines[:2] == files[:2]
    assert len(lines) == 5
    rest = np.concatenate(snaps[1:])
    for k, path in enumerate(lines[2:]):
        assert path.endswith("q_batch-Train-2-%d.txt" % (k + 1))
        got = np.loadtxt(tmp_path / path, dtype=np.int64).reshape(-1, 2)
        assert np.array_equal(got, rest[100 * k:100 * (k + 1)])
