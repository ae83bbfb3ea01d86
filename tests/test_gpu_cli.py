"""The tree_svd CLI (drop-in for the reference drivers' 12-argument main) on a
tiny dataset laid out like the reference's DY_Dataset / DY_LP_Dataset."""
import os
import subprocess

import numpy as np
import pytest

import tsvd_gb300 as T
import workloads as W
from helpers import gram_rel_err

pytestmark = pytest.mark.gpu

CLI = os.path.join(os.path.dirname(os.path.abspath(T.__file__)), "tree_svd")


def _dataset(root, sub, name, snaps, src, extra=None):
    d = os.path.join(root, sub, name)
    os.makedirs(d)
    files = [os.path.join(d, "subset.txt")]
    np.savetxt(files[0], np.asarray(src), fmt="%d")
    for k, e in enumerate(snaps):
        files.append(os.path.join(d, "snap%d.txt" % k))
        np.savetxt(files[-1], e, fmt="%d %d")
    with open(os.path.join(d, "config.txt"), "w") as f:
        f.write("\n".join(files) + "\n")
    for fname, pairs in (extra or {}).items():
        np.savetxt(os.path.join(d, fname), pairs, fmt="%d %d")


def _cfg():
    c = W.scaled("rmat-u-100k", n=6000, m=40000, sources=160, n_parts=4, rank_d=128,
                 snapshots=3)
    c["rmax"] = 1e-5
    return c


def test_cli_nc_writes_the_reference_csv(tmp_path):
    cfg = _cfg()
    _, snaps, src = W.build(cfg, seed=41)
    _dataset(str(tmp_path), "DY_Dataset", "tiny", snaps, src)
    os.makedirs(tmp_path / "EB")
    args = [CLI, "u_nc", "tiny", "EB/", "0.2", "6", "0.00001", "1", "4", "2", str(cfg["n"]),
            "2", "2", "0.3"]
    r = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    outs = list((tmp_path / "EB").glob("tiny0.300000_*_4_2_De_svd_u_Dppr_parallel_bound_nodegree_U.csv"))
    assert len(outs) == 1
    emb = np.loadtxt(outs[0], delimiter=",")
    assert emb.shape == ((len(snaps)) * len(src), 128)
    with T.Session(cfg["n"], src, alpha=0.2, rmax=1e-5, n_parts=4, hierarchy_n=2, passes_q=6,
                   dynamic_ppr_start_iter=2, lazy_update_start_iter=2, delta=0.3) as s:
        for k, e in enumerate(snaps):
            s.step(e)
            # two GPU runs differ by the order of the push's atomic adds (PPR
            # equal within the rmax bound), which moves the embedding's tail
            got = emb[k * len(src):(k + 1) * len(src)]
            ref = s.embedding()
            sg = np.linalg.svd(got, compute_uv=False)[:16]
            sr = np.linalg.svd(ref, compute_uv=False)[:16]
            assert np.allclose(sg, sr, rtol=5e-3)
            assert gram_rel_err(got, ref) < 3e-2


def test_cli_lp_prints_link_prediction_precision(tmp_path):
    cfg = _cfg()
    _, snaps, src = W.build(cfg, seed=43)
    rng = np.random.default_rng(0)
    last = snaps[-1]
    pos = last[np.isin(last[:, 0], src)][:40]
    assert len(pos) >= 10
    neg = np.stack([rng.choice(src, 200), rng.integers(0, cfg["n"], 200)], 1)
    _dataset(str(tmp_path), "DY_LP_Dataset", "tiny", snaps[:-1], src,
             {"tiny-Pos_LP_Test.txt": pos, "tiny-Neg_LP_Test.txt": neg})
    args = [CLI, "u_lp", "tiny", "EB/", "0.2", "6", "0.00001", "1", "4", "2", str(cfg["n"]),
            "2", "2", "0.3"]
    r = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    prec = [float(l.split(":")[1]) for l in r.stdout.splitlines()
            if l.startswith("link prediction precision")]
    assert len(prec) == len(snaps) - 1
    # the same loop through the library: positives then negatives, each a
    # sorted set, k = the number of positive pairs read
    pos_u, neg_u = np.unique(pos, axis=0), np.unique(neg, axis=0)
    pos_set = {tuple(p) for p in pos_u}
    pp = np.concatenate([pos_u, neg_u]).astype(np.int32)
    flags = np.array([1] * len(pos_u) + [tuple(p) in pos_set for p in neg_u], np.uint8)
    with T.Session(cfg["n"], src, alpha=0.2, rmax=1e-5, n_parts=4, hierarchy_n=2, passes_q=6,
                   dynamic_ppr_start_iter=2, lazy_update_start_iter=2, delta=0.3,
                   transform=T.TRANSFORM_LOG10_LP, root_scaling=T.ROOT_U,
                   lp_right_factor=True) as s:
        for k, e in enumerate(snaps[:-1]):
            s.step(e)
            ref = T.lp_precision(s.lp_scores(pp), flags, len(pos))
            assert abs(ref - prec[k]) <= 2.0 / len(pos)
