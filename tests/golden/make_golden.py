"""Generates tests/golden/ref_ppr_*.npz from the reference's own code.

Runs the reference's graph store (Code/Graph_dynamic.h, fed through its own
file reader) and its dense-path refresh + push functions
(Code/ppr_computation_store_dynamic.h, compiled from the reference sources by
oracle/build_ref.sh into oracle/_ref/libtsvd_ref.so) on small seeded graphs,
and stores the inputs and the reference's outputs (adjacency, degrees,
residue, reserve, accumulated dense matrix) after every snapshot.

    sh oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import native  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (directed, n, S, snapshot sizes, alpha, rmax, dynamic_start, nparts, seed)
    "undirected": (0, 240, 8, [600, 80, 80], 0.2, 1e-4, 2, 4, 101),
    "directed": (1, 240, 8, [700, 90, 90], 0.2, 1e-4, 2, 4, 202),
    "undirected_scratch": (0, 180, 6, [400, 60], 0.5, 1e-3, 100, 3, 303),
}


def make(name, directed, n, S, sizes, alpha, rmax, dyn, nparts, seed):
    rng = np.random.default_rng(seed)
    snaps = []
    for k in sizes:
        e = rng.integers(0, n, size=(k, 2)).astype(np.int32)
        e = e[e[:, 0] != e[:, 1]]
        snaps.append(e)
    deg0 = np.bincount(snaps[0].ravel(), minlength=n)
    sources = np.sort(rng.choice(np.nonzero(deg0)[0], S, replace=False)).astype(np.int32)
    g = native.RefGraph(n, directed)
    fwd = native.RefPPR(n, sources, nparts, alpha, rmax)
    tr = native.RefPPR(n, sources, nparts, alpha, rmax) if directed else None
    out = dict(directed=directed, n=n, sources=sources, alpha=alpha, rmax=rmax,
               dynamic_start=dyn, nparts=nparts, nsnap=len(snaps))
    with tempfile.TemporaryDirectory() as d:
        for it, e in enumerate(snaps, start=1):
            path = os.path.join(d, "s%d.txt" % it)
            native.write_edge_file(path, e, trailing_newline=True)
            g.insert_file(path)
            out["edges_%d" % it] = e
            for dirn in range(2 if directed else 1):
                off, nb = g.adjacency(dirn)
                deg, former = g.degrees(dirn)
                out["off_%d_%d" % (it, dirn)] = off
                out["nbr_%d_%d" % (it, dirn)] = nb
                out["former_%d_%d" % (it, dirn)] = former
                st = fwd if dirn == 0 else tr
                st.step(g, dirn, it, dyn)
                out["r_%d_%d" % (it, dirn)] = st.state(0)
                out["p_%d_%d" % (it, dirn)] = st.state(1)
            out["dense_%d" % it] = fwd.dense() + (tr.dense() if tr is not None else 0.0)
    np.savez_compressed(os.path.join(HERE, "ref_ppr_%s.npz" % name), **out)


if __name__ == "__main__":
    if not native.ref_available():
        native.build_ref()
    for name, args in CASES.items():
        make(name, *args)
        print("wrote", name)
